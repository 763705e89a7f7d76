"""The C++ facade (include/CadR): CadR's Renderer / StateSet / Drawable /
Geometry / MatrixList / DataStorage API over the C ABI.

The CPU part runs the reference's allocator placement checks
(tests/DataAllocationTest.cpp), HandleTable growth and StateSet recording
with host memory standing in for the device; the GPU part runs the pass
through the facade's Renderer and compares it with the oracle."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(tmp_path):
    from cadr_gb300 import build
    lib_dir = os.path.dirname(build.FACADE_LIB)
    exe = tmp_path / "facade_test"
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "facade_test.cpp"), "-o", str(exe),
                    "-L", lib_dir, "-lcadr", "-lcadr_cuda", "-L", os.path.join(ROOT, "oracle", "_build"),
                    "-lcadr_oracle", f"-Wl,-rpath,{lib_dir}:{os.path.join(ROOT, 'oracle', '_build')}", "-fopenmp"],
                   check=True)
    return exe


def test_facade_host_side(cuda_lib, oracle_lib, tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([str(exe), "cpu"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "parent/child lists ok" in r.stdout
    assert "drawable api ok" in r.stdout
    assert "frame info host ok" in r.stdout
    assert "finalize ok" in r.stdout
    assert "data allocation api ok" in r.stdout
    assert "facade cpu ok" in r.stdout


@pytest.mark.gpu
def test_facade_renderer_on_gpu(cuda_lib, oracle_lib, tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([str(exe), "gpu"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "gpu resident: 5 frames equal to the copying path" in r.stdout
    assert "gpu frame info ok" in r.stdout
    assert "facade gpu ok" in r.stdout


def test_reference_parent_child_test(cuda_lib):
    """The reference's tests/ParentChildTest.cpp, compiled unchanged against
    the facade's headers and library (oracle/Makefile, target ref-api), runs
    to completion: StateSet's childList / parentList keep the reference's
    interface.  Only where the CADR sources are present."""
    from oracle import bind
    from cadr_gb300 import build
    ref = bind.reference_root()
    if not ref:
        pytest.skip("CADR sources not present")
    build.build_facade()
    oracle_dir = os.path.join(ROOT, "oracle")
    subprocess.run(["make", "-s", "--no-print-directory", "-C", oracle_dir, "ref-api", f"REF={ref}",
                    f"LIB={os.path.dirname(build.FACADE_LIB)}"], check=True)
    exe = os.path.join(oracle_dir, "_ref", "parent_child_test")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr


def test_facade_with_glm(cuda_lib, tmp_path):
    """With GLM on the include path the facade's matrix type is glm::mat4,
    as in the reference: tests/cpp/facade_glm_test.cpp fills MatrixLists
    from glm::mat4 values and in place (editNewContent) and uses the
    Geometry helpers, against the same library.  GLM is the reference's
    copy (3rdParty/GLM), so only where the CADR sources are present."""
    from oracle import bind
    from cadr_gb300 import build
    ref = bind.reference_root()
    if not ref:
        pytest.skip("CADR sources (and their GLM) not present")
    lib_dir = os.path.dirname(build.build_facade())
    exe = tmp_path / "facade_glm_test"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ref, "3rdParty", "GLM"),
                    os.path.join(ROOT, "tests", "cpp", "facade_glm_test.cpp"), "-o", str(exe),
                    "-L", lib_dir, "-lcadr", "-lcadr_cuda", f"-Wl,-rpath,{lib_dir}"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "facade glm ok" in r.stdout
