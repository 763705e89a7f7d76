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
    assert "facade cpu ok" in r.stdout


@pytest.mark.gpu
def test_facade_renderer_on_gpu(cuda_lib, oracle_lib, tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([str(exe), "gpu"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "gpu resident: 3 frames equal to the copying path" in r.stdout
    assert "facade gpu ok" in r.stdout
