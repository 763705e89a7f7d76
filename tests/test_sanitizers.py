"""Host code under AddressSanitizer and UndefinedBehaviorSanitizer (CPU
only): the C++ facade's host-side test program (allocation placement,
handle tables, StateSet recording checked by the oracle, parent/child
lists, the DataAllocation interface, frame timing), and the oracle itself
over small scenes and Tier A images, both built with
-fsanitize=address,undefined.  Any report fails the test."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SAN = ["-fsanitize=address,undefined", "-fno-omit-frame-pointer", "-fno-sanitize-recover=all", "-g", "-O1"]
ENV = dict(os.environ, UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")


def _runtime(name):
    p = subprocess.run(["gcc", f"-print-file-name={name}"], capture_output=True, text=True).stdout.strip()
    return p if os.path.isabs(p) and os.path.exists(p) else None


@pytest.fixture(scope="module")
def sanitizers():
    asan, ubsan = _runtime("libasan.so"), _runtime("libubsan.so")
    if not asan or not ubsan:
        pytest.skip("the compiler's sanitizer runtimes are not installed")
    return asan, ubsan


def test_facade_host_side_under_sanitizers(cuda_lib, sanitizers, tmp_path):
    from cadr_gb300 import build
    lib_dir = os.path.dirname(build.LIB)
    oracle_o = tmp_path / "oracle.o"
    subprocess.run(["gcc", *SAN, "-std=c11", "-ffp-contract=off", "-fopenmp", "-I", os.path.join(ROOT, "include"),
                    "-c", os.path.join(ROOT, "oracle", "cadr_oracle.c"), "-o", str(oracle_o)], check=True)
    facade = sorted(os.path.join(ROOT, "cadr_gb300", "facade", f)
                    for f in os.listdir(os.path.join(ROOT, "cadr_gb300", "facade")) if f.endswith(".cpp"))
    exe = tmp_path / "facade_test_san"
    subprocess.run(["g++", *SAN, "-std=c++17", "-I", os.path.join(ROOT, "include"), *facade,
                    os.path.join(ROOT, "tests", "cpp", "facade_test.cpp"), str(oracle_o), "-o", str(exe),
                    "-L", lib_dir, "-lcadr_cuda", f"-Wl,-rpath,{lib_dir}", "-fopenmp", "-lm"], check=True)
    r = subprocess.run([str(exe), "cpu"], capture_output=True, text=True, timeout=600, env=ENV)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "facade cpu ok" in r.stdout
    assert "ERROR: AddressSanitizer" not in r.stderr and "runtime error" not in r.stderr


ORACLE_CASES = r'''
import sys
sys.path.insert(0, sys.argv[1])
from oracle import bind
bind.LIB_PATH = sys.argv[2]
from cadr_gb300 import scenes, tier_a
for n, lv, S, lods, empty in [(1, 0, 1, 1, ()), (2049, 3, 7, 3, (6,)), (100_003, 3, 64, 3, (5, 17)),
                              (40_000, 2, 3000, 3, ())]:
    sc = scenes.small_scene(seed=n, n=n, num_levels=lv, num_state_sets=S, num_lods=lods,
                            empty_state_sets=empty, fanout=3)
    bind.cull(sc, sc.views[0], threads=2, want_world=True)
sc = scenes.config1()
bind.cull(sc, sc.views[0], threads=2)
for kw in [dict(n=300, num_geometries=100), dict(n=5000), dict(n=3000, num_geometries=50, extra_handles=4200000)]:
    im = tier_a.build(seed=7, base=1 << 40, **kw)
    bind.process_drawables(im.image, im.base, im.level, im.root, im.drawables, threads=2)
print("oracle cases ok")
'''


def test_oracle_under_sanitizers(sanitizers, tmp_path):
    asan, ubsan = sanitizers
    so = tmp_path / "liboracle_san.so"
    subprocess.run(["gcc", *SAN, "-fPIC", "-shared", "-std=c11", "-ffp-contract=off", "-fopenmp",
                    "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "oracle", "cadr_oracle.c"),
                    "-o", str(so), "-lm"], check=True)
    script = tmp_path / "cases.py"
    script.write_text(ORACLE_CASES)
    # The interpreter itself is not instrumented: the runtimes are preloaded
    # and leak checking (which would report the interpreter's) is off.
    env = dict(ENV, LD_PRELOAD=f"{asan} {ubsan}", ASAN_OPTIONS="detect_leaks=0")
    r = subprocess.run([sys.executable, str(script), ROOT, str(so)], capture_output=True, text=True, timeout=900,
                       env=env)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "oracle cases ok" in r.stdout
    assert "ERROR: AddressSanitizer" not in r.stderr and "runtime error" not in r.stderr
