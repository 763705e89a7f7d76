"""The GPU parity tests again, against the bounds-checked build of the
library (cadr_gb300.build.build_checked(): the same sources compiled with
CADR_BOUNDS_CHECK).  There every index a kernel derives itself (each
command slot against its StateSet region, each count against its region's
size, plane words, the scene's per-tile region table, the batched form's
work items) is checked before the access it guards; a failed check sets
CADR_DEVERR_BOUNDS, which the tests' device-error checks turn into a
failure.  This stands in for compute-sanitizer, which is not available on
every machine these tests run on."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MODULES = ["test_gpu_cull.py", "test_gpu_batched.py", "test_gpu_shard.py", "test_gpu_pack.py", "test_gpu_tier_a.py"]


def test_parity_suite_under_the_bounds_checked_build(cuda_lib):
    from cadr_gb300 import build
    path = build.build_checked()
    env = dict(os.environ, CADR_CUDA_LIB=path)
    probe = subprocess.run([sys.executable, "-c", "from cadr_gb300 import lib; print(lib.load().cadr_build_flags())"],
                           env=env, cwd=ROOT, capture_output=True, text=True, timeout=120)
    assert probe.stdout.strip() == "1", probe.stdout + probe.stderr  # CADR_BUILD_BOUNDS_CHECK
    cmd = [sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider",
           "-k", "not full_size", *[os.path.join(ROOT, "tests", m) for m in MODULES]]
    r = subprocess.run(cmd, env=env, cwd=ROOT, capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert " passed" in r.stdout and " failed" not in r.stdout
