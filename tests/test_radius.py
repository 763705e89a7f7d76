"""The device's bounding-sphere radius routine (float-float fast path with
a double fallback, cadr_gb300/csrc/fp.cuh) compiled for the host must equal
the reference's double evaluation on every sampled input."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_radius_fast_path_is_exact(tmp_path):
    exe = tmp_path / "radius_test"
    subprocess.run(["g++", "-O2", "-ffp-contract=off", os.path.join(ROOT, "tests", "cpp", "radius_test.cpp"),
                    "-o", str(exe), "-lm"], check=True)
    r = subprocess.run([str(exe), "20000000", "11"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches=0" in r.stdout
