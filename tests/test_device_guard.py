"""The library never leaves the calling thread on another CUDA device.

Entry points switch to their context's device only through
cadr::DeviceGuard, which gives the caller's device back on every return
path.  The guard is tested on the CPU against a fake runtime; a static
check of the sources shows that every entry point doing device work holds
one and that nothing else switches devices on a caller's thread."""
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "cadr_gb300", "csrc")
CUDA_INC = "/usr/local/cuda/include"


def test_device_guard_restores_the_callers_device(tmp_path):
    exe = tmp_path / "device_guard_test"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", CUDA_INC,
                    os.path.join(ROOT, "tests", "cpp", "device_guard_test.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "device guard ok" in r.stdout


def _entry_points():
    """(file, name, body) of every exported function in the CUDA sources."""
    out = []
    for f in sorted(os.listdir(CSRC)):
        if not f.endswith(".cu"):
            continue
        src = open(os.path.join(CSRC, f)).read()
        for m in re.finditer(r"^CADR_API [^\n]*?\b(cadr_\w+)\(", src, re.M):
            i = src.index("{", m.end())
            depth, j = 0, i
            while True:
                if src[j] == "{":
                    depth += 1
                elif src[j] == "}":
                    depth -= 1
                    if depth == 0:
                        break
                j += 1
            out.append((f, m.group(1), src[i:j + 1]))
    return out


DEVICE_WORK = re.compile(r"cudaMalloc|cudaFree\b|cudaMemcpy|cudaMemset|cudaStreamCreate|cudaEventCreate|"
                         r"cudaDeviceSynchronize|cudaLaunch|<<<|\blaunch_\w+\(|propagate_levels|scratch_reserve|"
                         r"cudaGraph|cudaMemGetInfo|cudaMallocHost|cuMem")


def test_every_entry_point_with_device_work_holds_a_guard():
    eps = _entry_points()
    assert len(eps) > 40
    missing = [f"{f}:{n}" for f, n, body in eps if DEVICE_WORK.search(body) and "DeviceGuard" not in body]
    # Pinned host memory belongs to no device.
    missing = [m for m in missing if not m.endswith(("cadr_host_alloc_pinned", "cadr_host_free_pinned"))]
    assert not missing, missing


def test_no_other_device_switch_on_a_callers_thread():
    hits = []
    for f in sorted(os.listdir(CSRC)):
        if f == "device_guard.h" or not f.endswith((".cu", ".cuh", ".h")):
            continue
        for k, line in enumerate(open(os.path.join(CSRC, f)), 1):
            if "cudaSetDevice(" in line and not line.lstrip().startswith("//"):
                hits.append((f, k))
    # The serving scheduler's own thread is the one other place.
    assert [h[0] for h in hits] == ["server.cu"], hits
