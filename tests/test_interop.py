"""The Vulkan side of the shared output buffers (cadr_gb300/interop/
vulkan_import.c) compiles against the Vulkan headers: compile-only, since
neither machine has a Vulkan device.  The CUDA side is tested on the GPU
(tests/test_gpu_export.py)."""
import os
import shutil
import subprocess

import pytest

from oracle import bind

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_vulkan_import_compiles():
    root = bind.reference_root()
    inc = os.path.join(root, "3rdParty", "Vulkan", "include") if root else ""
    if not inc or not os.path.isdir(inc) or not shutil.which("gcc"):
        pytest.skip("the Vulkan headers or gcc are not on this machine")
    src = os.path.join(ROOT, "cadr_gb300", "interop", "vulkan_import.c")
    r = subprocess.run(["gcc", "-std=c11", "-fsyntax-only", "-Wall", "-Wextra", "-Werror", "-I", inc, src],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
