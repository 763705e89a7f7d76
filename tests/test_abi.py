"""The C-ABI library builds for sm_103a, loads, and exports every entry
point include/cadr_cuda.h declares (CPU only: no compute call)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for f in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            names += re.findall(r"CADR_API\s+[\w\s\*]+?\b(cadr_\w+)\s*\(", src)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(cuda_lib):
    from cadr_gb300 import lib
    names = declared_symbols()
    assert len(names) > 30
    out = subprocess.run(["nm", "-D", "--defined-only", lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (cadr_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        getattr(cuda_lib, n)
    # the ctypes signature table covers the whole ABI
    assert set(names) == set(lib._SIGS), set(names) ^ set(lib._SIGS)


def test_library_is_built_for_sm_103a(cuda_lib):
    from cadr_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert "-fmad=false" in build.NVCC_FLAGS  # the bit-exact arithmetic relies on it


def test_struct_layouts_match_header(tmp_path):
    """sizeof/offsetof of the ABI structs from a C compiler agree with the
    Python mirrors."""
    from cadr_gb300 import lib
    from cadr_gb300.scenes import CMD_DTYPE, LOD_DTYPE
    from cadr_gb300.tier_a import DRAWABLE_DTYPE
    from cadr_gb300.views import VIEW_DTYPE
    prog = tmp_path / "sz.c"
    prog.write_text("""
#include <stdio.h>
#include <stddef.h>
#include "cadr_cuda.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n",
    sizeof(cadr_draw_indirect_cmd), sizeof(cadr_draw_indexed_cmd), sizeof(cadr_drawable_gpu_data),
    sizeof(cadr_drawable_pointers), sizeof(cadr_lod), sizeof(cadr_view), sizeof(cadr_scene_desc),
    sizeof(cadr_scene_buffers), sizeof(cadr_batch_view), sizeof(cadr_tuning), sizeof(cadr_server_config),
    sizeof(cadr_request_result), offsetof(cadr_batch_view, cmds), sizeof(cadr_frame_info),
    offsetof(cadr_frame_info, level_ms));
  return 0; }
""")
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(prog), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    want = [16, CMD_DTYPE.itemsize, DRAWABLE_DTYPE.itemsize, 32, LOD_DTYPE.itemsize, VIEW_DTYPE.itemsize,
            C.sizeof(lib.SceneDesc), C.sizeof(lib.SceneBuffers), C.sizeof(lib.BatchView), C.sizeof(lib.Tuning),
            C.sizeof(lib.ServerConfig), C.sizeof(lib.RequestResult), lib.BatchView.cmds.offset,
            C.sizeof(lib.FrameInfo), lib.FrameInfo.level_ms.offset]
    assert got == want
    assert got[:6] == [16, 20, 48, 32, 16, 144]


def test_status_strings_and_no_device_error(cuda_lib):
    """Without a GPU the context cannot be created and the call says why."""
    from cadr_gb300 import lib
    assert cuda_lib.cadr_status_string(lib.TIMEOUT) == b"timeout"
    assert cuda_lib.cadr_abi_version() == 1
    assert cuda_lib.cadr_build_flags() == 0  # the product build
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        h = C.c_void_p()
        st = cuda_lib.cadr_context_create(0, C.byref(h))
        assert st != lib.OK and not h.value
        assert cuda_lib.cadr_last_error()


def test_null_arguments_are_rejected(cuda_lib):
    from cadr_gb300 import lib
    assert cuda_lib.cadr_context_create(0, None) == lib.INVALID_ARG
    assert cuda_lib.cadr_cull(None, None, None, None, None, None) == lib.INVALID_ARG
    assert cuda_lib.cadr_process_drawables(None, 1, None, None, 0, None, None, None) == lib.INVALID_ARG
    assert cuda_lib.cadr_server_submit(None, None, None, 0, None) == lib.INVALID_ARG
    assert cuda_lib.cadr_context_record_timestamp(None, 0, 0, None) == lib.INVALID_ARG
    assert cuda_lib.cadr_context_read_timestamps(None, 0, None) == lib.INVALID_ARG


def test_bounds_checked_build_compiles_and_says_so(cuda_lib):
    """The bounds-checked build (CADR_BOUNDS_CHECK) of the same sources
    compiles for sm_103a, exports the same entry points and reports itself
    through cadr_build_flags()."""
    from cadr_gb300 import build
    path = build.build_checked()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    assert set(declared_symbols()) <= set(re.findall(r"\bT (cadr_\w+)", out))
    checked = C.CDLL(path)
    checked.cadr_build_flags.restype = C.c_uint32
    assert checked.cadr_build_flags() == 1  # CADR_BUILD_BOUNDS_CHECK


def test_headers_compile_on_their_own(tmp_path):
    """Each public header compiles by itself: cadr_cuda.h as C99 and C++17,
    every include/CadR header as C++17 (a drop-in user includes them one by
    one, as CadR's own headers are included)."""
    inc = os.path.join(ROOT, "include")
    c = tmp_path / "h.c"
    c.write_text("#include <cadr_cuda.h>\n")
    subprocess.run(["gcc", "-std=c99", "-fsyntax-only", "-Wall", "-Wextra", "-Werror", "-I", inc, str(c)], check=True)
    for h in ["cadr_cuda.h"] + ["CadR/" + f for f in sorted(os.listdir(os.path.join(inc, "CadR"))) if f.endswith(".h")]:
        src = tmp_path / "h.cpp"
        src.write_text(f"#include <{h}>\n")
        r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-Werror", "-I", inc, str(src)],
                           capture_output=True, text=True)
        assert r.returncode == 0, h + "\n" + r.stderr[-2000:]
