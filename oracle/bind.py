"""ctypes binding of oracle/_build/libcadr_oracle.so, oracle/_ref/libcadr_ref.so
and oracle/_ref/libcadr_ref_shader.so.

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcadr_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libcadr_ref.so")
REF_SHADER_PATH = os.path.join(HERE, "_ref", "libcadr_ref_shader.so")


def reference_root() -> str:
    """Location of the CADR reference sources: $CADR_REFERENCE_ROOT, else
    the default of the build recipe (oracle/Makefile); "" when neither
    holds the sources."""
    root = os.environ.get("CADR_REFERENCE_ROOT", "")
    if not root:
        r = subprocess.run(["make", "-s", "--no-print-directory", "-C", HERE, "print-ref"],
                           capture_output=True, text=True)
        root = r.stdout.strip() if r.returncode == 0 else ""
    return root if root and os.path.isdir(os.path.join(root, "src", "CadR")) else ""


_lib = None
_ref = None
_ref_shader = None


def build(with_ref: bool = True) -> None:
    """Compiles the oracle (and, when the CADR sources are present, the
    reference shim) with oracle/Makefile."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if with_ref:
        subprocess.run(["make", "-s", "--no-print-directory", "-C", HERE, "ref-if-present"], check=True)


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class OracleLib:
    def __init__(self, path: str):
        self.lib = C.CDLL(path)
        L = self.lib
        vp, u64, u32, i32 = C.c_void_p, C.c_uint64, C.c_uint32, C.c_int
        L.oracle_process_drawables.argtypes = [vp, u64, u64, u32, u64, vp, u64, vp, vp, i32]
        L.oracle_process_drawables.restype = i32
        L.oracle_mat4_mul.argtypes = [vp, vp, vp]
        L.oracle_sphere_transform.argtypes = [vp, vp, vp]
        L.oracle_cull.argtypes = [u32, vp, vp, vp, u64, vp, vp, vp, vp, u32, vp, u32, u32, vp, vp,
                                  vp, vp, vp, vp, vp, i32]
        L.oracle_cull.restype = i32
        L.oracle_cull_spheres.argtypes = [u64, vp, vp, u32, vp, u32, u32, vp, vp, vp, vp, vp, i32]
        L.oracle_cull_spheres.restype = i32
        L.oracle_max_threads.restype = i32
        L.oracle_pack_state_sets.argtypes = [u32, vp, u64, vp, vp, vp, vp, vp]
        L.oracle_pack_state_sets.restype = i32
        L.oracle_check_draws.argtypes = [vp, u32, vp, vp, u64, vp, vp, i32]
        L.oracle_check_draws.restype = i32


def load() -> OracleLib:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(with_ref=False)
        _lib = OracleLib(LIB_PATH)
    return _lib


def load_ref():
    """The reference-math shim, or None when it was not built (it needs the
    CADR sources, which only the build container has)."""
    global _ref
    if _ref is None and os.path.exists(REF_PATH):
        _ref = C.CDLL(REF_PATH)
        _ref.ref_mat4_mul.argtypes = [C.c_void_p] * 3
        _ref.ref_sphere_transform.argtypes = [C.c_void_p] * 3
        _ref.ref_glm_version.restype = C.c_int
    return _ref


def load_ref_shader():
    """The reference's processDrawables shader compiled as C++
    (ref_shader_shim.h, ref_shader_harness.cpp), or None when it was not
    built (it needs the CADR sources)."""
    global _ref_shader
    if _ref_shader is None and os.path.exists(REF_SHADER_PATH):
        L = C.CDLL(REF_SHADER_PATH)
        u32, u64 = C.c_uint32, C.c_uint64
        L.cadr_ref_shader_process.argtypes = [u32, u64, u64, u64, u64, u64]
        L.cadr_ref_shader_process.restype = C.c_int
        L.cadr_ref_shader_map.argtypes = [u64, u64]
        L.cadr_ref_shader_map.restype = C.c_int
        L.cadr_ref_shader_unmap.argtypes = [u64, u64]
        L.cadr_ref_shader_unmap.restype = C.c_int
        _ref_shader = L
    return _ref_shader


def ref_shader_process_drawables(image: np.ndarray, image_base: int, handle_level: int, root: int,
                                 drawables: np.ndarray):
    """Runs the reference's shader over a memory image laid out for
    image_base (256-byte aligned, as Tier A images are): the image is copied
    to host memory mapped at exactly that address, one shader invocation runs
    per drawable, and the mapping is removed.  The shader dereferences the
    addresses its tables hold, so the image must hold every PrimitiveSet and
    MatrixList the drawables reach.  Returns (indirect uint32 [N,4], pointers
    uint64 [N,4]), or None when the address range is not free."""
    L = load_ref_shader()
    if L is None:
        raise RuntimeError("oracle/_ref/libcadr_ref_shader.so is not built (make -C oracle ref)")
    size = max(int(image.nbytes), 1)
    size = (size + 4095) & ~4095
    if L.cadr_ref_shader_map(image_base, size) != 0:
        return None
    try:
        C.memmove(image_base, image.ctypes.data, int(image.nbytes))
        d = np.ascontiguousarray(drawables)
        n = int(d.shape[0])
        ind = np.zeros((n, 4), np.uint32)
        ptr = np.zeros((n, 4), np.uint64)
        rc = L.cadr_ref_shader_process(handle_level, root, d.ctypes.data, n, ind.ctypes.data, ptr.ctypes.data)
        if rc != 0:
            raise ValueError("cadr_ref_shader_process: handle level %d" % handle_level)
        return ind, ptr
    finally:
        L.cadr_ref_shader_unmap(image_base, size)


def max_threads() -> int:
    return load().lib.oracle_max_threads()


def mat4_mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    out = np.empty(16, np.float32)
    load().lib.oracle_mat4_mul(_p(a), _p(b), _p(out))
    return out


def sphere_transform(m: np.ndarray, s: np.ndarray) -> np.ndarray:
    m = np.ascontiguousarray(m, np.float32)
    s = np.ascontiguousarray(s, np.float32)
    out = np.empty(4, np.float32)
    load().lib.oracle_sphere_transform(_p(m), _p(s), _p(out))
    return out


def cull(scene, view, threads: int = 0, want_world: bool = False):
    """Plain pass over a cadr_gb300.scenes.Scene: returns dict with cmds
    (CMD_DTYPE [N]), counts [S], marginal [ceil(N/32)] and optionally world
    [N,16] / world_sphere [N,4]."""
    from cadr_gb300.scenes import CMD_DTYPE
    L = load().lib
    n = scene.n
    S = scene.num_state_sets
    nl = len(scene.level_local)
    sizes = np.array(scene.level_sizes + [0], np.uint64)
    locs = [np.ascontiguousarray(a, np.float32) for a in scene.level_local]
    pars = [None if p is None else np.ascontiguousarray(p, np.uint32) for p in scene.level_parent]
    loc_ptrs = (C.c_void_p * max(1, nl))(*[a.ctypes.data for a in locs])
    par_ptrs = (C.c_void_p * max(1, nl))(*[0 if p is None else p.ctypes.data for p in pars])
    cmds = np.zeros(n, CMD_DTYPE)
    counts = np.zeros(S, np.uint32)
    marginal = np.zeros((n + 31) // 32, np.uint32)
    world = np.empty((n, 16), np.float32) if want_world else None
    wsph = np.empty((n, 4), np.float32) if want_world else None
    view = np.ascontiguousarray(view)
    rc = L.oracle_cull(nl, _p(sizes), C.cast(loc_ptrs, C.c_void_p), C.cast(par_ptrs, C.c_void_p),
                       n, _p(scene.local), _p(scene.parent), _p(scene.sphere), _p(scene.geometry),
                       S, _p(scene.state_set_offsets), scene.num_geometries, scene.num_lods,
                       _p(scene.lods), _p(view), _p(cmds), _p(counts), _p(marginal), _p(world),
                       _p(wsph), threads)
    if rc != 0:
        raise ValueError("oracle_cull rejected the scene")
    out = {"cmds": cmds, "counts": counts, "marginal": marginal}
    if want_world:
        out["world"], out["world_sphere"] = world, wsph
    return out


def cull_spheres(world_sphere, geometry, offsets, lods, num_lods, view, threads: int = 0):
    from cadr_gb300.scenes import CMD_DTYPE
    L = load().lib
    n = int(world_sphere.shape[0])
    S = int(offsets.shape[0] - 1)
    cmds = np.zeros(n, CMD_DTYPE)
    counts = np.zeros(S, np.uint32)
    marginal = np.zeros((n + 31) // 32, np.uint32)
    ws = np.ascontiguousarray(world_sphere, np.float32)
    rc = L.oracle_cull_spheres(n, _p(ws), _p(geometry), S, _p(offsets), lods.shape[0] // num_lods,
                               num_lods, _p(lods), _p(np.ascontiguousarray(view)), _p(cmds),
                               _p(counts), _p(marginal), threads)
    if rc != 0:
        raise ValueError("oracle_cull_spheres rejected the input")
    return {"cmds": cmds, "counts": counts, "marginal": marginal}


def process_drawables(image: np.ndarray, image_base: int, handle_level: int, root: int,
                      drawables: np.ndarray, threads: int = 0):
    """Tier A over a memory image (uint8 array standing for device memory at
    image_base).  Returns (indirect uint32 [N,4], pointers uint64 [N,4])."""
    L = load().lib
    n = int(drawables.shape[0])
    ind = np.zeros((n, 4), np.uint32)
    ptr = np.zeros((n, 4), np.uint64)
    rc = L.oracle_process_drawables(_p(image), image_base, image.nbytes, handle_level, root,
                                    _p(np.ascontiguousarray(drawables)), n, _p(ind), _p(ptr),
                                    threads)
    if rc != 0:
        raise ValueError("oracle_process_drawables: a lookup left the memory image")
    return ind, ptr


def pack_state_sets(dfs_order, state_set_of_slot, list_index_of_slot, pool):
    """StateSet packing of the records `pool` (one per slot; any 48-byte
    record dtype).  Returns (packed records, region offsets [S + 1])."""
    L = load().lib
    dfs = np.ascontiguousarray(dfs_order, np.uint32)
    ss = np.ascontiguousarray(state_set_of_slot, np.uint32)
    li = np.ascontiguousarray(list_index_of_slot, np.uint32)
    pool = np.ascontiguousarray(pool)
    assert pool.dtype.itemsize == 48
    packed = np.zeros_like(pool)
    offsets = np.zeros(len(dfs) + 1, np.uint32)
    rc = L.oracle_pack_state_sets(len(dfs), _p(dfs), len(ss), _p(ss), _p(li), _p(pool), _p(packed), _p(offsets))
    if rc != 0:
        raise ValueError("oracle_pack_state_sets: the layout is not a set of lists")
    return packed, offsets


class _Region(C.Structure):
    _fields_ = [("bytes", C.c_void_p), ("base", C.c_uint64), ("size", C.c_uint64)]


def check_draws(regions, indirect, pointers, view, threads: int = 0):
    """The consumer check over host copies of device memory.  regions:
    [(uint8 array, device base address)]; indirect uint32 [N,4]; pointers
    uint64 [N,4]; view: a cadr_gb300.lib.ConsumerView.  Returns the
    per-draw (checksum, pulled, flags) records."""
    from cadr_gb300 import lib as cl
    L = load().lib
    arr = (_Region * max(1, len(regions)))()
    keep = []
    for k, (b, base) in enumerate(regions):
        b = np.ascontiguousarray(b, np.uint8)
        keep.append(b)
        arr[k].bytes, arr[k].base, arr[k].size = b.ctypes.data, base, b.nbytes
    ind = np.ascontiguousarray(indirect, np.uint32)
    ptr = np.ascontiguousarray(pointers, np.uint64)
    n = int(ind.shape[0])
    out = np.zeros(n, cl.DRAW_CHECK_DTYPE)
    L.oracle_check_draws(C.cast(arr, C.c_void_p), len(regions), _p(ind), _p(ptr), n, C.cast(C.pointer(view), C.c_void_p),
                         _p(out), threads)
    return out


def valid_cmds(cmds: np.ndarray, counts: np.ndarray, offsets: np.ndarray) -> np.ndarray:
    """Concatenation of the valid prefix of every StateSet region."""
    parts = [cmds[int(offsets[s]):int(offsets[s]) + int(counts[s])] for s in range(len(counts))]
    return np.concatenate(parts) if parts else cmds[:0]
