"""ctypes binding of libcadr_cuda.so (the C ABI declared in include/cadr_cuda.h).

This is the reference-facing call path the tests and the benchmark drive.
There is no fallback: when the CUDA library is missing, load() raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .scenes import CMD_DTYPE, LOD_DTYPE, Scene
from .views import VIEW_DTYPE

HERE = os.path.dirname(os.path.abspath(__file__))
# CADR_CUDA_LIB names another build of the same C ABI to load instead (the
# bounds-checked build, cadr_gb300.build.build_checked(), in its tests).
LIB_PATH = os.environ.get("CADR_CUDA_LIB") or os.path.join(HERE, "_lib", "libcadr_cuda.so")
MAX_LEVELS = 16

STATUS = {0: "CADR_OK", 1: "CADR_ERR_INVALID_ARG", 2: "CADR_ERR_OUT_OF_MEMORY", 3: "CADR_ERR_TIMEOUT",
          4: "CADR_ERR_CUDA", 5: "CADR_ERR_DEVICE", 6: "CADR_ERR_NOT_READY", 7: "CADR_ERR_REJECTED"}
OK, INVALID_ARG, OUT_OF_MEMORY, TIMEOUT, CUDA, DEVICE, NOT_READY, REJECTED = range(8)
DEVERR_LOOKBACK_TIMEOUT, DEVERR_MBARRIER_TIMEOUT, DEVERR_BAD_INDEX, DEVERR_BOUNDS = 0x1, 0x2, 0x4, 0x8
FAULT_NONE, FAULT_SKIP_FIRST_TILE_PUBLISH, FAULT_SERVER_LAUNCH = 0, 1, 2

# Exported symbols of the C ABI (checked against include/cadr_cuda.h by the tests).
vp, u32, u64, i32, sz = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_size_t


class SceneDesc(C.Structure):
    _fields_ = [("num_levels", u32), ("num_state_sets", u32), ("level_size", u64 * MAX_LEVELS),
                ("num_drawables", u64), ("num_geometries", u32), ("num_lods", u32)]


class SceneBuffers(C.Structure):
    _fields_ = [("level_local", vp * MAX_LEVELS), ("level_parent", vp * MAX_LEVELS),
                ("level_world", vp * MAX_LEVELS), ("local", vp), ("parent", vp), ("sphere", vp),
                ("geometry", vp), ("state_set_offsets", vp), ("lods", vp), ("world", vp),
                ("world_sphere", vp)]


class View(C.Structure):
    _fields_ = [("raw", C.c_uint8 * 144)]


class BatchView(C.Structure):
    _fields_ = [("scene", vp), ("view", View), ("cmds", vp), ("counts", vp), ("marginal", vp)]


class Tuning(C.Structure):
    _fields_ = [("block_threads", u32), ("items_per_thread", u32), ("ctas_per_sm", u32),
                ("form", u32)]


BATCHED_PERSISTENT, BATCHED_THREE_LAUNCH = 0, 1


class MemoryRegion(C.Structure):
    _fields_ = [("base", u64), ("size", u64)]


class ConsumerView(C.Structure):
    _fields_ = [("view", C.c_float * 16), ("p11", C.c_float), ("p22", C.c_float), ("p33", C.c_float),
                ("p43", C.c_float), ("p31", C.c_float), ("p32", C.c_float), ("p34", C.c_float),
                ("p41", C.c_float), ("p42", C.c_float), ("p44", C.c_float), ("reserved", u32 * 2)]


DRAW_CHECK_DTYPE = np.dtype([("checksum", np.uint64), ("pulled", np.uint32), ("flags", np.uint32)])
DRAW_BAD_INDEX_READ, DRAW_BAD_VERTEX_READ, DRAW_BAD_MATRIX_LIST, DRAW_BAD_INSTANCE, DRAW_BAD_DRAWABLE_DATA = (
    0x1, 0x2, 0x4, 0x8, 0x10)


def consumer_view(view_matrix, p11, p22, p33, p43, p31=0.0, p32=0.0, p34=-1.0, p41=0.0, p42=0.0, p44=0.0):
    """cadr_consumer_view from a column-major 4x4 view matrix (16 floats)
    and the projection members of the consumer shader."""
    v = ConsumerView()
    m = np.ascontiguousarray(view_matrix, np.float32).reshape(16)
    for k in range(16):
        v.view[k] = float(m[k])
    v.p11, v.p22, v.p33, v.p43 = p11, p22, p33, p43
    v.p31, v.p32, v.p34, v.p41, v.p42, v.p44 = p31, p32, p34, p41, p42, p44
    return v


class ServerConfig(C.Structure):
    _fields_ = [("max_inflight_batches", u32), ("max_batch_views", u32), ("window_ns", u64),
                ("memory_budget_bytes", u64), ("reserve_bytes", u64)]


class RequestResult(C.Structure):
    _fields_ = [("request_id", u64), ("status", i32), ("num_views", u32), ("submit_ns", u64),
                ("complete_ns", u64), ("cmds", vp * 4), ("counts", vp * 4)]


class FrameInfo(C.Structure):
    _fields_ = [("frame", u64), ("propagate_ms", C.c_float), ("leaf_ms", C.c_float), ("total_ms", C.c_float),
                ("stream_ms", C.c_float), ("num_levels", u32), ("level_ms", C.c_float * MAX_LEVELS)]


_SIGS = {
    "cadr_status_string": ([i32], C.c_char_p),
    "cadr_last_error": ([], C.c_char_p),
    "cadr_abi_version": ([], i32),
    "cadr_build_flags": ([], u32),
    "cadr_context_create": ([i32, C.POINTER(vp)], i32),
    "cadr_context_destroy": ([vp], i32),
    "cadr_context_stream": ([vp], vp),
    "cadr_context_upload_stream": ([vp], vp),
    "cadr_context_set_spin_limit_ns": ([vp, u64], i32),
    "cadr_context_synchronize": ([vp], i32),
    "cadr_context_launch_count": ([vp], u64),
    "cadr_measure_stream_mix": ([vp, u64, u32, C.POINTER(C.c_double)], i32),
    "cadr_shared_buffer_create": ([vp, sz, C.POINTER(vp)], i32),
    "cadr_shared_buffer_device_ptr": ([vp], vp),
    "cadr_shared_buffer_size": ([vp], sz),
    "cadr_shared_buffer_export_fd": ([vp, C.POINTER(C.c_int)], i32),
    "cadr_shared_buffer_import_fd": ([vp, C.c_int, sz, C.POINTER(vp)], i32),
    "cadr_shared_buffer_destroy": ([vp], i32),
    "cadr_context_check_device_error": ([vp, C.POINTER(u32)], i32),
    "cadr_debug_set_fault": ([vp, u32], i32),
    "cadr_context_set_collect_frame_info": ([vp, i32], i32),
    "cadr_context_get_frame_infos": ([vp, C.POINTER(FrameInfo), u32, C.POINTER(u32)], i32),
    "cadr_context_record_timestamp": ([vp, u64, u32, vp], i32),
    "cadr_context_read_timestamps": ([vp, u64, C.POINTER(u64)], i32),
    "cadr_device_alloc": ([vp, sz, C.POINTER(vp)], i32),
    "cadr_device_free": ([vp, vp], i32),
    "cadr_host_alloc_pinned": ([sz, C.POINTER(vp)], i32),
    "cadr_host_free_pinned": ([vp], i32),
    "cadr_upload": ([vp, vp, vp, sz, vp], i32),
    "cadr_download": ([vp, vp, vp, sz, vp], i32),
    "cadr_stream_synchronize": ([vp], i32),
    "cadr_download_commands": ([vp, vp, vp, vp, vp, u32, C.POINTER(u64), vp], i32),
    "cadr_process_drawables": ([vp, u32, vp, vp, u64, vp, vp, vp], i32),
    "cadr_scene_create": ([vp, C.POINTER(SceneDesc), C.POINTER(vp)], i32),
    "cadr_scene_destroy": ([vp], i32),
    "cadr_scene_get_buffers": ([vp, C.POINTER(SceneBuffers)], i32),
    "cadr_scene_upload_level": ([vp, u32, vp, vp, u64, u64], i32),
    "cadr_scene_upload_drawables": ([vp, vp, vp, vp, vp, u64, u64], i32),
    "cadr_scene_upload_state_sets": ([vp, vp], i32),
    "cadr_scene_upload_lods": ([vp, vp], i32),
    "cadr_scene_commit": ([vp], i32),
    "cadr_scene_propagate": ([vp, i32, vp], i32),
    "cadr_cull": ([vp, vp, vp, vp, vp, vp], i32),
    "cadr_cull_static_scratch": ([vp, vp, vp, vp, vp, vp], i32),
    "cadr_cull_shard_count": ([vp, vp, vp, vp, vp], i32),
    "cadr_cull_shard_write": ([vp, vp, u32, vp, u64, vp], i32),
    "cadr_cull_batched": ([vp, C.POINTER(BatchView), u32, C.POINTER(Tuning), i32, vp], i32),
    "cadr_autotune_batched": ([vp, C.POINTER(BatchView), u32, u32, C.POINTER(Tuning),
                               C.POINTER(C.c_float)], i32),
    "cadr_get_tuning": ([vp, C.POINTER(Tuning)], i32),
    "cadr_context_set_tuning_cache": ([vp, C.c_char_p], i32),
    "cadr_autotune_with": ([C.c_char_p, C.c_char_p, vp, vp, C.POINTER(Tuning), C.POINTER(C.c_float),
                            C.POINTER(i32)], i32),
    "cadr_tuning_cache_lookup": ([C.c_char_p, C.c_char_p, C.POINTER(Tuning), C.POINTER(C.c_float)], i32),
    "cadr_tuning_cache_store": ([C.c_char_p, C.c_char_p, C.POINTER(Tuning), C.c_float], i32),
    "cadr_set_tuning": ([vp, C.POINTER(Tuning)], i32),
    "cadr_pack_create": ([vp, u32, C.POINTER(vp)], i32),
    "cadr_pack_destroy": ([vp], i32),
    "cadr_pack_set_layout": ([vp, u32, u32, vp, vp, vp, vp], i32),
    "cadr_pack_upload": ([vp, vp, u32, u32, vp], i32),
    "cadr_pack_repack": ([vp, vp], i32),
    "cadr_pack_patch": ([vp, vp, vp, u32, vp], i32),
    "cadr_pack_buffers": ([vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(u32)], i32),
    "cadr_pack_process_drawables": ([vp, u32, vp, u32, vp, vp, vp], i32),
    "cadr_check_draws": ([vp, vp, vp, u64, C.POINTER(MemoryRegion), u32, C.POINTER(ConsumerView), vp, vp], i32),
    "cadr_server_create": ([vp, C.POINTER(ServerConfig), C.POINTER(vp)], i32),
    "cadr_server_destroy": ([vp], i32),
    "cadr_server_submit": ([vp, vp, vp, u32, C.POINTER(u64)], i32),
    "cadr_server_poll": ([vp, C.POINTER(RequestResult), u32, C.POINTER(u32)], i32),
    "cadr_server_release": ([vp, u64], i32),
    "cadr_server_drain": ([vp], i32),
}

_lib = None


class CadrError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


def load() -> C.CDLL:
    """Loads the in-tree libcadr_cuda.so.  Raises when it has not been built:
    this package has no CPU fallback."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with cadr_gb300.build.build()")
        lib = C.CDLL(LIB_PATH)
        for name, (args, res) in _SIGS.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
    return _lib


def check(status: int) -> None:
    if status != OK:
        raise CadrError(status, load().cadr_last_error().decode())


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, DeviceBuffer):
        return a.ptr
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return int(a)


def view_struct(rec: np.ndarray) -> View:
    rec = np.ascontiguousarray(rec, VIEW_DTYPE).reshape(-1)
    v = View()
    C.memmove(C.addressof(v), rec.ctypes.data, 144)
    return v


class DeviceBuffer:
    """Device memory owned through cadr_device_alloc / cadr_device_free."""

    def __init__(self, ctx: "Context", nbytes: int):
        self.ctx = ctx
        self.nbytes = int(nbytes)
        p = vp()
        check(load().cadr_device_alloc(ctx.handle, self.nbytes, C.byref(p)))
        self.ptr = p.value or 0

    def free(self):
        if self.ptr:
            load().cadr_device_free(self.ctx.handle, self.ptr)
            self.ptr = 0

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class PinnedBuffer:
    """Page-locked host memory (cadr_host_alloc_pinned) viewed as numpy."""

    def __init__(self, nbytes: int):
        p = vp()
        check(load().cadr_host_alloc_pinned(int(nbytes), C.byref(p)))
        self.ptr = p.value
        self.nbytes = int(nbytes)
        self.array = np.ctypeslib.as_array((C.c_uint8 * max(1, self.nbytes)).from_address(self.ptr))

    def view(self, dtype, shape):
        return self.array[: int(np.prod(shape)) * np.dtype(dtype).itemsize].view(dtype).reshape(shape)

    def free(self):
        if self.ptr:
            load().cadr_host_free_pinned(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Context:
    def __init__(self, device: int = 0):
        self.lib = load()
        h = vp()
        check(self.lib.cadr_context_create(device, C.byref(h)))
        self.handle = h.value

    def close(self):
        if self.handle:
            self.lib.cadr_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return self.lib.cadr_context_stream(self.handle) or 0

    def sync(self):
        check(self.lib.cadr_context_synchronize(self.handle))

    def check_device_error(self) -> int:
        bits = u32()
        st = self.lib.cadr_context_check_device_error(self.handle, C.byref(bits))
        if st != OK:
            raise CadrError(st, self.lib.cadr_last_error().decode())
        return bits.value

    def device_error_status(self):
        bits = u32()
        st = self.lib.cadr_context_check_device_error(self.handle, C.byref(bits))
        return st, bits.value

    def set_spin_limit_ns(self, ns: int):
        check(self.lib.cadr_context_set_spin_limit_ns(self.handle, int(ns)))

    def set_fault(self, fault: int):
        check(self.lib.cadr_debug_set_fault(self.handle, fault))

    def collect_frame_info(self, on: bool):
        check(self.lib.cadr_context_set_collect_frame_info(self.handle, 1 if on else 0))

    def frame_infos(self, with_levels: bool = False):
        """Finished frames as (propagate, leaf, total, stream) ms tuples; with
        with_levels, each tuple ends with the list of per-level times
        (levels 1..L-1)."""
        buf = (FrameInfo * 256)()
        n = u32()
        out = []
        while True:
            check(self.lib.cadr_context_get_frame_infos(self.handle, buf, 256, C.byref(n)))
            for i in range(n.value):
                f = buf[i]
                t = (f.propagate_ms, f.leaf_ms, f.total_ms, f.stream_ms)
                if with_levels:
                    t += ([f.level_ms[l] for l in range(1, f.num_levels)],)
                out.append(t)
            if n.value < 256:
                return out

    def measure_stream_mix(self, n: int, reps: int = 20) -> float:
        """GB/s of the leaf stream's traffic without its arithmetic."""
        g = C.c_double()
        check(self.lib.cadr_measure_stream_mix(self.handle, n, reps, C.byref(g)))
        return g.value

    @property
    def launch_count(self) -> int:
        return int(self.lib.cadr_context_launch_count(self.handle))

    def alloc(self, nbytes: int) -> DeviceBuffer:
        return DeviceBuffer(self, nbytes)

    def upload(self, dst, src: np.ndarray, stream=None):
        src = np.ascontiguousarray(src)
        check(self.lib.cadr_upload(self.handle, _ptr(dst), src.ctypes.data, src.nbytes, stream))

    def to_device(self, src: np.ndarray) -> DeviceBuffer:
        src = np.ascontiguousarray(src)
        b = self.alloc(max(16, src.nbytes))
        self.upload(b, src)
        self.sync()
        return b

    def download(self, src, dtype, shape, stream=None) -> np.ndarray:
        out = np.empty(shape, dtype)
        check(self.lib.cadr_download(self.handle, out.ctypes.data, _ptr(src), out.nbytes, stream))
        check(self.lib.cadr_stream_synchronize(stream or self.stream))
        return out

    def process_drawables(self, level: int, root: int, drawables, n: int, indirect, pointers, stream=None):
        check(self.lib.cadr_process_drawables(self.handle, level, root, _ptr(drawables), n,
                                              _ptr(indirect), _ptr(pointers), stream))

    def check_draws(self, indirect, pointers, n: int, regions, view: "ConsumerView", out, stream=None):
        """cadr_check_draws; regions: [(base, size)]; out: device buffer of
        n DRAW_CHECK_DTYPE records."""
        arr = (MemoryRegion * max(1, len(regions)))()
        for k, (b, sz) in enumerate(regions):
            arr[k].base, arr[k].size = b, sz
        check(self.lib.cadr_check_draws(self.handle, _ptr(indirect), _ptr(pointers), n, arr, len(regions),
                                        C.byref(view), _ptr(out), stream))

    def get_tuning(self) -> Tuning:
        t = Tuning()
        check(self.lib.cadr_get_tuning(self.handle, C.byref(t)))
        return t

    def set_tuning(self, block_threads, items_per_thread, ctas_per_sm, form=0):
        t = Tuning(block_threads, items_per_thread, ctas_per_sm, form)
        check(self.lib.cadr_set_tuning(self.handle, C.byref(t)))


class SharedBuffer:
    """cadr_shared_buffer: device memory a Vulkan device can import by file
    descriptor.  `ptr` is its device address in this context."""

    def __init__(self, ctx: "Context", nbytes: int = 0, fd: int | None = None, import_bytes: int = 0):
        """A new buffer of `nbytes`, or with `fd` the import of an exported
        descriptor of `import_bytes` (the descriptor stays the caller's)."""
        self.ctx, h = ctx, vp()
        if fd is not None:
            check(ctx.lib.cadr_shared_buffer_import_fd(ctx.handle, fd, import_bytes, C.byref(h)))
        else:
            check(ctx.lib.cadr_shared_buffer_create(ctx.handle, nbytes, C.byref(h)))
        self.handle = h.value
        self.ptr = ctx.lib.cadr_shared_buffer_device_ptr(self.handle)
        self.nbytes = ctx.lib.cadr_shared_buffer_size(self.handle)

    def __int__(self) -> int:
        return int(self.ptr)

    def export_fd(self) -> int:
        fd = C.c_int(-1)
        check(self.ctx.lib.cadr_shared_buffer_export_fd(self.handle, C.byref(fd)))
        return fd.value

    def close(self):
        if self.handle:
            check(self.ctx.lib.cadr_shared_buffer_destroy(self.handle))
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CullOutputs:
    """Device output buffers of one view of one scene."""

    def __init__(self, ctx: Context, n: int, num_state_sets: int, marginal: bool = True):
        self.n, self.S = n, num_state_sets
        self.cmds = ctx.alloc(max(16, n * 20))
        self.counts = ctx.alloc(max(16, num_state_sets * 4))
        self.marginal = ctx.alloc(max(16, ((n + 31) // 32) * 4)) if marginal else None
        self.ctx = ctx

    def fetch(self, stream=None) -> dict:
        counts = self.ctx.download(self.counts, np.uint32, (self.S,), stream)
        cmds = self.ctx.download(self.cmds, CMD_DTYPE, (self.n,), stream)
        out = {"counts": counts, "cmds": cmds}
        if self.marginal is not None:
            out["marginal"] = self.ctx.download(self.marginal, np.uint32, ((self.n + 31) // 32,), stream)
        return out


class DeviceScene:
    """A cadr_scene created from a host Scene (scenes.Scene)."""

    def __init__(self, ctx: Context, scene: Scene, upload: bool = True):
        self.ctx, self.host = ctx, scene
        d = SceneDesc()
        d.num_levels = len(scene.level_local)
        d.num_state_sets = scene.num_state_sets
        for l, a in enumerate(scene.level_local):
            d.level_size[l] = a.shape[0]
        d.num_drawables = scene.n
        d.num_geometries = scene.num_geometries
        d.num_lods = scene.num_lods
        h = vp()
        check(ctx.lib.cadr_scene_create(ctx.handle, C.byref(d), C.byref(h)))
        self.handle = h.value
        if upload:
            self.upload_all()

    def upload_all(self):
        s, L = self.host, self.ctx.lib
        for l, (loc, par) in enumerate(zip(s.level_local, s.level_parent)):
            check(L.cadr_scene_upload_level(self.handle, l, _ptr(np.ascontiguousarray(loc)),
                                            _ptr(None if par is None else np.ascontiguousarray(par)),
                                            0, loc.shape[0]))
        check(L.cadr_scene_upload_drawables(self.handle, _ptr(s.local), _ptr(s.parent), _ptr(s.sphere),
                                            _ptr(s.geometry), 0, s.n))
        check(L.cadr_scene_upload_state_sets(self.handle, _ptr(s.state_set_offsets)))
        check(L.cadr_scene_upload_lods(self.handle, _ptr(np.ascontiguousarray(s.lods, LOD_DTYPE))))
        check(L.cadr_scene_commit(self.handle))

    def buffers(self) -> SceneBuffers:
        b = SceneBuffers()
        check(self.ctx.lib.cadr_scene_get_buffers(self.handle, C.byref(b)))
        return b

    def propagate(self, world_spheres: bool = True, stream=None):
        check(self.ctx.lib.cadr_scene_propagate(self.handle, 1 if world_spheres else 0, stream))

    def cull(self, view: np.ndarray, out: CullOutputs, stream=None):
        v = np.ascontiguousarray(view, VIEW_DTYPE)
        check(self.ctx.lib.cadr_cull(self.handle, v.ctypes.data, out.cmds.ptr, out.counts.ptr,
                                     out.marginal.ptr if out.marginal is not None else None, stream))

    def close(self):
        if self.handle:
            self.ctx.lib.cadr_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_views(items) -> C.Array:
    """items: iterable of (DeviceScene, view record, CullOutputs)."""
    items = list(items)
    arr = (BatchView * len(items))()
    for k, (ds, view, out) in enumerate(items):
        arr[k].scene = ds.handle
        arr[k].view = view_struct(view)
        arr[k].cmds = out.cmds.ptr
        arr[k].counts = out.counts.ptr
        arr[k].marginal = out.marginal.ptr if out.marginal is not None else None
    return arr


def cull_batched(ctx: Context, arr, tuning: Tuning | None = None, use_graph: bool = True, stream=None):
    check(ctx.lib.cadr_cull_batched(ctx.handle, arr, len(arr), C.byref(tuning) if tuning else None,
                                    1 if use_graph else 0, stream))


# cadr_time_tuning_fn: (const cadr_tuning*, void* user, float* ms) -> cadr_status
TIME_TUNING_FN = C.CFUNCTYPE(i32, C.POINTER(Tuning), vp, C.POINTER(C.c_float))


def autotune_with(cache_path, key: str, time_fn):
    """The autotuner's search without a GPU: time_fn(Tuning) -> ms.  Returns
    (best Tuning, its ms, whether it came from the cache)."""
    def cb(tp, user, ms_out):
        ms_out[0] = float(time_fn(tp.contents))
        return OK
    fn = TIME_TUNING_FN(cb)
    best, ms, hit = Tuning(), C.c_float(), i32()
    check(load().cadr_autotune_with(cache_path.encode() if cache_path else None, key.encode(),
                                    C.cast(fn, vp), None, C.byref(best), C.byref(ms), C.byref(hit)))
    return best, ms.value, bool(hit.value)


def set_tuning_cache(ctx: Context, path):
    check(ctx.lib.cadr_context_set_tuning_cache(ctx.handle, path.encode() if path else None))


def autotune_batched(ctx: Context, arr, reps: int = 5):
    t = Tuning()
    ms = C.c_float()
    check(ctx.lib.cadr_autotune_batched(ctx.handle, arr, len(arr), reps, C.byref(t), C.byref(ms)))
    return t, ms.value


class Pack:
    """Device-resident StateSet packing of Tier A records (cadr_pack_*)."""

    def __init__(self, ctx: Context, capacity: int):
        self.ctx = ctx
        self.lib = ctx.lib
        h = vp()
        check(self.lib.cadr_pack_create(ctx.handle, capacity, C.byref(h)))
        self.handle = h.value

    def set_layout(self, dfs_order, state_set_of_slot, list_index_of_slot, stream=None):
        dfs = np.ascontiguousarray(dfs_order, np.uint32)
        ss = np.ascontiguousarray(state_set_of_slot, np.uint32)
        li = np.ascontiguousarray(list_index_of_slot, np.uint32)
        check(self.lib.cadr_pack_set_layout(self.handle, len(ss), len(dfs), _ptr(dfs), _ptr(ss), _ptr(li), stream))
        self.num_state_sets = len(dfs)

    def upload(self, records: np.ndarray, first: int = 0, stream=None):
        r = np.ascontiguousarray(records)
        assert r.dtype.itemsize == 48
        check(self.lib.cadr_pack_upload(self.handle, _ptr(r), first, len(r), stream))

    def repack(self, stream=None):
        check(self.lib.cadr_pack_repack(self.handle, stream))

    def patch(self, slots, records: np.ndarray, stream=None):
        sl = np.ascontiguousarray(slots, np.uint32)
        r = np.ascontiguousarray(records)
        assert r.dtype.itemsize == 48 and len(r) == len(sl)
        check(self.lib.cadr_pack_patch(self.handle, _ptr(sl), _ptr(r), len(sl), stream))

    def process_drawables(self, level: int, root: int, n_draw: int, indirect, pointers, stream=None):
        check(self.lib.cadr_pack_process_drawables(self.handle, level, root, n_draw, _ptr(indirect),
                                                   _ptr(pointers), stream))

    def buffers(self):
        packed, offsets, n = vp(), vp(), u32()
        check(self.lib.cadr_pack_buffers(self.handle, C.byref(packed), C.byref(offsets), C.byref(n)))
        return packed.value, offsets.value, n.value

    def fetch(self, dtype):
        """(packed records as `dtype`, region offsets) after a device sync."""
        packed, offsets, n = self.buffers()
        self.ctx.sync()
        return (self.ctx.download(packed, dtype, (n,)),
                self.ctx.download(offsets, np.uint32, (self.num_state_sets + 1,)))

    def close(self):
        if self.handle:
            self.lib.cadr_pack_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    def __init__(self, ctx: Context, max_inflight: int = 4, max_batch_views: int = 64,
                 window_ns: int = 200_000, memory_budget: int = 0, reserve: int = 0):
        self.ctx = ctx
        cfg = ServerConfig(max_inflight, max_batch_views, window_ns, memory_budget, reserve)
        h = vp()
        check(ctx.lib.cadr_server_create(ctx.handle, C.byref(cfg), C.byref(h)))
        self.handle = h.value
        self._res = (RequestResult * 256)()

    def submit(self, scene: DeviceScene, views: np.ndarray) -> int:
        v = np.ascontiguousarray(views, VIEW_DTYPE).reshape(-1)
        rid = u64()
        check(self.ctx.lib.cadr_server_submit(self.handle, scene.handle, v.ctypes.data, v.shape[0],
                                              C.byref(rid)))
        return rid.value

    def poll(self):
        n = u32()
        check(self.ctx.lib.cadr_server_poll(self.handle, self._res, 256, C.byref(n)))
        # copies: the next poll reuses the buffer
        return [RequestResult.from_buffer_copy(self._res[i]) for i in range(n.value)]

    def release(self, rid: int):
        check(self.ctx.lib.cadr_server_release(self.handle, rid))

    def drain(self):
        check(self.ctx.lib.cadr_server_drain(self.handle))

    def close(self):
        if self.handle:
            self.ctx.lib.cadr_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
