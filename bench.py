"""Benchmark of the drawable-processing pass on GB300.

Default workload: the plain pass on the large CAD scene (C2: 16,777,216
drawables in 256 StateSets, hierarchy 4,096 -> 65,536 -> 1,048,576 ->
drawables, 3 LODs, seed 1).  One step = one full pass: propagation of every
hierarchy level, then the leaf stage (world matrices, bounding spheres,
frustum cull, LOD, per-StateSet compaction) in three launches: the stream
kernel, the tile scan and the write kernel.

  value  Gdrawables/s with the scene resident in HBM (inputs 1.6 GB > L2, so
         no L2 flush between steps is needed)
  e2e    same metric through the C ABI with host buffers: every step uploads
         all per-drawable inputs from pinned host memory, runs the pass and
         reads the per-StateSet counts and the visible commands back; the
         median of three runs of the loop (the host link is shared with the
         host's other GPUs)
  roofline  the dominant kernel (the leaf stream kernel): its algorithmic
         bytes per launch over its average launch time, CUDA events on the
         launching stream; `leaf_stage` gives the same for the three leaf
         launches together

Beside the headline, the same line carries (N=1): `batched` (C4, 256 uneven
views in one persistent launch against 256 plain passes), `tier_a` (the
reference shader's pass), `c3` (the deep-hierarchy scene at its full
4,194,304 drawables, with per-level propagation times), `serving` (C5,
Poisson requests for 60 s with p50/p99 latency) and `cpu_baseline` (the
oracle on all host cores and on one, median of 5 passes each).

`--impl reference` times the CPU restatement of the pass (the oracle,
OpenMP over all host cores) on the same workload: the reference itself has
no CPU implementation of the pass, and its GPU path (Vulkan shaders) cannot
run without a graphics stack.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gdrawables/s culled+compacted"
UNIT = "Gdrawables/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=16_777_216, help="drawables of the C2 scene")
    ap.add_argument("--e2e-steps", type=int, default=0, help="e2e steps (default: min(steps, 50))")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-form (C4) and Tier A measurements")
    ap.add_argument("--no-c3", action="store_true", help="skip the deep-hierarchy (C3) measurement")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-form (C5) measurement")
    ap.add_argument("--plain-duration", type=float, default=10.0,
                    help="serving: seconds of the request stream the one-request-per-launch loop serves")
    ap.add_argument("--form", default="plain", choices=["plain", "serving", "tier-a", "batched", "c3"])
    ap.add_argument("--batched-tuning", default="", help="batched: block_threads,items_per_thread,ctas_per_sm[,form] "
                                                           "instead of the autotuner's pick")
    ap.add_argument("--rate", type=float, default=20000.0, help="serving: requests per second")
    ap.add_argument("--duration", type=float, default=60.0, help="serving: seconds of request stream")
    ap.add_argument("--serving-scenes", type=int, default=64)
    ap.add_argument("--inflight", type=int, default=8, help="serving: batches in flight")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def measured_sm_max_mhz() -> float:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f).get("sm_max_mhz", 2070.0))
    return 2070.0


def committed_traffic(key: str):
    """Per-launch DRAM traffic on the full C2 scene from the committed ncu
    summary of the leaf stage (`key`: stream_kernel_traffic_bytes or
    leaf_stage_traffic_bytes), or None."""
    p = os.path.join(ROOT, "profiles", "leaf_stage_c2.md")
    if not os.path.exists(p):
        return None
    m = re.search(key + r":\s*([0-9.eE+]+)", open(p).read())
    return float(m.group(1)) if m else None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.proc, self.lines = index, None, []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def bench_config(sc, world: int) -> dict:
    """The workload description both arms print (identical dicts)."""
    return {"workload": f"C2 plain pass, {sc.n} drawables, {sc.num_state_sets} StateSets (Zipf 1.1), levels "
                        f"{sc.level_sizes}, {sc.num_lods} LODs, seed 1",
            "l2": "inputs larger than L2 (no flush)",
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU"}


def committed_profile_value(name: str, key: str):
    """A `key: value` figure from a committed ncu summary under profiles/."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    m = re.search(re.escape(key) + r":\s*([0-9.eE+]+)", open(p).read())
    return float(m.group(1)) if m else None


def leaf_algorithmic_bytes(sc, visible: int) -> int:
    """Compulsory DRAM bytes of the leaf stage: per drawable the local
    matrix (64), parent index (4), local sphere (16), geometry index (4) and
    world matrix written (64); per visible drawable its 20-byte command; the
    marginal bitmask (N/8); every parent world matrix read once.  The
    stage's own bit-planes and tile words are not counted."""
    n = sc.n
    parents = sc.level_sizes[-1] if sc.level_sizes else 0
    return n * (64 + 4 + 16 + 4 + 64) + 20 * visible + (n + 7) // 8 + 64 * parents


def stream_algorithmic_bytes(sc) -> int:
    """The stream kernel's share of leaf_algorithmic_bytes: everything but
    the geometry indices and the commands, which the write kernel moves."""
    n = sc.n
    parents = sc.level_sizes[-1] if sc.level_sizes else 0
    return n * (64 + 4 + 16 + 64) + (n + 7) // 8 + 64 * parents


def level_algorithmic_bytes(sc, l: int) -> int:
    """Internal level l >= 1: local read 64, parent index 4, world write 64
    per node; every parent's world matrix read once."""
    return sc.level_sizes[l] * (64 + 4 + 64) + sc.level_sizes[l - 1] * 64


def step_algorithmic_bytes(sc, visible: int) -> int:
    """The whole step: the leaf stage plus every internal level l >= 1."""
    return leaf_algorithmic_bytes(sc, visible) + sum(level_algorithmic_bytes(sc, l)
                                                     for l in range(1, len(sc.level_sizes)))


def time_plain_pass(ctx, ds, sc, out, steps: int, warmup: int):
    """K untraced passes timed with CUDA events on the context stream, then
    K traced passes (frame timing) for the per-kernel and per-level shares.
    Returns (ms per untraced pass, frames, visible, launches per pass)."""
    import torch
    view = sc.views[0]
    for _ in range(warmup):
        ds.cull(view, out)
    ctx.sync()
    ctx.check_device_error()
    visible = int(ctx.download(out.counts, np.uint32, (sc.num_state_sets,)).sum())
    stream = torch.cuda.ExternalStream(ctx.stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctx.sync()
    l0 = ctx.launch_count
    ev0.record(stream)
    for _ in range(steps):
        ds.cull(view, out)
    ev1.record(stream)
    ctx.sync()
    launches = (ctx.launch_count - l0) // max(1, steps)
    ms = ev0.elapsed_time(ev1) / steps
    ctx.check_device_error()
    ctx.collect_frame_info(True)
    for _ in range(steps):
        ds.cull(view, out)
    ctx.sync()
    frames = ctx.frame_infos(with_levels=True)
    ctx.collect_frame_info(False)
    ctx.check_device_error()
    return ms, frames, visible, launches


def run_c3(ctx, steps: int, warmup: int, peak: float):
    """C3, the deep-hierarchy scene at its stated size: 4,194,304 drawables
    under an 8-level BFS tree (branching U{2..16}), 16 StateSets, 2 LODs.
    One pass per step as in the headline; per-level propagation times from
    traced passes; checked in full against the oracle."""
    from cadr_gb300 import lib, scenes
    from oracle import bind
    t0 = time.time()
    sc = scenes.config3()
    gen_s = time.time() - t0
    ds = lib.DeviceScene(ctx, sc)
    out = lib.CullOutputs(ctx, sc.n, sc.num_state_sets)
    ms, frames, visible, launches = time_plain_pass(ctx, ds, sc, out, steps, warmup)
    got = out.fetch()
    ref = bind.cull(sc, sc.views[0], threads=bind.max_threads())
    same = bool(np.array_equal(got["counts"], ref["counts"]) and np.array_equal(
        bind.valid_cmds(got["cmds"], got["counts"], sc.state_set_offsets).view(np.uint8),
        bind.valid_cmds(ref["cmds"], ref["counts"], sc.state_set_offsets).view(np.uint8)) and
        np.array_equal(got["marginal"], ref["marginal"]))
    mean = lambda k: float(np.mean([f[k] for f in frames]))
    prop_ms, leaf_ms, stream_ms = mean(0), mean(1), mean(3)
    level_ms = [float(np.mean([f[4][l] for f in frames])) for l in range(len(sc.level_sizes) - 1)]
    sizes = sc.level_sizes
    levels = []
    for l in range(1, len(sizes)):
        b = level_algorithmic_bytes(sc, l)
        t = level_ms[l - 1]
        levels.append({"level": l, "nodes": sizes[l], "ms": t, "algorithmic_bytes": b,
                       "gbs": b / (t / 1e3) / 1e9 if t > 0 else None})
    step_bytes = step_algorithmic_bytes(sc, visible)
    stream_bytes = stream_algorithmic_bytes(sc)
    leaf_bytes = leaf_algorithmic_bytes(sc, visible)
    return {
        "workload": f"C3 deep hierarchy, {sc.n} drawables, 16 StateSets, 2 LODs, seed 2, internal levels {sizes}",
        "internal_nodes": int(sum(sizes)), "ms_per_pass": ms, "gdrawables_per_s": sc.n / (ms / 1e3) / 1e9,
        "visible_fraction": visible / sc.n, "launches_per_pass": launches,
        "step": {"algorithmic_bytes": step_bytes, "gbs": step_bytes / (ms / 1e3) / 1e9,
                 "frac": step_bytes / (ms / 1e3) / 1e9 / peak},
        "traced": {"propagate_ms": prop_ms, "leaf_ms": leaf_ms, "stream_ms": stream_ms,
                   "leaf_fraction_of_traced_pass": leaf_ms / (prop_ms + leaf_ms),
                   "stream_kernel": {"algorithmic_bytes": stream_bytes,
                                     "frac": stream_bytes / (stream_ms / 1e3) / 1e9 / peak},
                   "leaf_stage": {"algorithmic_bytes": leaf_bytes,
                                  "frac": leaf_bytes / (leaf_ms / 1e3) / 1e9 / peak},
                   "levels": levels,
                   "level_imbalance": {"largest_over_smallest_nodes": max(sizes[1:]) / min(sizes[1:]),
                                       "slowest_over_fastest_ms": max(level_ms) / min(level_ms)}},
        "bit_exact_vs_oracle": same, "scene_generation_s": gen_s,
    }


def run_batched(ctx, steps: int, warmup: int, num_scenes: int = 32, tuning_override: str = ""):
    """Batched form on C4: 256 views (8 per scene) over 32 scenes of
    1,000 .. 2,000,000 drawables, culled by one persistent launch replayed
    from a captured CUDA graph with the autotuned shape, against 256
    sequential plain passes (each a full pass of its scene).  Returns the
    timings and whether all 256 outputs are bit-identical."""
    import torch
    from cadr_gb300 import lib, scenes
    from oracle import bind
    scs = scenes.config4(num_scenes=num_scenes)
    dss = [lib.DeviceScene(ctx, sc) for sc in scs]
    for ds in dss:
        ds.propagate(world_spheres=True)
    items, plain_outs = [], []
    for sc, ds in zip(scs, dss):
        for v in sc.views:
            items.append((ds, v, lib.CullOutputs(ctx, sc.n, sc.num_state_sets, marginal=False)))
            plain_outs.append(lib.CullOutputs(ctx, sc.n, sc.num_state_sets, marginal=False))
    arr = lib.batch_views(items)
    if tuning_override:
        f = [int(x) for x in tuning_override.split(",")]
        ctx.set_tuning(f[0], f[1], f[2], f[3] if len(f) > 3 else 0)
        tuning, tune_ms = ctx.get_tuning(), None
    else:
        tuning, tune_ms = lib.autotune_batched(ctx, arr, reps=3)
    stream = torch.cuda.ExternalStream(ctx.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def plain_step():
        k = 0
        for sc, ds in zip(scs, dss):
            for v in sc.views:
                o = plain_outs[k]
                lib.check(ctx.lib.cadr_cull(ds.handle, np.ascontiguousarray(v).ctypes.data, o.cmds.ptr,
                                            o.counts.ptr, None, None))
                k += 1

    def batched_step():
        lib.cull_batched(ctx, arr, None, use_graph=True)

    res = {}
    for name, fn in (("plain", plain_step), ("batched", batched_step)):
        for _ in range(warmup):
            fn()
        ctx.sync()
        l0 = ctx.launch_count
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        ctx.sync()
        res[name] = (e0.elapsed_time(e1) / steps, (ctx.launch_count - l0) // steps)
    ctx.check_device_error()
    identical = True
    for (ds, v, ob), op in zip(items, plain_outs):
        gb, gp = ob.fetch(), op.fetch()
        off = ds.host.state_set_offsets
        identical &= bool(np.array_equal(gb["counts"], gp["counts"]) and np.array_equal(
            bind.valid_cmds(gb["cmds"], gb["counts"], off).view(np.uint8),
            bind.valid_cmds(gp["cmds"], gp["counts"], off).view(np.uint8)))
    view_items = sum(sc.n * len(sc.views) for sc in scs)
    # Compulsory bytes of one batched launch: every scene's world spheres
    # and geometry ids once (16 + 4 B per drawable; its 8 views share them),
    # per view its 20-byte commands.  Tables and scratch are not counted.
    visible = sum(int(ob.fetch()["counts"].sum()) for _, _, ob in items)
    batched_bytes = sum(sc.n * 20 for sc in scs) + 20 * visible
    peak = measured_peak()[0]
    gbs = batched_bytes / (res["batched"][0] / 1e3) / 1e9
    # Issue ceiling: 4 warp instructions per cycle per SM at the maximum SM
    # clock, over the thread instructions per item of the committed ncu
    # capture of the batched kernel.
    ipi = committed_profile_value("batched_c4.md", "thread_instructions_per_item")
    import torch
    sms, mhz = torch.cuda.get_device_properties(0).multi_processor_count, measured_sm_max_mhz()
    ceiling = sms * 4 * 32 * mhz * 1e6 / ipi / 1e9 if ipi else None
    items_rate = view_items / (res["batched"][0] / 1e3) / 1e9
    return {
        "workload": f"C4: {len(items)} views over {len(scs)} scenes of {min(s.n for s in scs)}.."
                    f"{max(s.n for s in scs)} drawables (log-uniform), 4 perspective + 4 ortho cascades each",
        "view_drawables": view_items,
        "plain_ms": res["plain"][0], "batched_ms": res["batched"][0],
        "speedup": res["plain"][0] / res["batched"][0],
        "batched_gitems_per_s": view_items / (res["batched"][0] / 1e3) / 1e9,
        "plain_gitems_per_s": view_items / (res["plain"][0] / 1e3) / 1e9,
        "launches_per_step": {"plain": res["plain"][1], "batched": res["batched"][1]},
        "tuning": {"block_threads": tuning.block_threads, "items_per_thread": tuning.items_per_thread,
                   "ctas_per_sm": tuning.ctas_per_sm,
                   "form": "three-launch" if tuning.form == lib.BATCHED_THREE_LAUNCH else "persistent",
                   "autotune_ms": tune_ms},
        "bit_identical": identical,
        "roofline": {"bound": "issue", "algorithmic_bytes": batched_bytes, "achieved_gbs": gbs,
                     "frac_of_hbm": gbs / peak, "thread_instructions_per_item": ipi,
                     "issue_ceiling_gitems_per_s": ceiling,
                     "frac_of_issue_ceiling": items_rate / ceiling if ceiling else None,
                     "source": "instructions per item from profiles/batched_c4.md; ceiling = SMs x 4 warp "
                               "instructions per cycle x 32 threads x max SM clock"},
        "note": "batched: scenes propagated once (world spheres), one persistent launch over (view, tile) "
                "items from a captured CUDA graph; plain: 256 full passes",
    }


def run_tier_a(ctx, n: int, steps: int, warmup: int, peak: float):
    """Tier A (the reference shader's pass) on n drawables packed in StateSet
    order, 4,096 geometries, one MatrixList and one drawable-data allocation
    per drawable: 3-level handle tables.  Checked in full against the
    oracle.  148 algorithmic bytes per drawable."""
    import torch
    from cadr_gb300 import lib, tier_a
    from oracle import bind
    # The image holds absolute device addresses: size it first, then build it
    # for the buffer it will live in.
    dev = ctx.alloc(tier_a.image_size(n, num_geometries=4096) + 4096)
    im = tier_a.build(n, seed=7, base=dev.ptr, num_geometries=4096)
    ref_ind, ref_ptr = bind.process_drawables(im.image, im.base, im.level, im.root, im.drawables,
                                              threads=bind.max_threads())
    ctx.upload(dev, im.image)
    d = ctx.to_device(im.drawables)
    ind, ptr = ctx.alloc(n * 16), ctx.alloc(n * 32)
    stream = torch.cuda.ExternalStream(ctx.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(warmup):
        ctx.process_drawables(im.level, im.root, d, n, ind, ptr)
    ctx.sync()
    e0.record(stream)
    for _ in range(steps):
        ctx.process_drawables(im.level, im.root, d, n, ind, ptr)
    e1.record(stream)
    ctx.sync()
    ms = e0.elapsed_time(e1) / steps
    same = bool(np.array_equal(ctx.download(ind, np.uint32, (n, 4)), ref_ind) and
                np.array_equal(ctx.download(ptr, np.uint64, (n, 4)), ref_ptr))
    gbs = n * 148 / (ms / 1e3) / 1e9
    per = committed_profile_value("process_drawables_level3.md", "dram_bytes_per_drawable")
    out = {"workload": f"{n} drawables, 4,096 geometries, {im.num_handles} handles (level {im.level} tables)",
           "gdrawables_per_s": n / (ms / 1e3) / 1e9, "ms": ms, "algorithmic_bytes_per_drawable": 148,
           "achieved_gbs": gbs, "frac": gbs / peak, "frac_of_peak": gbs / peak,
           "traffic": per * n if per else None,
           "traffic_source": "ncu DRAM bytes per drawable of profiles/process_drawables_level3.md "
                             "(4,194,304-drawable capture) x drawables",
           "bit_exact_vs_oracle": same}
    out["pack"] = run_pack(ctx, im, steps, warmup, peak, ms, ref_ind, ref_ptr)
    out["consumer_check"] = run_consumer_check(ctx, steps=max(3, min(steps, 10)), warmup=2)
    return out


def run_consumer_check(ctx, steps: int, warmup: int, n: int = 262_144):
    """The vertex-pulling consumer check (cadr_check_draws) over the Tier A
    draws of an image with index, vertex and matrix data (64 geometries of
    1,024 vertices, 36..3,000 indices per PrimitiveSet): every vertex of
    every draw pulled and transformed as the consumer vertex shader would.
    Checked against the oracle on the first 4,096 draws."""
    import torch
    from cadr_gb300 import lib, tier_a
    from oracle import bind
    kw = dict(n=n, num_state_sets=8, num_geometries=64, prims_per_geometry=3, geometry_data=True)
    dev = ctx.alloc(tier_a.image_size(**{k: v for k, v in kw.items() if k != "num_state_sets"}) + 4096)
    im = tier_a.build(seed=31, base=dev.ptr, **kw)
    ctx.upload(dev, im.image)
    d = ctx.to_device(im.drawables)
    ind, ptr, out = ctx.alloc(n * 16), ctx.alloc(n * 32), ctx.alloc(n * 16)
    ctx.process_drawables(im.level, im.root, d, n, ind, ptr)
    view = np.eye(4, dtype=np.float32)
    view[3, 2] = -50.0
    f = 1.0 / np.tan(np.radians(30.0))
    cv = lib.consumer_view(view.reshape(16), p11=f / (16 / 9), p22=f, p33=500.0 / (0.5 - 500.0),
                           p43=0.5 * 500.0 / (0.5 - 500.0))
    regions = [(dev.ptr, im.image.nbytes)]
    stream = torch.cuda.ExternalStream(ctx.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(warmup):
        ctx.check_draws(ind, ptr, n, regions, cv, out)
    ctx.sync()
    e0.record(stream)
    for _ in range(steps):
        ctx.check_draws(ind, ptr, n, regions, cv, out)
    e1.record(stream)
    ctx.sync()
    ms = e0.elapsed_time(e1) / steps
    got = ctx.download(out, lib.DRAW_CHECK_DTYPE, (n,))
    g_ind = ctx.download(ind, np.uint32, (n, 4))
    g_ptr = ctx.download(ptr, np.uint64, (n, 4))
    k = 4096
    ref = bind.check_draws([(im.image, im.base)], g_ind[:k], g_ptr[:k], cv, threads=bind.max_threads())
    pulled = int(got["pulled"].astype(np.int64).sum())
    return {"workload": f"{n} Tier A draws, {pulled} vertex pulls", "ms": ms,
            "gpulls_per_s": pulled / (ms / 1e3) / 1e9, "draws_flagged": int((got["flags"] != 0).sum()),
            "oracle_equal_first_4096": bool(np.array_equal(got[:k], ref))}


def run_pack(ctx, im, steps: int, warmup: int, peak: float, tier_a_ms: float, ref_ind, ref_ptr):
    """The per-frame StateSet packing of the Tier A records.  The reference
    (StateSet::recordToCommandBuffer) copies each StateSet's list into the
    staging buffer on the host, one memcpy per StateSet, and uploads the
    staging buffer: both timed here (single host thread, pinned staging).
    Against it: the device-resident pack (cadr_pack_*), its full repack and
    a frame whose dirty rows (1% of the drawables, host records) are
    patched.  The packed array is checked against the oracle."""
    import torch
    from cadr_gb300 import lib, tier_a
    from oracle import bind
    n = im.drawables.shape[0]
    dfs, ss, li, perm, starts = tier_a.slot_layout(im.state_set_counts, seed=13)
    pool = np.ascontiguousarray(im.drawables[perm])
    # Reference path: the lists (one per StateSet, in list order) memcpy'd
    # into pinned staging at drawableCounter, then uploaded.
    lists = [np.ascontiguousarray(im.drawables[int(starts[j]):int(starts[j + 1])]) for j in range(len(dfs))]
    staging = lib.PinnedBuffer(n * 48)
    st_view = staging.view(tier_a.DRAWABLE_DTYPE, (n,))
    dev = ctx.alloc(n * 48)
    host_ms, h2d_ms = [], []
    for rep in range(max(3, warmup)):
        t0 = time.perf_counter()
        counter = 0
        for lst in lists:
            st_view[counter:counter + len(lst)] = lst
            counter += len(lst)
        t1 = time.perf_counter()
        ctx.upload(dev, st_view)
        ctx.sync()
        t2 = time.perf_counter()
        host_ms.append((t1 - t0) * 1e3)
        h2d_ms.append((t2 - t1) * 1e3)
    pk = lib.Pack(ctx, n)
    pk.set_layout(dfs, ss, li)
    pk.upload(pool)
    stream = torch.cuda.ExternalStream(ctx.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(warmup):
        pk.repack()
    ctx.sync()
    e0.record(stream)
    for _ in range(steps):
        pk.repack()
    e1.record(stream)
    ctx.sync()
    repack_ms = e0.elapsed_time(e1) / steps
    packed, offsets = pk.fetch(tier_a.DRAWABLE_DTYPE)
    ref, ref_off = bind.pack_state_sets(dfs, ss, li, pool)
    same = bool(np.array_equal(packed.view(np.uint8), ref.view(np.uint8)) and np.array_equal(offsets, ref_off))
    rs = np.random.default_rng(14)
    dirty = rs.choice(n, size=n // 100, replace=False).astype(np.uint32)
    d_rec = lib.PinnedBuffer(len(dirty) * 48)
    d_slots = lib.PinnedBuffer(len(dirty) * 4)
    d_rec.view(tier_a.DRAWABLE_DTYPE, (len(dirty),))[...] = pool[dirty]
    d_slots.view(np.uint32, (len(dirty),))[...] = dirty
    for _ in range(warmup):
        lib.check(ctx.lib.cadr_pack_patch(pk.handle, d_slots.ptr, d_rec.ptr, len(dirty), None))
    ctx.sync()
    e0.record(stream)
    for _ in range(steps):
        lib.check(ctx.lib.cadr_pack_patch(pk.handle, d_slots.ptr, d_rec.ptr, len(dirty), None))
    e1.record(stream)
    ctx.sync()
    patch_ms = e0.elapsed_time(e1) / steps
    ctx.check_device_error()
    pk.close()
    # Tier A straight from a pool whose slots follow drawable creation order
    # (the order of the MatrixList handles), outputs scattered to the packed
    # positions: no repack, and the handle-table reads of a warp coalesce.
    G = 4096
    region = np.repeat(np.arange(len(im.state_set_counts)), im.state_set_counts)
    slot_of_pos = im.drawables["matrix_list_handle"].astype(np.int64) - 1 - 3 * G
    c_ss = np.empty(n, np.uint32)
    c_li = np.empty(n, np.uint32)
    c_ss[slot_of_pos] = region
    c_li[slot_of_pos] = np.arange(n) - starts[region].astype(np.int64)
    c_pool = np.empty_like(im.drawables)
    c_pool[slot_of_pos] = im.drawables
    pk = lib.Pack(ctx, n)
    pk.set_layout(np.arange(len(im.state_set_counts), dtype=np.uint32), c_ss, c_li)
    pk.upload(c_pool)
    f_ind, f_ptr = ctx.alloc(n * 16), ctx.alloc(n * 32)
    for _ in range(warmup):
        pk.process_drawables(im.level, im.root, n, f_ind, f_ptr)
    ctx.sync()
    e0.record(stream)
    for _ in range(steps):
        pk.process_drawables(im.level, im.root, n, f_ind, f_ptr)
    e1.record(stream)
    ctx.sync()
    fused_ms = e0.elapsed_time(e1) / steps
    fused_same = bool(np.array_equal(ctx.download(f_ind, np.uint32, (n, 4)), ref_ind) and
                      np.array_equal(ctx.download(f_ptr, np.uint64, (n, 4)), ref_ptr))
    ctx.check_device_error()
    pk.close()
    repack_gbs = n * (48 + 48 + 4) / (repack_ms / 1e3) / 1e9
    return {"workload": f"{n} records of 48 B in {len(dfs)} StateSets, slots in random order",
            "reference_host_pack_ms": float(np.median(host_ms)),
            "reference_upload_ms": float(np.median(h2d_ms)),
            "device_repack_ms": repack_ms, "device_repack_gbs": repack_gbs,
            "device_repack_frac_of_peak": repack_gbs / peak,
            "patch_1pct_ms": patch_ms, "patch_rows": int(len(dirty)),
            "bit_exact_vs_oracle": same,
            "process_from_pool": {"ms": fused_ms, "gdrawables_per_s": n / (fused_ms / 1e3) / 1e9,
                                  "vs_packed_array_ms": tier_a_ms,
                                  "slots": "drawable creation order", "bit_exact_vs_oracle": fused_same}}


def measure_serving(ctx, rate: float, duration: float, plain_duration: float, num_scenes: int = 64,
                    inflight: int = 8) -> dict:
    """Serving form on C5: 64 resident scenes (10,000 .. 8,000,000 drawables,
    log-uniform, built as C2 with seeds 4000+i), a Poisson stream of cull
    requests (`rate` per second for `duration` seconds, 1-4 views each,
    random cameras with fovY U[30,90]), continuous batching with a 200 us
    window; beside it the plain loop that serves one request per launch in
    arrival order, over the first `plain_duration` seconds of the same
    stream.  Latency is submit -> completion; throughput counts (view,
    drawable) pairs.  A sample of served results is compared with the plain
    pass."""
    import time as _t
    from cadr_gb300 import lib, rng, scenes
    from oracle import bind
    t0 = _t.time()
    scs = scenes.config5_scenes(num_scenes=num_scenes)
    gen_s = _t.time() - t0
    dss = [lib.DeviceScene(ctx, sc) for sc in scs]
    for ds in dss:
        ds.propagate(world_spheres=True)
    ctx.sync()
    pool = np.concatenate([scenes.random_view(4, k) for k in range(2048)])
    # The request stream: exponential inter-arrival times, scene and views
    # drawn from the seeded stream.
    st = rng.Stream(4, "serving.requests")
    nreq = int(rate * duration)
    idx = np.arange(nreq, dtype=np.uint64)
    gaps = -np.log(1.0 - st.uniform(idx * np.uint64(4))) / rate
    arrive = np.cumsum(gaps)
    scene_of = st.integers(idx * np.uint64(4) + np.uint64(1), 0, len(scs) - 1)
    nview = st.integers(idx * np.uint64(4) + np.uint64(2), 1, 4)
    view0 = st.integers(idx * np.uint64(4) + np.uint64(3), 0, len(pool) - 4)

    def summarize(lat, items, wall):
        lat = np.asarray(lat)
        return {"requests": int(lat.size), "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3),
                "gdrawables_per_s": items / wall / 1e9, "wall_s": wall}

    # Continuous batching.
    srv = lib.Server(ctx, max_inflight=inflight, max_batch_views=64, window_ns=200_000)
    lat, items, sub_t, done = [], 0, {}, 0
    start = _t.perf_counter()
    k = 0
    while done < nreq:
        now = _t.perf_counter() - start
        while k < nreq and arrive[k] <= now:
            v = pool[view0[k]:view0[k] + nview[k]]
            rid = srv.submit(dss[scene_of[k]], v)
            sub_t[rid] = k
            k += 1
            now = _t.perf_counter() - start
        for r in srv.poll():
            assert r.status == lib.OK
            lat.append((r.complete_ns - r.submit_ns) * 1e-9)
            j = sub_t.pop(r.request_id)
            items += scs[scene_of[j]].n * int(nview[j])
            srv.release(r.request_id)
            done += 1
    wall = _t.perf_counter() - start
    batched = summarize(lat, items, wall)
    srv.close()

    # Plain loop: one request per launch, first come first served (it falls
    # behind the arrivals, so its queue grows for as long as it runs).
    outs = [lib.CullOutputs(ctx, sc.n, sc.num_state_sets, marginal=False) for sc in scs for _ in range(4)]
    lat, items = [], 0
    nplain = int(min(nreq, rate * min(duration, plain_duration)))
    start = _t.perf_counter()
    for j in range(nplain):
        now = _t.perf_counter() - start
        if now < arrive[j]:
            _t.sleep(max(0.0, arrive[j] - now - 50e-6))
            while _t.perf_counter() - start < arrive[j]:
                pass
        s = scene_of[j]
        v = pool[view0[j]:view0[j] + nview[j]]
        arr = lib.batch_views([(dss[s], v[q:q + 1], outs[4 * s + q]) for q in range(nview[j])])
        lib.cull_batched(ctx, arr, None, use_graph=False)
        ctx.sync()
        lat.append(_t.perf_counter() - start - arrive[j])
        items += scs[s].n * int(nview[j])
    wall = _t.perf_counter() - start
    plain = summarize(lat, items, wall)

    # Served results against the plain pass of the same scene and view.
    srv = lib.Server(ctx, max_inflight=inflight, max_batch_views=64, window_ns=200_000)
    ok, checked = True, 0
    for j in range(0, min(nreq, 64)):
        s = scene_of[j]
        v = pool[view0[j]:view0[j] + 1]
        rid = srv.submit(dss[s], v)
        srv.drain()
        res = {r.request_id: r for r in srv.poll()}[rid]
        counts = ctx.download(res.counts[0], np.uint32, (scs[s].num_state_sets,))
        cmds = ctx.download(res.cmds[0], scenes.CMD_DTYPE, (scs[s].n,))
        o = lib.CullOutputs(ctx, scs[s].n, scs[s].num_state_sets)
        dss[s].cull(v, o)
        ctx.sync()
        alone = o.fetch()
        ok &= bool(np.array_equal(counts, alone["counts"]) and np.array_equal(
            bind.valid_cmds(cmds, counts, scs[s].state_set_offsets).view(np.uint8),
            bind.valid_cmds(alone["cmds"], alone["counts"], scs[s].state_set_offsets).view(np.uint8)))
        checked += 1
        srv.release(rid)
    srv.close()
    for ds in dss:
        ds.close()
    return {
        "workload": f"C5: {len(scs)} resident scenes, {sum(s.n for s in scs)} drawables total, Poisson "
                    f"{rate:.0f} req/s for {duration:.0f} s, 1-4 views, 200 us window",
        "inflight_batches": inflight, "p50_ms": batched["p50_ms"], "p99_ms": batched["p99_ms"],
        "mean_ms": batched["mean_ms"], "gdrawables_per_s": batched["gdrawables_per_s"],
        "continuous_batching": batched,
        "plain_one_request_per_launch": dict(plain, seconds_of_stream=min(duration, plain_duration)),
        "served_equals_plain": ok, "served_checked": checked, "scene_generation_s": gen_s,
    }


def run_serving(args):
    """`--form serving`: the serving measurement alone, as its own line."""
    from cadr_gb300 import build, lib
    build.build()
    ctx = lib.Context(0)
    r = measure_serving(ctx, args.rate, args.duration, 20.0, args.serving_scenes, args.inflight)
    line = {"metric": "serving: Gdrawables/s and p50/p99 latency", "form": "serving",
            "value": r["gdrawables_per_s"], "unit": "Gdrawables/s", "n_gpus": 1, "higher_is_better": True,
            "config": {"workload": r["workload"], "inflight_batches": args.inflight}, "data": "synthetic", **r}
    print(json.dumps(line), flush=True)


def cpu_baseline(sc, view, passes: int = 5) -> dict:
    """The oracle on the full C2 scene: the median of `passes` passes on all
    host cores (the reported value) and of `passes` single-thread passes."""
    from oracle import bind
    import oracle
    oracle.build(with_ref=False)
    threads = bind.max_threads()

    def median_s(th):
        ts = []
        for _ in range(passes):
            t = time.perf_counter()
            bind.cull(sc, view, threads=th)
            ts.append(time.perf_counter() - t)
        return float(np.median(ts))

    all_s, one_s = median_s(threads), median_s(1)
    return {"value": sc.n / all_s / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"full C2 scene ({sc.n} drawables) per pass, median of {passes} passes",
            "all_cores_ms": all_s * 1e3, "single_thread_ms": one_s * 1e3,
            "single_thread_value": sc.n / one_s / 1e9}


def run_reference(args, sc, world, rank):
    """CPU restatement of the pass (the oracle) on all host cores: W
    warm-up steps, then exactly K timed steps.  A step is the full scene
    unless K of them would exceed a 150 s budget; then every step is a
    bounded sample, a smaller scene built by the same rules."""
    from cadr_gb300 import scenes
    from oracle import bind
    threads = bind.max_threads()
    view = sc.views[0]
    warm = []
    for _ in range(max(1, args.warmup)):
        t0 = time.perf_counter()
        bind.cull(sc, view, threads=threads)
        warm.append(time.perf_counter() - t0)
    step_sc, sample = sc, f"full C2 scene ({sc.n} drawables) per step"
    budget = 150.0
    if min(warm) * args.steps > budget:
        m = max(1 << 16, int(sc.n * budget / (min(warm) * args.steps)))
        step_sc = scenes.config2(n=m)
        sample = f"C2 rules at {m} drawables per step (bounded sample; {args.steps} steps within {budget:.0f} s)"
        bind.cull(step_sc, step_sc.views[0], threads=threads)
    steps = max(1, args.steps)
    t0 = time.perf_counter()
    for _ in range(steps):
        bind.cull(step_sc, step_sc.views[0], threads=threads)
    total = time.perf_counter() - t0
    ms = total / steps * 1e3
    value = step_sc.n * steps / total / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(sc, world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local = dist_env()
    if args.impl == "reference" and rank != 0:
        return
    if args.form == "serving":
        if rank == 0:
            run_serving(args)
        return
    if args.form == "batched":
        from cadr_gb300 import build, lib
        build.build()
        import oracle
        oracle.build(with_ref=False)
        ctx = lib.Context(local)
        print(json.dumps({"form": "batched", **run_batched(ctx, steps=args.steps, warmup=args.warmup,
                                                           tuning_override=args.batched_tuning)}))
        return
    if args.form == "c3":
        from cadr_gb300 import build, lib
        build.build()
        import oracle
        oracle.build(with_ref=False)
        ctx = lib.Context(local)
        print(json.dumps({"form": "c3", **run_c3(ctx, args.steps, args.warmup, measured_peak()[0])}))
        return
    if args.form == "tier-a":
        from cadr_gb300 import build, lib
        build.build()
        import oracle
        oracle.build(with_ref=False)
        ctx = lib.Context(local)
        print(json.dumps({"form": "tier-a", **run_tier_a(ctx, args.n, args.steps, args.warmup, measured_peak()[0])}))
        return
    from cadr_gb300 import scenes
    t0 = time.time()
    sc = scenes.config2(n=args.n)
    gen_s = time.time() - t0
    if args.impl == "reference":
        import oracle
        oracle.build(with_ref=False)
        run_reference(args, sc, world, rank)
        return

    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from cadr_gb300 import build, lib
    build.build()
    ctx = lib.Context(local)
    ds = lib.DeviceScene(ctx, sc)
    out = lib.CullOutputs(ctx, sc.n, sc.num_state_sets)
    view = sc.views[0]
    L = ctx.lib

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---- device-resident timed region ------------------------------------
    for _ in range(args.warmup):
        ds.cull(view, out)
    ctx.sync()
    ctx.check_device_error()
    counts = ctx.download(out.counts, np.uint32, (sc.num_state_sets,))
    visible = int(counts.sum())

    import torch
    torch.cuda.set_device(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    # The timed steps run untraced (no frame-timing events between the
    # launches, so the stream kernel overlaps the last level kernel's tail);
    # the same steps, traced, then give each kernel's share.
    barrier()
    ctx.sync()
    launches0 = ctx.launch_count
    ev0.record(stream)
    for _ in range(args.steps):
        ds.cull(view, out)
    ev1.record(stream)
    ctx.sync()
    barrier()
    launches = ctx.launch_count - launches0
    ms = ev0.elapsed_time(ev1) / args.steps
    ctx.check_device_error()
    ctx.collect_frame_info(True)
    for _ in range(args.steps):
        ds.cull(view, out)
    ctx.sync()
    frames = ctx.frame_infos()
    ctx.collect_frame_info(False)
    ctx.check_device_error()
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    leaf_ms = float(np.mean([f[1] for f in frames])) if frames else None
    prop_ms = float(np.mean([f[0] for f in frames])) if frames else None
    stream_ms = float(np.mean([f[3] for f in frames])) if frames else None

    out_ref = out.fetch()  # the device-resident pass's result, to check the e2e read-back against

    # ---- end to end through the C ABI with host buffers -------------------
    # Every step uploads all per-drawable and level inputs from pinned host
    # memory, culls, and reads back the counts and the valid command prefix
    # of every StateSet.  Two device scenes alternate, so that a step's
    # uploads (upload stream) overlap the previous step's pass and read-back
    # (compute stream); the scenes' own ordering events keep every upload
    # behind the pass that reads the scene before it, with no host sync.
    import torch
    e2e_steps = args.e2e_steps or min(args.steps, 50)
    pin = {}
    for name, a in [("local", sc.local), ("parent", sc.parent), ("sphere", sc.sphere), ("geometry", sc.geometry)]:
        b = lib.PinnedBuffer(a.nbytes)
        b.view(a.dtype, a.shape)[...] = a
        pin[name] = b
    lvl_pin = []
    for loc, par in zip(sc.level_local, sc.level_parent):
        bl = lib.PinnedBuffer(loc.nbytes)
        bl.view(loc.dtype, loc.shape)[...] = loc
        bp = None
        if par is not None:
            bp = lib.PinnedBuffer(par.nbytes)
            bp.view(par.dtype, par.shape)[...] = par
        lvl_pin.append((bl, bp, loc.shape[0]))
    pair = [ds, lib.DeviceScene(ctx, sc)]
    outs = [out, lib.CullOutputs(ctx, sc.n, sc.num_state_sets)]
    h_counts = [lib.PinnedBuffer(sc.num_state_sets * 4) for _ in range(2)]
    h_cmds = [lib.PinnedBuffer(sc.n * 20) for _ in range(2)]
    counts_ready = [torch.cuda.Event() for _ in range(2)]
    cstream = torch.cuda.ExternalStream(ctx.stream)
    offs = sc.state_set_offsets.astype(np.int64)
    h2d = sum(b.nbytes for b in pin.values()) + sum(bl.nbytes + (bp.nbytes if bp else 0) for bl, bp, _ in lvl_pin)

    def e2e_upload(k):
        d = pair[k % 2]
        for l, (bl, bp, n_l) in enumerate(lvl_pin):
            lib.check(L.cadr_scene_upload_level(d.handle, l, bl.ptr, bp.ptr if bp else None, 0, n_l))
        lib.check(L.cadr_scene_upload_drawables(d.handle, pin["local"].ptr, pin["parent"].ptr,
                                                pin["sphere"].ptr, pin["geometry"].ptr, 0, sc.n))

    def e2e_cull(k):
        j = k % 2
        pair[j].cull(view, outs[j])
        lib.check(L.cadr_download(ctx.handle, h_counts[j].ptr, outs[j].counts.ptr, sc.num_state_sets * 4, None))
        counts_ready[j].record(cstream)

    import ctypes
    offs_u32 = np.ascontiguousarray(sc.state_set_offsets, np.uint32)
    host_issue = [0.0]

    def e2e_readback(k):
        j = k % 2
        counts_ready[j].synchronize()
        t = time.perf_counter()
        nbytes = ctypes.c_uint64()
        lib.check(L.cadr_download_commands(ctx.handle, h_cmds[j].ptr, outs[j].cmds.ptr, h_counts[j].ptr,
                                           offs_u32.ctypes.data, sc.num_state_sets, ctypes.byref(nbytes), None))
        host_issue[0] += time.perf_counter() - t
        return sc.num_state_sets * 4 + nbytes.value

    def e2e_run(steps):
        d2h = 0
        e2e_upload(0)
        for k in range(steps):
            e2e_cull(k)
            if k + 1 < steps:
                e2e_upload(k + 1)
            d2h += e2e_readback(k)
        lib.check(L.cadr_stream_synchronize(ctx.stream))
        return d2h

    # The host link is shared with the other GPUs' jobs on the same host, so
    # the e2e loop and the uploads-alone loop (the host link's own bound on
    # a step: the same uploads back to back, no pass, no read-back) each run
    # three times, alternating, and each reports its median run.
    up_stream = L.cadr_context_upload_stream(ctx.handle)
    e2e_run(3)
    e2e_runs, up_runs, issue_runs = [], [], []
    d2h_total = 0
    for _rep in range(3):
        barrier()
        host_issue[0] = 0.0
        t1 = time.perf_counter()
        d2h_total = e2e_run(e2e_steps)
        e2e_runs.append((time.perf_counter() - t1) / e2e_steps)
        issue_runs.append(host_issue[0] / e2e_steps * 1e3)
        barrier()
        for k in range(2):
            e2e_upload(k)
        lib.check(L.cadr_stream_synchronize(up_stream))
        t2 = time.perf_counter()
        for k in range(e2e_steps):
            e2e_upload(k)
        lib.check(L.cadr_stream_synchronize(up_stream))
        up_runs.append((time.perf_counter() - t2) / e2e_steps)
    e2e_s = float(np.median(e2e_runs))
    upload_only_s = float(np.median(up_runs))
    readback_issue_ms = float(np.median(issue_runs))
    # The last step's read-back equals the device-resident pass's result
    # (the uploads-alone loop leaves the host read-back buffers alone).
    j = (e2e_steps - 1) % 2
    got_counts = h_counts[j].view(np.uint32, (sc.num_state_sets,)).copy()
    got_cmds = h_cmds[j].view(np.uint32, (sc.n, 5))
    ref_cmds = np.ascontiguousarray(out_ref["cmds"]).view(np.uint32).reshape(sc.n, 5)
    e2e_same = bool(np.array_equal(got_counts, out_ref["counts"]) and all(
        np.array_equal(got_cmds[int(offs[s]):int(offs[s]) + int(got_counts[s])],
                       ref_cmds[int(offs[s]):int(offs[s]) + int(got_counts[s])])
        for s in range(sc.num_state_sets)))
    clk = clocks.stop()
    e2e_value = world * sc.n / e2e_s / 1e9
    # The same traffic without the arithmetic, after the timed regions: the
    # bandwidth the stream kernel's access pattern can reach on this GPU.
    probe_gbs = ctx.measure_stream_mix(sc.n, 20)

    value = world * sc.n / (ms / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    leaf_bytes = leaf_algorithmic_bytes(sc, visible)
    achieved_stage = leaf_bytes / (leaf_ms / 1e3) / 1e9 if leaf_ms else None
    stream_bytes = stream_algorithmic_bytes(sc)
    achieved = stream_bytes / (stream_ms / 1e3) / 1e9 if stream_ms else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(sc, world),
        "visible_fraction": visible / sc.n,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None,
                     "traffic": committed_traffic("stream_kernel_traffic_bytes"),
                     "kernel": "leaf_stream_kernel (world matrices, spheres, cull, LOD; bit-planes)",
                     "algorithmic_bytes_per_launch": stream_bytes, "launch_ms": stream_ms,
                     "peak_source": f"{peak_kind} hbm_gbs",
                     "same_traffic_probe_gbs": probe_gbs,
                     "frac_of_probe": (achieved / probe_gbs) if achieved and probe_gbs else None},
        "leaf_stage": {"kernels": "leaf_stream_kernel + leaf_tile_scan_kernel + leaf_write_kernel",
                       "achieved": achieved_stage, "unit": "GB/s",
                       "frac": (achieved_stage / peak) if achieved_stage else None,
                       "algorithmic_bytes": leaf_bytes, "ms": leaf_ms,
                       "traffic": committed_traffic("leaf_stage_traffic_bytes")},
        "step": {"propagate_ms": prop_ms, "leaf_ms": leaf_ms,
                 "step_algorithmic_bytes": step_algorithmic_bytes(sc, visible),
                 "step_gbs": step_algorithmic_bytes(sc, visible) / (ms / 1e3) / 1e9},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h_total // max(1, e2e_steps), "ms_per_step": e2e_s * 1e3,
                "upload_only_ms_per_step": upload_only_s * 1e3,
                "runs": "median of 3 runs of the e2e loop and of the uploads-alone loop, alternating",
                "ms_per_step_runs": [r * 1e3 for r in e2e_runs],
                "upload_only_ms_runs": [r * 1e3 for r in up_runs],
                "readback_issue_host_ms_per_step": readback_issue_ms,
                "host_link_h2d_gbs": h2d / upload_only_s / 1e9,
                "pipelining": "two device scenes alternate; a step's uploads overlap the previous step's pass and read-back",
                "readback_equals_device_pass": e2e_same},
        "gpu_launches": launches,
        "clocks": clk,
        "scene_generation_s": gen_s,
    }
    if not args.no_batched:
        line["batched"] = run_batched(ctx, steps=max(3, min(args.steps, 20)), warmup=3)
        line["tier_a"] = run_tier_a(ctx, args.n, steps=max(3, min(args.steps, 50)), warmup=3, peak=peak)
    if not args.no_c3:
        line["c3"] = run_c3(ctx, steps=max(3, min(args.steps, 50)), warmup=3, peak=peak)
    if rank == 0 and world == 1 and not args.no_serving:
        line["serving"] = measure_serving(ctx, args.rate, args.duration, args.plain_duration,
                                          args.serving_scenes, args.inflight)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(sc, view)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
