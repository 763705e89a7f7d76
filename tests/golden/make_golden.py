"""Generates the golden fixtures of tests/golden/.

  ref_math.npz  matrix products and bounding-sphere transforms computed by the
                CADR reference's own code: GLM's mat4 operator* and
                CadR::BoundingSphere operator* (src/CadR/BoundingSphere.h:70-86),
                compiled from the reference sources into oracle/_ref by
                `make -C oracle ref`.  These pin the oracle's arithmetic.
  small.npz     a 1,500-drawable scene (2 internal levels, 6 StateSets of
                which one is empty, 3 LODs) with its inputs and the oracle's
                outputs, so GPU tests can check against stored bits.
  c1.json       hashes of the C1 inputs (generator reproducibility) and of
                the oracle's C1 outputs.
  tier_a.json   hashes of the Tier A outputs on three images (handle-table
                depths 1, 2, 3), computed by the reference's own
                processDrawables shader (src/CadR/shaders/processDrawables.comp)
                compiled as C++ into oracle/_ref by `make -C oracle ref`
                (oracle/ref_shader_shim.h); the oracle must give the same
                bits before they are written.

Run from the repository root in the build container (the reference sources
must be present):  python tests/golden/make_golden.py
"""
import ctypes as C
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import bind  # noqa: E402
from cadr_gb300 import scenes, tier_a  # noqa: E402

TIER_A_BASE = 0x7F0000000000


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def ref_math(n: int = 1024, seed: int = 20261203):
    ref = bind.load_ref()
    if ref is None:
        raise SystemExit("oracle/_ref/libcadr_ref.so missing: run `make -C oracle ref` first")
    rs = np.random.RandomState(seed)
    scale = rs.choice([1e-3, 0.5, 1.0, 3.0, 1e4], size=(n, 2))
    a = (rs.standard_normal((n, 16)) * scale[:, :1]).astype(np.float32)
    b = (rs.standard_normal((n, 16)) * scale[:, 1:]).astype(np.float32)
    s = (rs.standard_normal((n, 4)) * rs.choice([1e-2, 1.0, 1e3], size=(n, 1))).astype(np.float32)
    s[:, 3] = np.abs(s[:, 3])
    prod = np.empty((n, 16), np.float32)
    sph = np.empty((n, 4), np.float32)
    for i in range(n):
        ref.ref_mat4_mul(a[i].ctypes.data, b[i].ctypes.data, prod[i].ctypes.data)
        ref.ref_sphere_transform(a[i].ctypes.data, s[i].ctypes.data, sph[i].ctypes.data)
    np.savez_compressed(os.path.join(HERE, "ref_math.npz"), a=a, b=b, s=s, prod=prod, sphere=sph,
                        glm_version=np.array([ref.ref_glm_version()]))
    return a, b, s, prod, sph


def small_scene():
    sc = scenes.small_scene(seed=11, n=1500, num_levels=2, num_state_sets=6, num_lods=3,
                            empty_state_sets=(3,), camera_extent=600.0)
    o = bind.cull(sc, sc.views[0], threads=1, want_world=True)
    valid = bind.valid_cmds(o["cmds"], o["counts"], sc.state_set_offsets)
    np.savez_compressed(
        os.path.join(HERE, "small.npz"),
        level0_local=sc.level_local[0], level1_local=sc.level_local[1], level1_parent=sc.level_parent[1],
        local=sc.local, parent=sc.parent, sphere=sc.sphere, geometry=sc.geometry,
        offsets=sc.state_set_offsets, lods=sc.lods.view(np.uint32).reshape(-1, 4), num_lods=np.array([3]),
        view=sc.views[0].view(np.uint8), counts=o["counts"], valid_cmds=valid.view(np.uint32).reshape(-1, 5),
        marginal=o["marginal"], world=o["world"], world_sphere=o["world_sphere"])


def c1_summary():
    sc = scenes.config1()
    o = bind.cull(sc, sc.views[0], threads=1, want_world=True)
    valid = bind.valid_cmds(o["cmds"], o["counts"], sc.state_set_offsets)
    inputs = {"level0_local": sha(sc.level_local[0]), "local": sha(sc.local), "parent": sha(sc.parent),
              "sphere": sha(sc.sphere), "geometry": sha(sc.geometry), "offsets": sha(sc.state_set_offsets),
              "lods": sha(sc.lods), "view": sha(sc.views[0])}
    out = {"counts": o["counts"].tolist(), "valid_cmds": sha(valid), "marginal": sha(o["marginal"]),
           "world": sha(o["world"]), "world_sphere": sha(o["world_sphere"]),
           "visible": int(o["counts"].sum())}
    with open(os.path.join(HERE, "c1.json"), "w") as f:
        json.dump({"inputs": inputs, "outputs": out}, f, indent=1)


def tier_a_summary():
    res = {}
    for name, kw in {"level1": dict(n=300, num_geometries=100),
                     "level2": dict(n=5000),
                     "level3": dict(n=3000, num_geometries=50, extra_handles=4_200_000)}.items():
        im = tier_a.build(seed=7, base=TIER_A_BASE, **kw)
        ref = bind.ref_shader_process_drawables(im.image, im.base, im.level, im.root, im.drawables)
        assert ref is not None, "address range of the Tier A image is taken"
        ind, ptr = ref
        o_ind, o_ptr = bind.process_drawables(im.image, im.base, im.level, im.root, im.drawables, threads=1)
        assert np.array_equal(o_ind, ind) and np.array_equal(o_ptr, ptr), name
        res[name] = {"kwargs": kw, "level": im.level, "image": sha(im.image), "drawables": sha(im.drawables),
                     "indirect": sha(ind), "pointers": sha(ptr)}
    with open(os.path.join(HERE, "tier_a.json"), "w") as f:
        json.dump({"base": TIER_A_BASE, "seed": 7,
                   "computed_by": "src/CadR/shaders/processDrawables.comp compiled as C++ (oracle/ref_shader_shim.h)",
                   "images": res}, f, indent=1)


if __name__ == "__main__":
    oracle.build(with_ref=True)
    a, b, s, prod, sph = ref_math()
    # The oracle must reproduce the reference code before its outputs are frozen.
    for i in range(a.shape[0]):
        assert np.array_equal(bind.mat4_mul(a[i], b[i]).view(np.uint32), prod[i].view(np.uint32)), i
        assert np.array_equal(bind.sphere_transform(a[i], s[i]).view(np.uint32), sph[i].view(np.uint32)), i
    small_scene()
    c1_summary()
    tier_a_summary()
    print("golden fixtures written to", HERE)
