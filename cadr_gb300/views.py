"""Views (cameras and shadow cascades) in the layout of `cadr_view`.

All derived quantities (frustum planes, the view-space z row, the LOD
scale) are computed in float64 on the host and rounded once to float32, so
the device evaluates no transcendental function and the CUDA path and the
oracle see the same 144-byte record.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

VIEW_DTYPE = np.dtype([
    ("planes", np.float32, (6, 4)),
    ("view_z", np.float32, (4,)),
    ("lod_threshold", np.float32, (4,)),
    ("lod_scale", np.float32),
    ("near_z", np.float32),
    ("perspective", np.uint32),
    ("reserved", np.uint32),
])
assert VIEW_DTYPE.itemsize == 144


def _normalize(v):
    v = np.asarray(v, np.float64)
    return v / math.sqrt(float(v @ v))


def _basis(forward, up_hint=(0.0, 1.0, 0.0)):
    f = _normalize(forward)
    up = np.asarray(up_hint, np.float64)
    if abs(float(f @ _normalize(up))) > 0.999:
        up = np.array([0.0, 0.0, 1.0]) if abs(f[2]) < 0.9 else np.array([1.0, 0.0, 0.0])
    r = _normalize(np.cross(f, up))
    u = np.cross(r, f)
    return r, u, f


@dataclass
class Camera:
    position: np.ndarray
    forward: np.ndarray
    fov_y_deg: float
    aspect: float
    near: float
    far: float
    height_px: int
    lod_thresholds_px: tuple = ()

    def to_view(self) -> np.ndarray:
        r, u, f = _basis(self.forward)
        p = np.asarray(self.position, np.float64)
        ty = math.tan(math.radians(self.fov_y_deg) * 0.5)
        tx = ty * self.aspect
        # Inward plane normals in view space (camera looks down -Z), then
        # rotated to world space: n_w = nx*r + ny*u - nz*f, d = -n_w . p.
        planes_v = [
            (np.array([1.0, 0.0, -tx]) / math.sqrt(1 + tx * tx), 0.0),   # left
            (np.array([-1.0, 0.0, -tx]) / math.sqrt(1 + tx * tx), 0.0),  # right
            (np.array([0.0, 1.0, -ty]) / math.sqrt(1 + ty * ty), 0.0),   # bottom
            (np.array([0.0, -1.0, -ty]) / math.sqrt(1 + ty * ty), 0.0),  # top
            (np.array([0.0, 0.0, -1.0]), -self.near),                    # near
            (np.array([0.0, 0.0, 1.0]), self.far),                       # far
        ]
        rec = np.zeros(1, VIEW_DTYPE)
        for i, (nv, dv) in enumerate(planes_v):
            nw = nv[0] * r + nv[1] * u - nv[2] * f
            rec["planes"][0, i, :3] = nw
            rec["planes"][0, i, 3] = dv - float(nw @ p)
        rec["view_z"][0] = np.concatenate([-f, [float(f @ p)]])
        th = list(self.lod_thresholds_px)[:3]
        rec["lod_threshold"][0] = np.array(th + [0.0] * (4 - len(th)))
        rec["lod_scale"][0] = (self.height_px * 0.5) / ty
        rec["near_z"][0] = self.near
        rec["perspective"][0] = 1
        return rec


@dataclass
class OrthoBox:
    """Orthographic view volume: light-space axes (r, u, -f), extents in
    those coordinates relative to `origin`."""
    origin: np.ndarray
    forward: np.ndarray
    x_range: tuple
    y_range: tuple
    z_range: tuple      # depth along forward, (near, far)
    height_px: int
    lod_thresholds_px: tuple = ()

    def to_view(self) -> np.ndarray:
        r, u, f = _basis(self.forward)
        o = np.asarray(self.origin, np.float64)
        rec = np.zeros(1, VIEW_DTYPE)
        planes = [
            (r, -self.x_range[0]), (-r, self.x_range[1]),
            (u, -self.y_range[0]), (-u, self.y_range[1]),
            (f, -self.z_range[0]), (-f, self.z_range[1]),
        ]
        for i, (n, d) in enumerate(planes):
            rec["planes"][0, i, :3] = n
            rec["planes"][0, i, 3] = d - float(n @ o)
        rec["view_z"][0] = np.concatenate([-f, [float(f @ o)]])
        th = list(self.lod_thresholds_px)[:3]
        rec["lod_threshold"][0] = np.array(th + [0.0] * (4 - len(th)))
        half_h = 0.5 * (self.y_range[1] - self.y_range[0])
        rec["lod_scale"][0] = (self.height_px * 0.5) / half_h
        rec["near_z"][0] = self.z_range[0]
        rec["perspective"][0] = 0
        return rec


def shadow_cascades(cam: Camera, light_dir, num: int, max_dist: float,
                    lod_thresholds_px=()) -> list:
    """Orthographic cascades covering camera depth slices [z_i, z_{i+1}]
    (practical split, lambda = 0.5), each fitted around the slice's corners
    in light space and extended towards the light by max_dist."""
    r, u, f = _basis(cam.forward)
    p = np.asarray(cam.position, np.float64)
    ty = math.tan(math.radians(cam.fov_y_deg) * 0.5)
    tx = ty * cam.aspect
    n0, n1 = cam.near, min(cam.far, max_dist)
    splits = []
    for i in range(num + 1):
        lg = n0 * (n1 / n0) ** (i / num)
        un = n0 + (n1 - n0) * i / num
        splits.append(0.5 * lg + 0.5 * un)
    lr, lu, lf = _basis(light_dir)
    out = []
    for i in range(num):
        corners = []
        for z in (splits[i], splits[i + 1]):
            for sx in (-1, 1):
                for sy in (-1, 1):
                    corners.append(p + f * z + r * (sx * tx * z) + u * (sy * ty * z))
        c = np.array(corners)
        lx, ly, lz = c @ lr, c @ lu, c @ lf
        out.append(OrthoBox(origin=np.zeros(3), forward=lf,
                            x_range=(lx.min(), lx.max()), y_range=(ly.min(), ly.max()),
                            z_range=(lz.min() - max_dist, lz.max()),
                            height_px=cam.height_px, lod_thresholds_px=lod_thresholds_px))
    return out
