"""CPU oracle of the drawable-processing pass (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
this package, and only as the oracle the CUDA path is compared against
or as the timed CPU baseline.  The
product library (cadr_gb300, libcadr_cuda.so) never imports it.
"""
from .bind import (OracleLib, build, load, load_ref, cull, cull_spheres, process_drawables,
                   mat4_mul, sphere_transform)

__all__ = ["OracleLib", "build", "load", "load_ref", "cull", "cull_spheres",
           "process_drawables", "mat4_mul", "sphere_transform"]
