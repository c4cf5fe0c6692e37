"""ctypes binding of libcylag_gpu.so (the C ABI in include/cylag_gpu.h).

The library is loaded from ``cylag_gb300/_native``; if it is missing the
import fails loudly -- there is no CPU fallback for the particle step.
With CYLAG_DEBUG_BOUNDS=1 in the environment the bounds-checked build
(``libcylag_gpu_debug.so``, built on first use) is loaded instead.
"""
from __future__ import annotations

import ctypes as C
import os
import threading
from pathlib import Path

_DEBUG_BOUNDS = os.environ.get("CYLAG_DEBUG_BOUNDS") == "1"
_NATIVE = Path(__file__).resolve().parent / "_native" / (
    "libcylag_gpu_debug.so" if _DEBUG_BOUNDS else "libcylag_gpu.so")
_lock = threading.Lock()
_lib = None

CG_OK = 0
CG_EINVAL = -1
CG_ECUDA = -2
CG_ENOMEM_BUDGET = -3
CG_EDEVICE = -4
CG_ESTATE = -5

CG_ERR_INTERP_OUTSIDE = 1
CG_ERR_DEGENERATE_LAYER = 2
CG_ERR_RNG_LIMIT = 4
CG_ERR_UNSUPPORTED = 8
CG_ERR_NONFINITE = 16
CG_ERR_BOUNDS = 32

CG_PRECISION_FP64 = 0
CG_PRECISION_MIXED = 1

CG_NOALLOC_MAX_PARTICLES = 262144

P = C.c_void_p
I32 = C.c_int32
F64 = C.c_double


class MeshDesc(C.Structure):
    _fields_ = [("nv", I32), ("nt", I32), ("ne", I32), ("nopen", I32),
                ("x", P), ("y", P), ("triangles", P), ("gradx", P), ("grady", P),
                ("det", P), ("edges", P), ("triedge_map", P), ("edgetri_map", P),
                ("edges_labels", P), ("grid_x0", F64), ("grid_y0", F64),
                ("grid_inv_cell", F64), ("grid_nx", I32), ("grid_ny", I32),
                ("grid_start", P), ("grid_tris", P)]


class FieldsDesc(C.Structure):
    _fields_ = [("dim", I32), ("nlayers", I32), ("npoints", I32), ("ntimes", I32),
                ("times", P), ("elevation", P), ("velocity_x", P), ("velocity_y", P),
                ("velocity_z", P), ("turbulent_energy", P), ("dissipation", P),
                ("bottom", P), ("friction_model", I32), ("friction_coefficient", F64)]


class Params(C.Structure):
    _fields_ = [("model", I32), ("time_scheme", I32), ("rng_method", I32),
                ("diffusion_model", I32), ("diffusion_lsm2_option", I32),
                ("lsm3_edge_opt", I32), ("boundary_conditions", I32),
                ("boundary_conditions_type", I32), ("max_wall_rebounds", I32),
                ("bnd_statistics", I32), ("particle_velocity_init", I32),
                ("frozen_eulerian_fields", I32),
                ("initial_time", F64), ("final_time", F64), ("time_step", F64),
                ("horizontal_diffusivity", F64), ("vertical_diffusivity", F64),
                ("schmidt_number", F64), ("tl_horizontal", F64), ("tl_vertical", F64),
                ("rebound_damping_coef", F64), ("wall_roughness_angle", F64),
                ("stranding_probability", F64), ("water_density", F64),
                ("dim", I32), ("particle_density", F64),
                ("drag_coefficient_model", I32), ("drag_coefficient", F64),
                ("added_mass_force", I32), ("added_mass_coef", F64),
                ("buoyancy_velocity_model", I32), ("buoyancy_velocity", F64),
                ("precision", I32), ("seed", C.c_uint64), ("sort_period", I32)]


class StateDesc(C.Structure):
    _fields_ = [("n", I32), ("position", P), ("velocity", P), ("fluid_velocity_seen", P),
                ("last_position", P), ("last_velocity", P), ("tri", P), ("last_tri", P),
                ("lowerlayer", P), ("tag", P), ("diameter", P), ("rng_state", P),
                ("depth", P)]


class HostArrays(C.Structure):
    _fields_ = [("position", P), ("velocity", P), ("fluid_velocity_seen", P), ("tri", P),
                ("lowerlayer", P), ("tag", P), ("rng_state", P)]


# (name, restype, argtypes) for every symbol include/cylag_gpu.h declares
SIGNATURES = [
    ("cg_ctx_create", C.c_int, [I32, C.c_uint64, C.POINTER(P)]),
    ("cg_ctx_destroy", C.c_int, [P]),
    ("cg_last_error", C.c_int, [P, C.c_char_p, C.c_uint64]),
    ("cg_ctx_stream", C.c_uint64, [P]),
    ("cg_ctx_set_stream", C.c_int, [P, C.c_uint64]),
    ("cg_ctx_sync", C.c_int, [P]),
    ("cg_mesh_upload", C.c_int, [P, C.POINTER(MeshDesc)]),
    ("cg_fields_upload", C.c_int, [P, C.POINTER(FieldsDesc)]),
    ("cg_run_create", C.c_int, [P, C.POINTER(Params), C.POINTER(StateDesc), C.POINTER(P)]),
    ("cg_run_destroy", C.c_int, [P]),
    ("cg_run_seed", C.c_int, [P]),
    ("cg_run_init", C.c_int, [P]),
    ("cg_run_step", C.c_int, [P, I32, P]),
    ("cg_run_step_noalloc", C.c_int, [P, I32]),
    ("cg_run_writeback", C.c_int, [P]),
    ("cg_rng_draws", C.c_int, [P, C.c_uint64, C.c_uint64, I32, I32, C.c_int64, P]),
    ("cg_run_time", C.c_int, [P, C.POINTER(F64), C.POINTER(C.c_int64)]),
    ("cg_run_errors", C.c_int, [P, C.POINTER(C.c_uint32)]),
    ("cg_run_last_kernel_ms", C.c_int, [P, C.POINTER(F64), C.POINTER(I32)]),
    ("cg_run_last_kernel_split_ms", C.c_int, [P, C.POINTER(F64), C.POINTER(F64)]),
    ("cg_run_clock", C.c_int, [P, C.POINTER(F64), C.POINTER(F64), C.POINTER(C.c_int64)]),
    ("cg_run_resume", C.c_int, [P, F64, F64, C.c_int64]),
    ("cg_snapshot_txt", C.c_int, [C.c_char_p, C.c_int32, C.c_int32, C.c_double, C.c_int64,
                                  C.c_int32, P, P, P, P, P, P, P]),
    ("cg_snapshot_vtk", C.c_int, [C.c_char_p, C.c_int32, C.c_int32, C.c_double, C.c_int64,
                                  C.c_int32, P, P, P, P, P, P, P]),
    ("cg_run_step_host", C.c_int, [P, I32, C.POINTER(HostArrays), C.POINTER(HostArrays), I32, P]),
    ("cg_run_set_stranding_output", C.c_int, [P, C.c_int32]),
    ("cg_run_stranded", C.c_int, [P, P, C.POINTER(C.c_int32)]),
    ("cg_run_set_sections", C.c_int, [P, C.c_int32, P]),
    ("cg_run_section_stats", C.c_int, [P, P, C.POINTER(C.c_int32)]),
    ("cg_run_resize", C.c_int, [P, C.POINTER(StateDesc)]),
    ("cg_run_added", C.c_int, [P, C.c_int32]),
    ("cg_server_create", C.c_int, [P, I32, C.c_int64, I32, F64, C.POINTER(P)]),
    ("cg_server_destroy", C.c_int, [P]),
    ("cg_server_admit", C.c_int, [P, C.POINTER(Params), I32, P, F64, P, I32, C.POINTER(I32)]),
    ("cg_server_step", C.c_int, [P, I32]),
    ("cg_server_run_status", C.c_int, [P, I32, C.POINTER(I32)]),
    ("cg_server_read", C.c_int, [P, I32, P, P, P, P, P, P, C.POINTER(C.c_uint32)]),
    ("cg_server_release", C.c_int, [P, I32]),
    ("cg_server_stats", C.c_int, [P, C.POINTER(I32), C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                  C.POINTER(C.c_int64), C.POINTER(F64)]),
]


def library_path() -> Path:
    return _NATIVE


def load():
    """Load libcylag_gpu.so and declare every entry point."""
    global _lib
    with _lock:
        if _lib is None:
            if _DEBUG_BOUNDS:
                from .build import build
                build(debug_bounds=True)
            if not _NATIVE.exists():
                raise ImportError(
                    f"{_NATIVE} is missing: build it with `python -m cylag_gb300.build` "
                    "(the GPU particle step has no CPU fallback)")
            L = C.CDLL(str(_NATIVE))
            for name, res, args in SIGNATURES:
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


class CylagGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def check(ctx, rc):
    if rc == CG_OK:
        return
    buf = C.create_string_buffer(512)
    if ctx:
        load().cg_last_error(ctx, buf, 512)
    msg = buf.value.decode(errors="replace")
    if rc == CG_EINVAL:
        raise ValueError(msg)
    raise CylagGpuError(rc, msg)
