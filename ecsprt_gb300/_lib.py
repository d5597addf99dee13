"""ctypes binding of libecsgpu (include/ecsgpu.h, include/ecs_serve.h) and
libecshost (include/ecs_host.h).

The libraries are built in-tree by :mod:`ecsprt_gb300.build`.  Loading never
falls back to another implementation: if ``libecsgpu.so`` is missing or
cannot be loaded, :func:`gpu` raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_BUILD = Path(__file__).resolve().parent / "_build"
GPU_LIB_PATH = _BUILD / "libecsgpu.so"
HOST_LIB_PATH = _BUILD / "libecshost.so"

ECS_OK = 0
ECS_ERR_INVALID = -1
ECS_ERR_NOMEM = -2
ECS_ERR_NOT_CONVERGED = -3
ECS_ERR_NONFINITE = -4
ECS_ERR_TIMEOUT = -5
ECS_ERR_CUDA = -6
ECS_ERR_COLLISION = -7
ECS_ERR_RANGE = -8
ECS_ERR_STATE = -9
ECS_ERR_UNSUPPORTED = -10

ECS_PREC_FP64 = 0
ECS_PREC_MIXED = 1

BC_NAMES = ("periodic", "inject-reflect", "inject-advect")


class EcsParams(C.Structure):
    _fields_ = [
        ("ndim", C.c_int32), ("Nx", C.c_int32), ("Ny", C.c_int32), ("Nz", C.c_int32),
        ("bc", C.c_int32 * 3),
        ("lhs_type", C.c_int32), ("rhs_type", C.c_int32),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("x0", C.c_double), ("y0", C.c_double), ("z0", C.c_double),
        ("x1", C.c_double), ("y1", C.c_double), ("z1", C.c_double),
        ("Lx", C.c_double), ("Ly", C.c_double), ("Lz", C.c_double),
        ("qi", C.c_double), ("mi", C.c_double), ("B0", C.c_double), ("E0", C.c_double), ("n0", C.c_double),
        ("nui", C.c_double),
        ("viT", C.c_double), ("viTx", C.c_double), ("viTy", C.c_double), ("viTz", C.c_double),
        ("vi0x", C.c_double), ("vi0y", C.c_double), ("vi0z", C.c_double), ("vi0", C.c_double),
        ("Ti", C.c_double),
        ("qe", C.c_double), ("me", C.c_double), ("nue", C.c_double), ("Te", C.c_double),
        ("veTx", C.c_double), ("veTy", C.c_double), ("veTz", C.c_double), ("veT", C.c_double),
        ("ve0x", C.c_double), ("ve0y", C.c_double), ("ve0z", C.c_double), ("ve0", C.c_double),
        ("Omega_e", C.c_double), ("kappa_e", C.c_double), ("Omega_i", C.c_double), ("kappa_i", C.c_double),
        ("gammaT", C.c_double),
        ("mn", C.c_double), ("Tn", C.c_double), ("vnT", C.c_double),
        ("vn0x", C.c_double), ("vn0y", C.c_double), ("vn0z", C.c_double), ("vn0", C.c_double),
        ("scale", C.c_double),
        ("cth", C.c_double), ("cG", C.c_double),
    ]

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if name == "bc" else v
        return out


class EcsSolveStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("refinements", C.c_int32), ("relres", C.c_double), ("seconds", C.c_double)]


class EcsStepStats(C.Structure):
    _fields_ = [("collisions", C.c_int64), ("refused", C.c_int64), ("sorted", C.c_int32), ("solve", EcsSolveStats),
                ("particle_seconds", C.c_double), ("sort_seconds", C.c_double)]


class EcsPicApp(C.Structure):
    _fields_ = [("Nt", C.c_int32), ("dt", C.c_double), ("every", C.c_int32), ("Np", C.c_int64),
                ("pdist", C.c_int32), ("vdist", C.c_int32), ("output_particles", C.c_int32)]


class EcsSolverApp(C.Structure):
    _fields_ = [("input", C.c_char * 4096), ("flux_scale", C.c_double * 3), ("view_lhs", C.c_int32)]


ECS_SERVE_SOLVE = 0
ECS_SERVE_SIM = 1

ECS_INIT_SOBOL = 0
ECS_INIT_RANDOM = 2
ECS_INIT_SINUSOIDAL = 4
ECS_INIT_MODES = 16


class EcsDensityModes(C.Structure):
    _fields_ = [("nmodes", C.c_int32), ("k", (C.c_int32 * 3) * 16), ("amplitude", C.c_double * 16),
                ("phase", C.c_double * 16)]


class EcsServeConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_int64), ("max_inflight", C.c_int32), ("precision", C.c_int32),
                ("timeout_seconds", C.c_double)]


class EcsSolveRequest(C.Structure):
    _fields_ = [("density", C.c_void_p), ("flux_scale", C.c_double * 3), ("rtol", C.c_double),
                ("max_it", C.c_int32), ("phi_out", C.c_void_p)]


class EcsSimRequest(C.Structure):
    _fields_ = [("pos", C.c_void_p), ("vel", C.c_void_p), ("np", C.c_int64), ("seed", C.c_uint64),
                ("nsteps", C.c_int32), ("sort_every", C.c_int32), ("dt", C.c_double), ("rtol", C.c_double),
                ("max_it", C.c_int32), ("step_seconds", C.c_void_p), ("phi_out", C.c_void_p),
                ("pos_out", C.c_void_p), ("vel_out", C.c_void_p)]


class EcsServeResult(C.Structure):
    _fields_ = [("id", C.c_int64), ("kind", C.c_int32), ("status", C.c_int32), ("latency", C.c_double),
                ("queued", C.c_double), ("device_seconds", C.c_double), ("solve", EcsSolveStats),
                ("steps", C.c_int32), ("slot_reused", C.c_int32), ("message", C.c_char * 160)]


class EcsServeStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64),
                ("solves", C.c_int64), ("solve_p50", C.c_double), ("solve_p99", C.c_double),
                ("solve_mean", C.c_double), ("solve_max", C.c_double),
                ("steps", C.c_int64), ("step_p50", C.c_double), ("step_p99", C.c_double),
                ("device_bytes", C.c_int64), ("peak_device_bytes", C.c_int64),
                ("peak_inflight", C.c_int32), ("slots", C.c_int32),
                ("slots_created", C.c_int64), ("slot_hits", C.c_int64), ("evictions", C.c_int64),
                ("gpu_launches", C.c_int64), ("busy_seconds", C.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


_vp = C.c_void_p
_dp = C.POINTER(C.c_double)

# (name, restype, argtypes): every symbol include/ecsgpu.h and
# include/ecs_serve.h declare.
GPU_API = [
    ("ecs_version", C.c_char_p, []),
    ("ecs_status_string", C.c_char_p, [C.c_int]),
    ("ecs_last_error", C.c_char_p, [_vp]),
    ("ecs_ctx_create", C.c_int, [C.POINTER(EcsParams), C.c_int, C.c_int64, _vp, C.POINTER(_vp)]),
    ("ecs_ctx_destroy", C.c_int, [_vp]),
    ("ecs_ctx_sync", C.c_int, [_vp]),
    ("ecs_ctx_device_bytes", C.c_int64, [C.POINTER(EcsParams), C.c_int, C.c_int64]),
    ("ecs_set_sort_every", C.c_int, [_vp, C.c_int]),
    ("ecs_set_seed", C.c_int, [_vp, C.c_uint64]),
    ("ecs_set_warm_start", C.c_int, [_vp, C.c_int]),
    ("ecs_set_solver_graphs", C.c_int, [_vp, C.c_int]),
    ("ecs_particles_upload", C.c_int, [_vp, _vp, _vp, C.c_int64]),
    ("ecs_particles_download", C.c_int, [_vp, _vp, _vp]),
    ("ecs_particles_count", C.c_int64, [_vp]),
    ("ecs_particles_ids", C.c_int, [_vp, _vp]),
    ("ecs_particles_init", C.c_int, [_vp, C.c_int, C.c_int64, C.c_uint64, C.POINTER(EcsDensityModes)]),
    ("ecs_phi_upload", C.c_int, [_vp, _vp]),
    ("ecs_phi_download", C.c_int, [_vp, _vp]),
    ("ecs_moments_upload", C.c_int, [_vp, _vp]),
    ("ecs_moments_download", C.c_int, [_vp, _vp]),
    ("ecs_rhs_download", C.c_int, [_vp, _vp]),
    ("ecs_push", C.c_int, [_vp, C.c_double]),
    ("ecs_collide", C.c_int, [_vp, C.c_double]),
    ("ecs_move", C.c_int, [_vp, C.c_double]),
    ("ecs_collect", C.c_int, [_vp]),
    ("ecs_rhs", C.c_int, [_vp]),
    ("ecs_lhs", C.c_int, [_vp]),
    ("ecs_solve", C.c_int, [_vp, C.c_double, C.c_int, C.c_int, C.POINTER(EcsSolveStats)]),
    ("ecs_lhs_apply_host", C.c_int, [_vp, _vp, _vp]),
    ("ecs_rhs_noalloc", C.c_int, [C.POINTER(EcsParams), _vp, _vp, _vp]),
    ("ecs_step", C.c_int, [_vp, C.c_double, C.c_double, C.c_int, C.POINTER(EcsStepStats)]),
    ("ecs_step_host", C.c_int, [_vp, _vp, _vp, C.c_int64, C.c_double, C.c_double, C.c_int, _vp, _vp,
                                C.POINTER(EcsStepStats)]),
    ("ecs_launch_count", C.c_int64, [_vp]),
    ("ecs_fix_shifts", C.c_int, [C.POINTER(EcsParams), C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    # ecs_serve.h
    ("ecs_serve_create", C.c_int, [C.POINTER(EcsServeConfig), C.POINTER(_vp)]),
    ("ecs_serve_destroy", C.c_int, [_vp]),
    ("ecs_serve_submit_solve", C.c_int, [_vp, C.POINTER(EcsParams), C.POINTER(EcsSolveRequest),
                                         C.POINTER(C.c_int64)]),
    ("ecs_serve_submit_sim", C.c_int, [_vp, C.POINTER(EcsParams), C.POINTER(EcsSimRequest), C.POINTER(C.c_int64)]),
    ("ecs_serve_poll", C.c_int, [_vp, C.POINTER(EcsServeResult), C.c_int, C.c_int]),
    ("ecs_serve_pending", C.c_int64, [_vp]),
    ("ecs_serve_stats", C.c_int, [_vp, C.POINTER(EcsServeStats)]),
    ("ecs_serve_reset_stats", C.c_int, [_vp]),
    ("ecs_serve_request_bytes", C.c_int64, [C.POINTER(EcsParams), C.c_int, C.c_int, C.c_int64]),
    ("ecs_solve_density", C.c_int, [_vp, _vp, C.POINTER(C.c_double * 3), C.c_double, C.c_int, _vp,
                                    C.POINTER(EcsSolveStats)]),
    ("ecs_host_alloc", _vp, [C.c_size_t]),
    ("ecs_host_free", None, [_vp]),
]

HOST_API = [
    ("ecs_options_create", _vp, []),
    ("ecs_options_destroy", None, [_vp]),
    ("ecs_options_parse", C.c_int, [_vp, C.c_char_p]),
    ("ecs_options_load_file", C.c_int, [_vp, C.c_char_p]),
    ("ecs_options_get", C.c_char_p, [_vp, C.c_char_p, C.POINTER(C.c_int)]),
    ("ecs_params_from_options", C.c_int, [_vp, C.POINTER(EcsParams), C.c_char_p, C.c_int]),
    ("ecs_pic_app_from_options", C.c_int, [_vp, C.POINTER(EcsParams), C.POINTER(EcsPicApp), C.c_char_p, C.c_int]),
    ("ecs_solver_app_from_options", C.c_int, [_vp, C.POINTER(EcsSolverApp)]),
    ("ecs_echo_options", C.c_int, [C.c_char_p, _vp, C.POINTER(EcsParams)]),
    ("ecs_write_petsc_vec", C.c_int, [C.c_char_p, _vp, C.c_int64]),
    ("ecs_read_petsc_vec", C.c_int, [C.c_char_p, _vp, C.c_int64]),
    ("ecs_write_fluid", C.c_int, [C.c_char_p, _vp, _vp, _vp, C.c_int64]),
]

_gpu = None
_host = None


def _bind(lib, table):
    for name, res, args in table:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


def gpu():
    """The loaded libecsgpu; raises if it has not been built."""
    global _gpu
    if _gpu is None:
        if not GPU_LIB_PATH.exists():
            raise RuntimeError(f"{GPU_LIB_PATH} is missing: run `python -m ecsprt_gb300.build` (nvcc, sm_103a)")
        _gpu = _bind(C.CDLL(str(GPU_LIB_PATH)), GPU_API)
    return _gpu


def host():
    """The loaded libecshost (options, parameters, output files)."""
    global _host
    if _host is None:
        if not HOST_LIB_PATH.exists():
            raise RuntimeError(f"{HOST_LIB_PATH} is missing: run `python -m ecsprt_gb300.build`")
        _host = _bind(C.CDLL(str(HOST_LIB_PATH)), HOST_API)
    return _host
