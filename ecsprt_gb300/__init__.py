"""GB300 (sm_103a) implementation of the ECSPRT per-timestep hot path.

The compute lives in ``libecsgpu`` (CUDA C++, C ABI: include/ecsgpu.h); the
options database and output files in ``libecshost`` (C: include/ecs_host.h).
This module is a thin Python mirror of the reference's operator interface
(paths relative to the reference project):

=========================  ==============================================
reference                   here
=========================  ==============================================
ProcessOptions/SetUpContext :func:`params_from_options`
UpdateVelocities            :meth:`Context.update_velocities` (push, then
  (src/velocities.c:375)      collide when the neutral mass is positive)
BorisMoverBz3D              :meth:`Context.push`
ScatterElastic              :meth:`Context.collide`
UpdatePositions + BC        :meth:`Context.update_positions`
Collect3DFluidMoments       :meth:`Context.collect`
ComputeFullRHS3D            :meth:`Context.compute_rhs`
ComputeFullLHS3D            :meth:`Context.compute_lhs`
ComputePotential            :meth:`Context.compute_potential`
one step of src/pic.c:238   :meth:`Context.step`
=========================  ==============================================

Errors are raised as :class:`EcsError` carrying the library status code; the
reference's aborts (10 refused collisions, src/collisions.c:141-148; NaN) map
to ``ECS_ERR_COLLISION`` / ``ECS_ERR_NONFINITE``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import (ECS_PREC_FP64, ECS_PREC_MIXED, EcsParams, EcsPicApp, EcsSolveStats,
                   EcsSolverApp, EcsStepStats)

__all__ = [
    "ECS_PREC_FP64", "ECS_PREC_MIXED", "EcsError", "EcsParams", "Context", "Options",
    "params_from_options", "pic_app_from_options", "solver_app_from_options",
]


class EcsError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class Options:
    """PETSc-style options database (``-key value`` text or ``.ini`` files)."""

    def __init__(self, text: str = "", files=()):
        self._lib = _lib.host()
        self._h = self._lib.ecs_options_create()
        for f in files:
            if self._lib.ecs_options_load_file(self._h, str(f).encode()) != 0:
                raise EcsError(_lib.ECS_ERR_INVALID, f"cannot read options file {f}")
        if text:
            self.parse(text)

    def parse(self, text: str) -> "Options":
        rc = self._lib.ecs_options_parse(self._h, text.encode())
        if rc:
            raise EcsError(rc, "options parse failed")
        return self

    def get(self, key: str):
        found = C.c_int(0)
        v = self._lib.ecs_options_get(self._h, key.encode(), C.byref(found))
        if not found.value:
            return None
        return v.decode() if v is not None else True

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.ecs_options_destroy(self._h)
            self._h = None


def params_from_options(opts) -> EcsParams:
    """EcsParams from an options string or :class:`Options` (reference defaults)."""
    o = opts if isinstance(opts, Options) else Options(opts)
    p = EcsParams()
    err = C.create_string_buffer(256)
    rc = _lib.host().ecs_params_from_options(o._h, C.byref(p), err, 256)
    if rc:
        raise EcsError(rc, err.value.decode())
    return p


def pic_app_from_options(opts, params: EcsParams) -> EcsPicApp:
    o = opts if isinstance(opts, Options) else Options(opts)
    app = EcsPicApp()
    err = C.create_string_buffer(256)
    rc = _lib.host().ecs_pic_app_from_options(o._h, C.byref(params), C.byref(app), err, 256)
    if rc:
        raise EcsError(rc, err.value.decode())
    return app


def solver_app_from_options(opts) -> EcsSolverApp:
    o = opts if isinstance(opts, Options) else Options(opts)
    app = EcsSolverApp()
    _lib.host().ecs_solver_app_from_options(o._h, C.byref(app))
    return app


class Context:
    """Device state of one simulation (or solver) instance on one CUDA stream.

    ``precision`` is ``ECS_PREC_FP64`` (plain path) or ``ECS_PREC_MIXED``
    (cell-sorted FP32 particles, FP32 multigrid inside FP64 refinement).
    ``stream`` is an integer ``cudaStream_t`` (0: the context owns one).
    """

    def __init__(self, params: EcsParams, precision: int = ECS_PREC_MIXED, np_capacity: int = 0,
                 stream: int = 0):
        self._lib = _lib.gpu()
        self.params = params
        self.precision = precision
        h = C.c_void_p()
        rc = self._lib.ecs_ctx_create(C.byref(params), precision, int(np_capacity),
                                      C.c_void_p(stream) if stream else None, C.byref(h))
        if rc:
            raise EcsError(rc, self._lib.ecs_last_error(None).decode())
        self._h = h
        self.ncell = params.Nx * params.Ny * params.Nz
        self.shape = (params.Nz, params.Ny, params.Nx)

    # ---- plumbing --------------------------------------------------------
    def _check(self, rc: int):
        if rc:
            raise EcsError(rc, self._lib.ecs_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.ecs_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    @property
    def launches(self) -> int:
        return int(self._lib.ecs_launch_count(self._h))

    def sync(self):
        self._check(self._lib.ecs_ctx_sync(self._h))

    def set_sort_every(self, n: int):
        self._check(self._lib.ecs_set_sort_every(self._h, int(n)))

    def set_seed(self, seed: int):
        self._check(self._lib.ecs_set_seed(self._h, int(seed)))

    def set_warm_start(self, warm: bool):
        self._check(self._lib.ecs_set_warm_start(self._h, 1 if warm else 0))

    def set_solver_graphs(self, on: bool):
        """Run each FGMRES cycle as one CUDA graph (default) or step by step."""
        self._check(self._lib.ecs_set_solver_graphs(self._h, 1 if on else 0))

    # ---- data ----------------------------------------------------------
    def upload_particles(self, pos: np.ndarray, vel: np.ndarray):
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1, 3)
        if pos.shape != vel.shape:
            raise EcsError(_lib.ECS_ERR_INVALID, "pos and vel differ in shape")
        self._check(self._lib.ecs_particles_upload(self._h, _ptr(pos), _ptr(vel), pos.shape[0]))

    def download_particles(self):
        n = int(self._lib.ecs_particles_count(self._h))
        pos = np.empty((n, 3))
        vel = np.empty((n, 3))
        self._check(self._lib.ecs_particles_download(self._h, _ptr(pos), _ptr(vel)))
        return pos, vel

    @property
    def phi(self) -> np.ndarray:
        out = np.empty(self.shape)
        self._check(self._lib.ecs_phi_download(self._h, _ptr(out)))
        return out

    @phi.setter
    def phi(self, value):
        a = np.ascontiguousarray(value, dtype=np.float64).reshape(self.shape)
        self._check(self._lib.ecs_phi_upload(self._h, _ptr(a)))

    @property
    def moments(self) -> np.ndarray:
        out = np.empty(self.shape + (4,))
        self._check(self._lib.ecs_moments_download(self._h, _ptr(out)))
        return out

    @moments.setter
    def moments(self, value):
        a = np.ascontiguousarray(value, dtype=np.float64).reshape(self.shape + (4,))
        self._check(self._lib.ecs_moments_upload(self._h, _ptr(a)))

    @property
    def rhs(self) -> np.ndarray:
        out = np.empty(self.shape)
        self._check(self._lib.ecs_rhs_download(self._h, _ptr(out)))
        return out

    # ---- operators -------------------------------------------------------
    def push(self, dt: float):
        self._check(self._lib.ecs_push(self._h, float(dt)))

    def collide(self, dt: float):
        self._check(self._lib.ecs_collide(self._h, float(dt)))

    def update_velocities(self, dt: float):
        """UpdateVelocities: push, then collide if the neutral mass is positive."""
        self.push(dt)
        if self.params.mn > 0.0:
            self.collide(dt)

    def update_positions(self, dt: float):
        """UpdatePositions + ApplyBCAndMigrate."""
        self._check(self._lib.ecs_move(self._h, float(dt)))

    def collect(self):
        self._check(self._lib.ecs_collect(self._h))

    def compute_rhs(self):
        self._check(self._lib.ecs_rhs(self._h))

    def compute_lhs(self):
        self._check(self._lib.ecs_lhs(self._h))

    def solve(self, rtol: float = 1e-8, max_it: int = 200, warm_start: bool = False) -> EcsSolveStats:
        st = EcsSolveStats()
        self._check(self._lib.ecs_solve(self._h, float(rtol), int(max_it), 1 if warm_start else 0, C.byref(st)))
        return st

    def compute_potential(self, rtol: float = 1e-8, max_it: int = 200) -> EcsSolveStats:
        """ComputePotential: RHS, operator, then the solve from phi = 0."""
        self.compute_rhs()
        self.compute_lhs()
        return self.solve(rtol, max_it)

    def lhs_apply(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(self.shape)
        y = np.empty(self.shape)
        self._check(self._lib.ecs_lhs_apply_host(self._h, _ptr(x), _ptr(y)))
        return y

    def step(self, dt: float, rtol: float = 1e-8, max_it: int = 200) -> EcsStepStats:
        st = EcsStepStats()
        self._check(self._lib.ecs_step(self._h, float(dt), float(rtol), int(max_it), C.byref(st)))
        return st

    def step_host(self, pos: np.ndarray, vel: np.ndarray, dt: float, rtol: float = 1e-8, max_it: int = 200,
                  moments_out: np.ndarray | None = None, phi_out: np.ndarray | None = None) -> EcsStepStats:
        st = EcsStepStats()
        self._check(self._lib.ecs_step_host(
            self._h, _ptr(pos), _ptr(vel), pos.shape[0], float(dt), float(rtol), int(max_it),
            _ptr(moments_out) if moments_out is not None else None,
            _ptr(phi_out) if phi_out is not None else None, C.byref(st)))
        return st
