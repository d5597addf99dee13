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
src/solver.c:107-170        :meth:`Context.solve_density` (density in,
  (LoadFluidQuantities +      fluxes = flux_scale * density, potential out)
  ComputePotential)
=========================  ==============================================

:class:`Server` (include/ecs_serve.h) runs many stand-alone solves and small
simulations at once on one GPU: resident slots admitted against an HBM
budget, each solve one CUDA-graph launch, p50/p99 latency in its stats.

Errors are raised as :class:`EcsError` carrying the library status code; the
reference's aborts (10 refused collisions, src/collisions.c:141-148; NaN) map
to ``ECS_ERR_COLLISION`` / ``ECS_ERR_NONFINITE``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

import weakref

from . import _lib
from ._lib import (ECS_INIT_MODES, ECS_INIT_RANDOM, ECS_INIT_SINUSOIDAL, ECS_INIT_SOBOL, ECS_PREC_FP64,
                   ECS_PREC_MIXED, ECS_SERVE_SIM, ECS_SERVE_SOLVE, EcsDensityModes, EcsParams, EcsPicApp,
                   EcsServeConfig, EcsServeResult, EcsServeStats, EcsSimRequest, EcsSolveRequest, EcsSolveStats,
                   EcsSolverApp, EcsStepStats)

__all__ = [
    "ECS_INIT_MODES", "ECS_INIT_RANDOM", "ECS_INIT_SINUSOIDAL", "ECS_INIT_SOBOL", "density_modes",
    "ECS_PREC_FP64", "ECS_PREC_MIXED", "ECS_SERVE_SIM", "ECS_SERVE_SOLVE", "EcsError", "EcsParams", "Context",
    "Options", "Server", "pinned_empty", "serve_request_bytes", "params_from_options", "pic_app_from_options", "solver_app_from_options",
]


class EcsError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def _f64(a, shape=None, writeable=False, name="array") -> np.ndarray:
    """a as it is, if it is a C-contiguous float64 array (of `shape`); the
    library reads and writes through its address."""
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous:
        raise ValueError(f"{name} must be a C-contiguous float64 numpy array")
    if shape is not None and a.size != int(np.prod(shape)):
        raise ValueError(f"{name} has {a.size} values, expected {int(np.prod(shape))}")
    if writeable and not a.flags.writeable:
        raise ValueError(f"{name} must be writeable")
    return a


def density_modes(modes) -> EcsDensityModes:
    """EcsDensityModes from [(kx, ky, kz, amplitude, phase), ...]: density
    1 + sum a cos(2 pi k.(x/L) + phase)."""
    m = EcsDensityModes()
    modes = list(modes)
    if len(modes) > 16:
        raise ValueError("at most 16 modes")
    m.nmodes = len(modes)
    for q, (kx, ky, kz, a, ph) in enumerate(modes):
        m.k[q][0], m.k[q][1], m.k[q][2] = int(kx), int(ky), int(kz)
        m.amplitude[q] = float(a)
        m.phase[q] = float(ph)
    return m


def pinned_empty(shape) -> np.ndarray:
    """Uninitialised float64 array in page-locked host memory: request
    buffers the copy engines read and write directly."""
    n = int(np.prod(shape))
    lib = _lib.gpu()
    ptr = lib.ecs_host_alloc(max(n, 1) * 8)
    if not ptr:
        raise MemoryError(f"page-locked allocation of {n * 8} bytes failed")
    buf = (C.c_double * max(n, 1)).from_address(ptr)
    weakref.finalize(buf, lib.ecs_host_free, C.c_void_p(ptr))
    return np.ctypeslib.as_array(buf)[:n].reshape(shape)


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
        self.nd = 2 if params.ndim == 2 else 3  # components an ion in host arrays

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
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, self.nd)
        vel = np.ascontiguousarray(vel, dtype=np.float64).reshape(-1, self.nd)
        if pos.shape != vel.shape:
            raise EcsError(_lib.ECS_ERR_INVALID, "pos and vel differ in shape")
        self._check(self._lib.ecs_particles_upload(self._h, _ptr(pos), _ptr(vel), pos.shape[0]))

    def init_particles(self, dist: int, np_: int, seed: int = 20261203, modes=None):
        """Initial ions generated on the device (ecs_particles_init): Sobol
        positions as the reference's (``ECS_INIT_SOBOL``), uniform random
        (``ECS_INIT_RANDOM``), the reference's sinusoidal rejection
        (``ECS_INIT_SINUSOIDAL``) or Fourier-mode densities (``ECS_INIT_MODES``,
        ``modes`` from :func:`density_modes`); Maxwellian velocities."""
        m = modes if modes is None or isinstance(modes, EcsDensityModes) else density_modes(modes)
        self._check(self._lib.ecs_particles_init(self._h, int(dist), int(np_), int(seed),
                                                 C.byref(m) if m is not None else None))

    def download_particles(self):
        n = int(self._lib.ecs_particles_count(self._h))
        pos = np.empty((n, self.nd))
        vel = np.empty((n, self.nd))
        self._check(self._lib.ecs_particles_download(self._h, _ptr(pos), _ptr(vel)))
        return pos, vel

    def particle_ids(self) -> np.ndarray:
        """Identity of each ion in the order of :meth:`download_particles`:
        its index in the arrays of the last upload (ecs_particles_ids)."""
        n = int(self._lib.ecs_particles_count(self._h))
        ids = np.empty(n, dtype=np.int32)
        self._check(self._lib.ecs_particles_ids(self._h, _ptr(ids)))
        return ids

    def download_particles_in_upload_order(self):
        """The ions in the order of the last upload (the mixed path's cell
        sort reorders them on the device)."""
        pos, vel = self.download_particles()
        ids = self.particle_ids()
        out_p, out_v = np.empty_like(pos), np.empty_like(vel)
        out_p[ids] = pos
        out_v[ids] = vel
        return out_p, out_v

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

    def solve_density(self, density: np.ndarray, flux_scale=(1.0, 1.0, 1.0), rtol: float = 1e-8,
                      max_it: int = 200, phi_out: np.ndarray | None = None):
        """The stand-alone solver (src/solver.c:158-163): moments from a
        density (fluxes = flux_scale * density, src/file-io.c:51-59), RHS,
        operator and the solve from phi = 0, as one CUDA graph.  Returns
        (phi, stats)."""
        d = _f64(density, self.shape, name="density")
        phi = phi_out if phi_out is not None else np.empty(self.shape)
        _f64(phi, self.shape, writeable=True, name="phi_out")
        fs = (C.c_double * 3)(*[float(v) for v in flux_scale])
        st = EcsSolveStats()
        self._check(self._lib.ecs_solve_density(self._h, _ptr(d), C.byref(fs), float(rtol), int(max_it), _ptr(phi),
                                                C.byref(st)))
        return phi.reshape(self.shape), st

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


def serve_request_bytes(params: EcsParams, precision: int = ECS_PREC_MIXED, kind: int = ECS_SERVE_SOLVE,
                        np_: int = 0) -> int:
    """Device bytes a served request's slot is charged (ecs_serve_request_bytes)."""
    return int(_lib.gpu().ecs_serve_request_bytes(C.byref(params), int(precision), int(kind), int(np_)))


def _result_dict(r: EcsServeResult) -> dict:
    return {
        "id": int(r.id), "kind": "solve" if r.kind == ECS_SERVE_SOLVE else "sim", "status": int(r.status),
        "latency": r.latency, "queued": r.queued, "device_seconds": r.device_seconds,
        "iterations": int(r.solve.iterations), "refinements": int(r.solve.refinements), "relres": r.solve.relres,
        "steps": int(r.steps), "slot_reused": bool(r.slot_reused), "message": r.message.decode(errors="replace"),
    }


class Server:
    """Request loop on one GPU (include/ecs_serve.h).

    Stand-alone solves (:meth:`submit_solve`) and simulation instances
    (:meth:`submit_sim`) are admitted first come, first served as worker
    slots and the HBM budget allow; their device state stays resident, solve
    slots are reused by later requests with the same parameters, and the
    work of concurrent requests overlaps on the GPU.  The arrays passed to a
    request are held until its result is polled; page-locked ones
    (:func:`pinned_empty`) are copied by DMA directly.
    """

    def __init__(self, hbm_budget_bytes: int, max_inflight: int = 8, precision: int = ECS_PREC_MIXED,
                 timeout_seconds: float = 60.0):
        self._lib = _lib.gpu()
        cfg = EcsServeConfig(int(hbm_budget_bytes), int(max_inflight), int(precision), float(timeout_seconds))
        h = C.c_void_p()
        rc = self._lib.ecs_serve_create(C.byref(cfg), C.byref(h))
        if rc:
            raise EcsError(rc, "server create failed")
        self._h = h
        self.precision = precision
        self._live = {}  # id -> arrays the request reads or writes

    def close(self):
        if getattr(self, "_h", None):
            self._lib.ecs_serve_destroy(self._h)
            self._h = None
            self._live.clear()

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def request_bytes(self, params: EcsParams, kind: int = ECS_SERVE_SOLVE, np_: int = 0) -> int:
        return serve_request_bytes(params, self.precision, kind, np_)

    def submit_solve(self, params: EcsParams, density: np.ndarray, phi_out: np.ndarray,
                     flux_scale=(1.0, 1.0, 1.0), rtol: float = 1e-8, max_it: int = 200) -> int:
        shape = (params.Nz, params.Ny, params.Nx)
        _f64(density, shape, name="density")
        _f64(phi_out, shape, writeable=True, name="phi_out")
        req = EcsSolveRequest(density.ctypes.data, (C.c_double * 3)(*[float(v) for v in flux_scale]),
                              float(rtol), int(max_it), phi_out.ctypes.data)
        rid = C.c_int64()
        rc = self._lib.ecs_serve_submit_solve(self._h, C.byref(params), C.byref(req), C.byref(rid))
        if rc:
            raise EcsError(rc, "solve request refused")
        self._live[rid.value] = (params, density, phi_out)
        return rid.value

    def submit_sim(self, params: EcsParams, pos: np.ndarray, vel: np.ndarray, nsteps: int, dt: float,
                   seed: int = 20261203, rtol: float = 1e-8, max_it: int = 200, sort_every: int = 0,
                   step_seconds: np.ndarray | None = None, phi_out: np.ndarray | None = None,
                   pos_out: np.ndarray | None = None, vel_out: np.ndarray | None = None) -> int:
        n = pos.shape[0]
        nd = 2 if params.ndim == 2 else 3
        _f64(pos, (n, nd), name="pos")
        _f64(vel, (n, nd), name="vel")
        outs = {"step_seconds": (step_seconds, (int(nsteps),)), "phi_out": (phi_out, (params.Nz, params.Ny, params.Nx)),
                "pos_out": (pos_out, (n, nd)), "vel_out": (vel_out, (n, nd))}
        ptrs = {}
        for k, (a, shp) in outs.items():
            ptrs[k] = None
            if a is not None:
                _f64(a, shp, writeable=True, name=k)
                ptrs[k] = a.ctypes.data
        req = EcsSimRequest(pos.ctypes.data, vel.ctypes.data, n, int(seed), int(nsteps), int(sort_every),
                            float(dt), float(rtol), int(max_it), ptrs["step_seconds"], ptrs["phi_out"],
                            ptrs["pos_out"], ptrs["vel_out"])
        rid = C.c_int64()
        rc = self._lib.ecs_serve_submit_sim(self._h, C.byref(params), C.byref(req), C.byref(rid))
        if rc:
            raise EcsError(rc, "simulation request refused")
        self._live[rid.value] = (params, pos, vel, step_seconds, phi_out, pos_out, vel_out)
        return rid.value

    def poll(self, max_results: int = 256, timeout_ms: int = 0) -> list:
        """Finished requests as dicts (id, kind, status, latency, ...)."""
        buf = (EcsServeResult * max_results)()
        n = self._lib.ecs_serve_poll(self._h, buf, max_results, int(timeout_ms))
        if n < 0:
            raise EcsError(n, "poll failed")
        out = []
        for q in range(n):
            self._live.pop(int(buf[q].id), None)
            out.append(_result_dict(buf[q]))
        return out

    def wait_all(self, timeout_s: float = 600.0) -> list:
        """Poll until every submitted request has a result."""
        import time
        out = []
        t_end = time.monotonic() + timeout_s
        while self.pending > 0:
            if time.monotonic() > t_end:
                raise TimeoutError(f"{self.pending} requests still pending")
            out += self.poll(256, 100)
        return out

    @property
    def pending(self) -> int:
        return int(self._lib.ecs_serve_pending(self._h))

    def stats(self) -> dict:
        st = EcsServeStats()
        rc = self._lib.ecs_serve_stats(self._h, C.byref(st))
        if rc:
            raise EcsError(rc, "stats failed")
        return st.as_dict()

    def reset_stats(self):
        self._lib.ecs_serve_reset_stats(self._h)
