"""ctypes wrapper of oracle/_ref/libecsref.so: the reference's own hot-path C
sources (unmodified, compiled from where they lie) linked with the PETSc-API
shim in oracle/ref_shim.

TEST INFRASTRUCTURE ONLY, and only where the reference sources are present
(the container that holds the reference checkout).  Build with
``build(<reference>/src)`` or ``make -C oracle/ref_shim REF=<reference>/src``;
without an argument :func:`build` takes the checkout from the environment
variable ECSPRT_REFERENCE.

The reference keeps process-global RNG and Sobol state (src/random.c), so
callers that need a freshly started reference run each case in its own
process.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_ref" / "libecsref.so"


def env_ref_src() -> Path | None:
    """<checkout>/src of the reference named by ECSPRT_REFERENCE, or None."""
    root = os.environ.get("ECSPRT_REFERENCE")
    return Path(root) / "src" if root else None


def available() -> bool:
    src = env_ref_src()
    return LIB_PATH.exists() or (src is not None and src.exists())


def build(ref_src: Path | None = None) -> Path:
    ref_src = ref_src if ref_src is not None else env_ref_src()
    if ref_src is None or not Path(ref_src).exists():
        raise RuntimeError(f"reference sources not found (given {ref_src}; set ECSPRT_REFERENCE)")
    subprocess.run(["make", "-s", "-C", str(HERE / "ref_shim"), f"REF={ref_src}"], check=True)
    return LIB_PATH


def _p(a):
    return C.c_void_p(a.ctypes.data)


class Ref:
    """One reference context (the library holds a single global context)."""

    def __init__(self, opts: str, Np: int):
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        L.ref_param_names.restype = C.c_char_p
        L.ref_last_error.restype = C.c_char_p
        for name in ("ref_push", "ref_collide", "ref_update_velocities", "ref_update_positions"):
            getattr(L, name).argtypes = [C.c_double]
        self.L = L
        rc = L.ref_setup(opts.encode(), int(Np))
        if rc:
            raise RuntimeError(f"ref_setup failed ({rc}): {L.ref_last_error().decode()}")
        names = L.ref_param_names().decode().split(",")
        vals = np.zeros(len(names) + 8)
        n = L.ref_params(_p(vals))
        self.params = dict(zip(names, vals[:n].tolist()))
        self.shape = tuple(int(self.params[k]) for k in ("Nz", "Ny", "Nx"))

    def _rc(self, rc, what):
        if rc:
            raise RuntimeError(f"{what} failed ({rc}): {self.L.ref_last_error().decode()}")
        return rc

    @property
    def np(self) -> int:
        return self.L.ref_np()

    def set_particles(self, pos, vel):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        self.L.ref_set_particles(_p(pos), _p(vel), pos.shape[0])

    def get_particles(self):
        n, nd = self.np, int(self.params["ndim"])
        pos = np.zeros((n, nd))
        vel = np.zeros((n, nd))
        self.L.ref_get_particles(_p(pos), _p(vel))
        return pos, vel

    def set_phi(self, phi):
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        self.L.ref_set_phi(_p(phi))

    def set_moments(self, m):
        m = np.ascontiguousarray(m, dtype=np.float64)
        self.L.ref_set_moments(_p(m))

    def get_moments(self):
        m = np.zeros(self.shape + (4,))
        self.L.ref_get_moments(_p(m))
        return m

    def push(self, dt):
        return self._rc(self.L.ref_push(dt), "push")

    def collide(self, dt):
        return self.L.ref_collide(dt)

    def update_velocities(self, dt):
        return self.L.ref_update_velocities(dt)

    def update_positions(self, dt):
        return self._rc(self.L.ref_update_positions(dt), "update_positions")

    def collect(self):
        return self._rc(self.L.ref_collect(), "collect")

    def init_positions(self, pdist=0):
        return self._rc(self.L.ref_init_positions(pdist), "init_positions")

    def init_velocities(self):
        return self._rc(self.L.ref_init_velocities(), "init_velocities")

    def rhs(self):
        b = np.zeros(self.shape)
        self._rc(self.L.ref_rhs(_p(b)), "rhs")
        return b

    def lhs_dense(self):
        n = self.L.ref_lhs_size()
        A = np.zeros((n, n))
        rc = self.L.ref_lhs_dense(_p(A))
        if rc < 0:
            raise RuntimeError("lhs failed")
        return A

    def echo_options(self, path):
        return self._rc(self.L.ref_echo_options(str(path).encode()), "echo_options")

    def ran1(self, seed, n):
        s = C.c_long(seed)
        out = np.zeros(n, dtype=np.float32)
        self.L.ref_ran1(C.byref(s), n, _p(out))
        return out, s.value

    def ran3(self, seed, n):
        s = C.c_long(seed)
        out = np.zeros(n, dtype=np.float32)
        self.L.ref_ran3(C.byref(s), n, _p(out))
        return out, s.value

    def gasdev(self, seed, n):
        s = C.c_long(seed)
        out = np.zeros(n, dtype=np.float32)
        self.L.ref_gasdev(C.byref(s), n, _p(out))
        return out, s.value
