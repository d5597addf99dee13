"""ctypes wrapper of the ECSPRT oracle (oracle/ecs_oracle.c).

TEST INFRASTRUCTURE: the oracle is the checker.  Only tests/,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use it.  The
product path (ecsprt_gb300) never imports this module.

Also wraps ``oracle/_ref/libecsref.so`` (the reference's own sources compiled
against the PETSc-API shim, :mod:`oracle.ref`) when it has been built.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"


class OrcParams(C.Structure):
    _fields_ = [
        ("Nx", C.c_int), ("Ny", C.c_int), ("Nz", C.c_int), ("bc", C.c_int * 3),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("x0", C.c_double), ("y0", C.c_double), ("z0", C.c_double),
        ("x1", C.c_double), ("y1", C.c_double), ("z1", C.c_double),
        ("Lx", C.c_double), ("Ly", C.c_double), ("Lz", C.c_double),
        ("qi", C.c_double), ("mi", C.c_double), ("B0", C.c_double), ("E0", C.c_double),
        ("nui", C.c_double), ("viT", C.c_double), ("vi0", C.c_double * 3),
        ("mn", C.c_double), ("vnT", C.c_double), ("vn0", C.c_double * 3), ("vn0mag", C.c_double),
        ("kappa_e", C.c_double), ("scale", C.c_double), ("cth", C.c_double), ("cG", C.c_double),
        ("n0", C.c_double), ("lhs_type", C.c_int), ("rhs_type", C.c_int), ("ndim", C.c_int),
    ]


def build() -> Path:
    """Compile the oracle (make -C oracle)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        P = C.POINTER(OrcParams)
        vp = C.c_void_p
        sig = {
            "orc_push": (C.c_int, [P, C.c_int, vp, vp, vp, C.c_double]),
            "orc_move": (C.c_int, [P, C.c_int, vp, vp, C.c_double]),
            "orc_collect": (C.c_int, [P, C.c_int, vp, vp, vp]),
            "orc_collect_fixed": (C.c_int, [P, C.c_int, vp, vp, C.c_int, C.c_int, vp, vp]),
            "orc_collect_mt": (C.c_int, [P, C.c_int, vp, vp, vp]),
            "orc_rhs": (C.c_int, [P, vp, vp]),
            "orc_lhs_dense": (C.c_int, [P, vp, vp]),
            "orc_lhs_apply": (C.c_int, [P, vp, vp, vp]),
            "orc_gmres": (C.c_int, [P, vp, vp, vp, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_double)]),
            "orc_rng_reset": (None, []),
            "orc_ran1_n": (C.c_int, [C.POINTER(C.c_long), C.c_int, vp]),
            "orc_ran3_n": (C.c_int, [C.POINTER(C.c_long), C.c_int, vp]),
            "orc_gasdev_n": (C.c_int, [C.POINTER(C.c_long), C.c_int, vp]),
            "orc_sobol": (C.c_int, [P, C.c_int, vp]),
            "orc_push2d": (C.c_int, [P, C.c_int, vp, vp, vp, C.c_double]),
            "orc_move2d": (C.c_int, [P, C.c_int, vp, vp, C.c_double]),
            "orc_collect2d": (C.c_int, [P, C.c_int, vp, vp, vp]),
            "orc_collect2d_fixed": (C.c_int, [P, C.c_int, vp, vp, C.c_int, C.c_int, vp]),
            "orc_normal_velocities": (C.c_int, [vp, vp, C.c_int, vp]),
            "orc_collide": (C.c_int, [P, C.c_int, vp, C.c_double, vp]),
            "orc_collision_count": (C.c_int, [P, C.c_int, C.c_double]),
            "orc_num_threads": (C.c_int, []),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return C.c_void_p(a.ctypes.data)


KB = 1.3807e-23  # src/constants.h:7
Q = 1.6022e-19   # src/constants.h:4


def from_ref_context(d: dict) -> dict:
    """Parameter dict in EcsParams naming from the reference context values
    (oracle/ref.py Ref.params): boundary triplet, and the RHS coefficients of
    src/rhs.c:291-292 evaluated in the same order."""
    out = dict(d)
    out["bc"] = [int(d["xBC"]), int(d["yBC"]), int(d["zBC"])]
    out["lhs_type"], out["rhs_type"] = int(d["lhsType"]), int(d["rhsType"])
    out["cth"] = d["gammaT"] * KB * d["Te"] / Q
    out["cG"] = (1 + d["kappa_e"] * d["kappa_e"]) * d["me"] * d["nue"] / Q
    return out


def params_from(p) -> OrcParams:
    """OrcParams from an EcsParams-like object or dict of the derived context."""
    if isinstance(p, dict) and "bc" not in p:
        p = from_ref_context(p)
    g = (lambda k: p[k]) if isinstance(p, dict) else (lambda k: getattr(p, k))
    o = OrcParams()
    o.Nx, o.Ny, o.Nz = int(g("Nx")), int(g("Ny")), int(g("Nz"))
    bc = g("bc")
    for d in range(3):
        o.bc[d] = 0 if int(bc[d]) == 0 else 1
    for k in ("dx", "dy", "dz", "x0", "y0", "z0", "x1", "y1", "z1", "Lx", "Ly", "Lz",
              "qi", "mi", "B0", "E0", "nui", "viT", "mn", "vnT", "kappa_e", "scale", "cth", "cG", "n0"):
        setattr(o, k, float(g(k)))
    o.lhs_type, o.rhs_type = int(g("lhs_type")), int(g("rhs_type"))
    o.ndim = int(g("ndim"))
    o.vi0[0], o.vi0[1], o.vi0[2] = float(g("vi0x")), float(g("vi0y")), float(g("vi0z"))
    o.vn0[0], o.vn0[1], o.vn0[2] = float(g("vn0x")), float(g("vn0y")), float(g("vn0z"))
    o.vn0mag = float(g("vn0"))
    return o


class Oracle:
    """FP64 restatement of the reference's hot path (arrays are numpy)."""

    def __init__(self, params):
        self.L = lib()
        self.p = params_from(params)
        self.shape = (self.p.Nz, self.p.Ny, self.p.Nx)

    def push(self, pos, vel, phi, dt):
        vel = np.array(vel, dtype=np.float64, order="C")
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        f = self.L.orc_push2d if self.p.ndim == 2 else self.L.orc_push
        f(C.byref(self.p), pos.shape[0], _p(pos), _p(vel), _p(phi), dt)
        return vel

    def move(self, pos, vel, dt):
        pos = np.array(pos, dtype=np.float64, order="C")
        vel = np.array(vel, dtype=np.float64, order="C")
        f = self.L.orc_move2d if self.p.ndim == 2 else self.L.orc_move
        f(C.byref(self.p), pos.shape[0], _p(pos), _p(vel), dt)
        return pos, vel

    def collect(self, pos, vel):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        out = np.zeros(self.shape + (4,))
        f = self.L.orc_collect2d if self.p.ndim == 2 else self.L.orc_collect
        f(C.byref(self.p), pos.shape[0], _p(pos), _p(vel), _p(out))
        return out

    def collect_mt(self, pos, vel):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        out = np.zeros(self.shape + (4,))
        self.L.orc_collect_mt(C.byref(self.p), pos.shape[0], _p(pos), _p(vel), _p(out))
        return out

    def collect_fixed(self, pos, vel, shift_n, shift_f):
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        vel = np.ascontiguousarray(vel, dtype=np.float64)
        out = np.zeros(self.shape + (4,))
        if self.p.ndim == 2:
            self.L.orc_collect2d_fixed(C.byref(self.p), pos.shape[0], _p(pos), _p(vel), shift_n, shift_f, _p(out))
            return out, None
        acc = np.zeros(self.shape + (4,), dtype=np.int64)
        self.L.orc_collect_fixed(C.byref(self.p), pos.shape[0], _p(pos), _p(vel), shift_n, shift_f, _p(out), _p(acc))
        return out, acc

    def rhs(self, moments):
        m = np.ascontiguousarray(moments, dtype=np.float64)
        b = np.zeros(self.shape)
        self.L.orc_rhs(C.byref(self.p), _p(m), _p(b))
        return b

    def lhs_dense(self, density):
        n = np.ascontiguousarray(density, dtype=np.float64)
        N = n.size
        A = np.zeros((N, N))
        self.L.orc_lhs_dense(C.byref(self.p), _p(n), _p(A))
        return A

    def lhs_apply(self, density, x):
        n = np.ascontiguousarray(density, dtype=np.float64)
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.shape)
        self.L.orc_lhs_apply(C.byref(self.p), _p(n), _p(x), _p(y))
        return y

    def solve(self, density, b, rtol=1e-12, maxit=20000, restart=60):
        n = np.ascontiguousarray(density, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.shape)
        rel = C.c_double(0)
        its = self.L.orc_gmres(C.byref(self.p), _p(n), _p(b), _p(x), rtol, maxit, restart, C.byref(rel))
        return x, its, rel.value

    def solve_fft(self, density, b, rtol=1e-13, maxit=400, restart=40):
        """The same converged potential as :meth:`solve`, reached faster on a
        fully periodic grid: restarted GMRES right-preconditioned by the
        operator assembled from the mean density (constant coefficients, so
        a periodic convolution that the FFT diagonalises; its stencil is the
        oracle operator's response to a unit impulse).  The operator applied
        is the oracle's variable-coefficient one throughout, the iterate is
        kept mean-free as the reference's null-space projection does, and
        the stop test is the true FP64 residual ||b - A x|| / ||b||.  Grids
        with a non-periodic axis use :meth:`solve`."""
        if any(int(c) for c in self.p.bc):
            return self.solve(density, b, rtol=rtol)
        n = np.ascontiguousarray(density, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        imp = np.zeros(self.shape)
        imp[0, 0, 0] = 1.0
        lam = np.fft.fftn(self.lhs_apply(np.full(self.shape, n.mean()), imp))
        lam[0, 0, 0] = np.inf  # the constant null space: no mean in the correction

        def prec(r):
            return np.real(np.fft.ifftn(np.fft.fftn(r) / lam))

        def mf(v):
            return v - v.mean()

        bnorm = np.linalg.norm(b)
        x = np.zeros(self.shape)
        if bnorm == 0.0:
            return x, 0, 0.0
        its = 0
        while True:
            r = b - self.lhs_apply(n, x)
            rel = np.linalg.norm(r) / bnorm
            if rel <= rtol or its >= maxit:
                return mf(x), its, rel
            beta = np.linalg.norm(r)
            V = [r / beta]
            Z = []
            H = np.zeros((restart + 1, restart))
            for j in range(restart):
                z = prec(V[j])
                Z.append(z)
                w = self.lhs_apply(n, z)
                for q in range(j + 1):  # modified Gram-Schmidt, twice
                    h = np.vdot(V[q], w)
                    H[q, j] += h
                    w = w - h * V[q]
                for q in range(j + 1):
                    h = np.vdot(V[q], w)
                    H[q, j] += h
                    w = w - h * V[q]
                H[j + 1, j] = np.linalg.norm(w)
                its += 1
                e1 = np.zeros(j + 2)
                e1[0] = beta
                y, *_ = np.linalg.lstsq(H[: j + 2, : j + 1], e1, rcond=None)
                est = np.linalg.norm(H[: j + 2, : j + 1] @ y - e1) / bnorm
                if H[j + 1, j] == 0.0 or est <= 0.1 * rtol or its >= maxit:
                    break
                V.append(w / H[j + 1, j])
            x = mf(x + sum(yq * zq for yq, zq in zip(y, Z)))

    def collide(self, vel, dt):
        vel = np.array(vel, dtype=np.float64, order="C")
        stats = np.zeros(3, dtype=np.int64)
        ns = self.L.orc_collide(C.byref(self.p), vel.shape[0], _p(vel), dt, _p(stats))
        return vel, ns, stats

    def collision_count(self, np_, dt):
        return self.L.orc_collision_count(C.byref(self.p), np_, dt)

    def sobol(self, np_):
        pos = np.zeros((np_, 3))
        self.L.orc_sobol(C.byref(self.p), np_, _p(pos))
        return pos


def rng_reset():
    lib().orc_rng_reset()


def ran1(seed, n):
    s = C.c_long(seed)
    out = np.zeros(n, dtype=np.float32)
    lib().orc_ran1_n(C.byref(s), n, _p(out))
    return out, s.value


def ran3(seed, n):
    s = C.c_long(seed)
    out = np.zeros(n, dtype=np.float32)
    lib().orc_ran3_n(C.byref(s), n, _p(out))
    return out, s.value


def gasdev(seed, n):
    s = C.c_long(seed)
    out = np.zeros(n, dtype=np.float32)
    lib().orc_gasdev_n(C.byref(s), n, _p(out))
    return out, s.value


def normal_velocities(vT, v0, np_):
    vT = np.ascontiguousarray(vT, dtype=np.float64)
    v0 = np.ascontiguousarray(v0, dtype=np.float64)
    vel = np.zeros((np_, 3))
    lib().orc_normal_velocities(_p(vT), _p(v0), np_, _p(vel))
    return vel


def num_threads() -> int:
    return lib().orc_num_threads()
