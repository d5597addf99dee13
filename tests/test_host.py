"""Host layer (libecshost) and the C-ABI surface; no GPU needed."""
import ctypes
import re
import struct
from pathlib import Path

import numpy as np
import pytest

import ecsprt_gb300 as E
from ecsprt_gb300 import _lib

ROOT = Path(__file__).resolve().parent.parent

# EcsParams field name for each reference context value (oracle/ref.py names)
REF_TO_ECS = {
    "ndim": "ndim", "Nx": "Nx", "Ny": "Ny", "Nz": "Nz", "dx": "dx", "dy": "dy", "dz": "dz",
    "Lx": "Lx", "Ly": "Ly", "Lz": "Lz", "x0": "x0", "y0": "y0", "z0": "z0", "x1": "x1", "y1": "y1",
    "z1": "z1", "qi": "qi", "mi": "mi", "B0": "B0", "E0": "E0", "n0": "n0", "nui": "nui", "viT": "viT",
    "viTx": "viTx", "viTy": "viTy", "viTz": "viTz", "vi0x": "vi0x", "vi0y": "vi0y", "vi0z": "vi0z",
    "vi0": "vi0", "Ti": "Ti", "Omega_i": "Omega_i", "kappa_i": "kappa_i", "qe": "qe", "me": "me",
    "nue": "nue", "Te": "Te", "kappa_e": "kappa_e", "Omega_e": "Omega_e", "mn": "mn", "Tn": "Tn",
    "vnT": "vnT", "vn0x": "vn0x", "vn0y": "vn0y", "vn0z": "vn0z", "vn0": "vn0", "scale": "scale",
    "gammaT": "gammaT", "lhsType": "lhs_type", "rhsType": "rhs_type",
}


@pytest.mark.parametrize("case", ["c1", "edge", "fb"])
def test_params_match_reference_context(built, golden, case):
    """ProcessOptions + SetUpContext + NormalizeGrid reproduce the
    reference's derived context values exactly."""
    g = golden[case]
    p = E.params_from_options(g["opts"])
    for rk, ek in REF_TO_ECS.items():
        assert getattr(p, ek) == g["params"][rk], (rk, getattr(p, ek), g["params"][rk])
    assert list(p.bc) == [int(g["params"][k]) for k in ("xBC", "yBC", "zBC")]


def test_defaults_and_overrides(built):
    p = E.params_from_options("")
    assert (p.Nx, p.Ny, p.Nz) == (7, 7, 7)
    assert p.dx == 1.0 / 7 and p.x0 == 0.0 and p.x1 == 1.0
    assert p.lhs_type == 2 and p.rhs_type == 2 and p.ndim == 3
    assert p.mn == p.mi == 1.6726e-27
    p = E.params_from_options("-Nx 8 -da_grid_x 12 -vi0 2 -vi0y -1 -xBC periodic -zBC inject-reflect")
    assert p.Nx == 12
    assert (p.vi0x, p.vi0y, p.vi0z) == (2.0, -1.0, 2.0)
    assert list(p.bc) == [0, 0, 1]
    with pytest.raises(E.EcsError):
        E.params_from_options("-lhs nonsense")


def test_options_file_and_pic_app(built, tmp_path):
    ini = tmp_path / "petsc.ini"
    ini.write_text("# comment line\n-Nx 16 -Ny 16\n-Nz 8   # trailing comment\n-dx 0.5 -dy 0.5 -dz 0.5\n"
                   "-Np -4\n-Nt 3\n--every 2\n--output-particles\n-nui 0.05\n")
    o = E.Options(files=[ini])
    assert o.get("--output-particles") is True
    assert o.get("-Nz") == "8"
    p = E.params_from_options(o)
    app = E.pic_app_from_options(o, p)
    assert (app.Nt, app.every, app.Np, app.output_particles) == (3, 2, 4 * 16 * 16 * 8, 1)
    assert app.dt == 1.0 / 0.05
    assert app.pdist == 0
    s = E.solver_app_from_options("--input dens.bin --flux-scale 100.0 --y-flux-scale 3")
    assert s.input == b"dens.bin" and list(s.flux_scale) == [100.0, 3.0, 100.0]


def test_petsc_binary_vec(built, tmp_path):
    h = _lib.host()
    v = np.random.RandomState(0).standard_normal(37)
    f = tmp_path / "position.bin"
    assert h.ecs_write_petsc_vec(str(f).encode(), v.ctypes.data, v.size) == 0
    raw = f.read_bytes()
    cid, n = struct.unpack(">ii", raw[:8])
    assert cid == 1211214 and n == 37
    np.testing.assert_array_equal(np.frombuffer(raw[8:], dtype=">f8"), v)
    w = np.zeros(37)
    assert h.ecs_read_petsc_vec(str(f).encode(), w.ctypes.data, 37) == 0
    np.testing.assert_array_equal(w, v)


def test_echo_options_matches_reference(built, golden, tmp_path):
    from oracle import ref as refmod

    if not refmod.LIB_PATH.exists():
        pytest.skip("reference shim library not built here")
    g = golden["c1"]
    o = E.Options(g["opts"])
    p = E.params_from_options(o)
    ours = tmp_path / "ours.log"
    assert _lib.host().ecs_echo_options(str(ours).encode(), o._h, ctypes.byref(p)) == 0
    import subprocess
    import sys

    theirs = tmp_path / "ref.log"
    code = ("import sys; sys.path.insert(0, %r); from oracle import ref; "
            "r = ref.Ref(%r, 8); r.echo_options(%r)") % (str(ROOT), g["opts"], str(theirs))
    subprocess.run([sys.executable, "-c", code], check=True)
    assert ours.read_text() == theirs.read_text()


def _declared(header):
    text = (ROOT / "include" / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ecs_[a-z0-9_]+)\s*\(", text)))


def test_gpu_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(str(_lib.GPU_LIB_PATH))
    names = _declared("ecsgpu.h") + _declared("ecs_serve.h")
    assert len(names) >= 35
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    bound = {n for n, _, _ in _lib.GPU_API}
    assert set(names) <= bound, set(names) - bound


def test_gpu_library_exports_operator_slots(built):
    text = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "ecs_compat.h").read_text(), flags=re.S)
    names = sorted(set(re.findall(r"\b(EcsGpu[A-Za-z0-9]+)\s*\(", text)))
    assert len(names) >= 20
    lib = ctypes.CDLL(str(_lib.GPU_LIB_PATH))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_host_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(str(_lib.HOST_LIB_PATH))
    names = _declared("ecs_host.h")
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings(built):
    lib = _lib.gpu()
    assert lib.ecs_status_string(0) == b"ok"
    assert lib.ecs_status_string(-3) == b"solve did not converge"
    assert lib.ecs_version().startswith(b"ecsprt-gb300")


def test_device_bytes_estimate(built):
    p = E.params_from_options("-Nx 128 -Ny 128 -Nz 128 -dx 1 -dy 1 -dz 1")
    b_mixed = _lib.gpu().ecs_ctx_device_bytes(ctypes.byref(p), 1, 134217728)
    b_fp64 = _lib.gpu().ecs_ctx_device_bytes(ctypes.byref(p), 0, 134217728)
    assert 7e9 < b_mixed < 12e9
    assert 6e9 < b_fp64 < 12e9


@pytest.mark.parametrize("viT,vi0", [(1.0, 0.0), (1.0, 1.0), (1.0, 0.5), (0.3, 0.0), (2.0, 7.0), (1e-4, 0.0)])
def test_fixed_point_shifts(built, viT, vi0):
    """Deposit quanta: density 2^-48 (FP64) or 2^-38 (mixed); flux
    2^-(S - e_v) with 2^e_v the velocity bound 16 (viT + vi0) rounded up to a
    power of two (e_v clamped to [-8, 40]); a host-only helper of the ABI."""
    import math
    p = E.params_from_options(f"-Nx 8 -Ny 8 -Nz 8 -dx 1 -dy 1 -dz 1 -viT {viT} -vi0x {vi0}")
    ev = min(max(math.ceil(math.log2(16.0 * (p.viT + p.vi0))), -8), 40)
    for prec, S, Sf in ((E.ECS_PREC_FP64, 48, 48), (E.ECS_PREC_MIXED, 38, 22)):
        sn, sf = ctypes.c_int32(), ctypes.c_int32()
        assert _lib.gpu().ecs_fix_shifts(ctypes.byref(p), prec, ctypes.byref(sn), ctypes.byref(sf)) == 0
        assert (sn.value, sf.value) == (S, Sf - ev)
    assert _lib.gpu().ecs_fix_shifts(None, 0, ctypes.byref(sn), ctypes.byref(sf)) == _lib.ECS_ERR_INVALID


@pytest.mark.parametrize("opts,expect", [
    ("", ("EcsGpuApply3DBC", "EcsGpuCollect3D", "EcsGpuPushBz3D", "EcsGpuFullLHS3D", "EcsGpuFullRHS3D")),
    ("-ndim 2 -mn 0", ("EcsGpuApply2DBC", "EcsGpuCollect2D", "EcsGpuPushBz2D", "EcsGpuFullLHS2D", "EcsGpuFullRHS2D")),
    ("-lhs laplacian -rhs sinusoidal", ("EcsGpuApply3DBC", "EcsGpuCollect3D", "EcsGpuPushBz3D",
                                        "EcsGpuLaplacianLHS3D", "EcsGpuSinusoidalRHS3D")),
    ("-ndim 2 -lhs identity -rhs constant", ("EcsGpuApply2DBC", "EcsGpuCollect2D", "EcsGpuPushBz2D",
                                             "EcsGpuIdentityLHS", "EcsGpuConstantRHS")),
])
def test_operator_binding_follows_setup(built, opts, expect):
    """EcsGpuBindOperatorsFor fills the slots by SetUpContext's rules
    (src/setup.c:23-105)."""
    lib = ctypes.CDLL(str(_lib.GPU_LIB_PATH))

    class Ops(ctypes.Structure):
        _fields_ = [(n, ctypes.c_void_p) for n in ("applyBC", "collect", "push", "collide", "lhs", "rhs")]

    p = E.params_from_options(opts)
    ops = Ops()
    assert lib.EcsGpuBindOperatorsFor(ctypes.byref(ops), ctypes.byref(p)) == 0
    addr = lambda n: ctypes.cast(getattr(lib, n), ctypes.c_void_p).value
    got = (ops.applyBC, ops.collect, ops.push, ops.lhs, ops.rhs)
    assert got == tuple(addr(n) for n in expect)
    assert ops.collide == addr("EcsGpuScatterElastic")
