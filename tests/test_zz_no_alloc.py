"""ecs_rhs_noalloc: the RHS entry point that makes no allocation.

It serves callers that own all of their device memory (a host framework
with its own pre-reserved pool, or a step loop that must not trigger the
device synchronisation an allocation can cause).  The caller passes device
input and output buffers; the entry point's reduction scratch is a fixed
__device__ array.  This test allocates the caller's buffers itself (as such a
caller would, from its own pool), calls the entry point through the C ABI
on several grids in a row (3-D and 2-D, the full RHS and the -rhs
sinusoidal and -rhs constant options), and checks each result against the
context entry point ecs_rhs and the reference's golden RHS with the RHS
tolerance used throughout the GPU tests (1e-14 relative).  It lives in a
file collected last so that a run stopping at the first failure has already
run every other test.
"""
import ctypes
import json

import numpy as np
import pytest

import ecsprt_gb300 as E
from conftest import GOLDEN, load_golden
from ecsprt_gb300 import _lib

pytestmark = pytest.mark.gpu

H2D, D2H = 1, 2


def _cudart():
    for name in ("libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so.13", "libcudart.so"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    pytest.skip("CUDA runtime not found")


def _rel_inf(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _rhs_with_context(p, moments):
    with E.Context(p, E.ECS_PREC_FP64, np_capacity=1) as ctx:
        ctx.moments = moments
        ctx.compute_rhs()
        return ctx.rhs


def _rhs_noalloc(rt, p, moments):
    m = np.ascontiguousarray(moments, dtype=np.float64)
    out = np.empty(m.shape[:3])
    dm, db = ctypes.c_void_p(), ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(dm), ctypes.c_size_t(m.nbytes)) == 0
    assert rt.cudaMalloc(ctypes.byref(db), ctypes.c_size_t(out.nbytes)) == 0
    try:
        assert rt.cudaMemcpy(dm, m.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(m.nbytes), H2D) == 0
        rc = _lib.gpu().ecs_rhs_noalloc(ctypes.byref(p), dm, db, None)
        assert rc == 0, _lib.gpu().ecs_last_error(None)
        assert rt.cudaDeviceSynchronize() == 0
        assert rt.cudaMemcpy(out.ctypes.data_as(ctypes.c_void_p), db, ctypes.c_size_t(out.nbytes), D2H) == 0
    finally:
        rt.cudaFree(dm)
        rt.cudaFree(db)
    return out


def _cases():
    """(name, params, moments, golden RHS) for the full RHS in 3-D (two
    grids) and 2-D, and the -rhs sinusoidal and -rhs constant options."""
    out = []
    for name in ("fb", "c1", "twod"):
        g = load_golden(name)
        out.append((name, E.params_from_options(g["opts"]), g["moments"], g["rhs"]))
    ops = np.load(GOLDEN / "ops.npz")
    variants = json.loads(str(ops["variants"]))
    for v in ("full_sin", "id_const"):
        p = E.params_from_options(str(ops["opts_base"]) + variants[v])
        dens = ops["full_sin_density"] if v == "full_sin" else np.zeros((p.Nz, p.Ny, p.Nx))
        m = np.zeros(dens.shape + (4,))
        m[..., 0] = dens
        out.append((v, p, m, ops[f"{v}_rhs"]))
    return out


def test_rhs_noalloc_matches_context_entry_point(built):
    rt = _cudart()
    cases = _cases()
    for name, p, moments, golden_rhs in cases + cases[:1]:  # consecutive calls share the scratch array
        expect = _rhs_with_context(p, moments)
        got = _rhs_noalloc(rt, p, moments)
        assert np.isfinite(got).all(), name
        assert _rel_inf(got, expect) <= 1e-14, name
        assert _rel_inf(got, golden_rhs) <= 1e-14, name


def test_rhs_noalloc_rejects_grids_beyond_its_scratch(built):
    p = E.params_from_options("-Nx 512 -Ny 512 -Nz 64 -dx 1 -dy 1 -dz 1")
    lib = _lib.gpu()
    rc = lib.ecs_rhs_noalloc(ctypes.byref(p), ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert rc == E._lib.ECS_ERR_INVALID
    assert b"exceed" in lib.ecs_last_error(None)
