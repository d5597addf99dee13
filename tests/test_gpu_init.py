"""Initial ions generated on the device (ecs_particles_init), and the
256 x 256 x 128 reflecting-z workload run at full size from them.

Tolerances:
  Sobol positions     bit-exact against the oracle (itself pinned to the
                      reference's Sobol golden vectors)
  velocities, random  statistical: mean within 5 sigma/sqrt(N) of the drift,
  and rejection       standard deviation within 5 sigma/sqrt(2N) of vT,
  positions           Kolmogorov-Smirnov p > 1e-4 against the target law (and,
                      for velocities, against the reference's gasdev stream);
                      Fourier coefficients of the sampled density within
                      5 standard errors of a/2
  full-size run       ion count conserved, every ion inside the domain
                      (device range flags), relres <= 1e-8; the density sums
                      to the ion count less the weight that ions of the top
                      cell layer put on the node layer above z = Lz, which a
                      reflecting (ghosted) z drops: between 0 and 1.2/Nz of
                      the ion count (about 1/(2 Nz) for a near-uniform
                      density)
"""
import math

import numpy as np
import pytest

import ecsprt_gb300 as E
from ecsprt_gb300 import workloads as W
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

stats = pytest.importorskip("scipy.stats")


def params(n=32, extra=""):
    return E.params_from_options(f"-Nx {n} -Ny {n} -Nz {n} -dx 1 -dy 1 -dz 1 -qi 1 -mi 1 -B0 0.1 -viT 1 "
                                 f"-vi0x 0.7 -vi0y -0.2 -nui 0.02 -nue 8.79e9 -Te 11604.5 -E0 0 {extra}")


@pytest.mark.parametrize("prec", [E.ECS_PREC_FP64, E.ECS_PREC_MIXED])
def test_sobol_positions_bit_exact(built, prec):
    p = params(32)
    N = 200_000
    pos_o = orc.Oracle(p).sobol(N)
    with E.Context(p, prec, np_capacity=N) as ctx:
        ctx.set_sort_every(0)
        ctx.init_particles(E.ECS_INIT_SOBOL, N)
        pos, _ = ctx.download_particles()
        if prec == E.ECS_PREC_MIXED:  # the same FP64 positions through an upload
            ctx.upload_particles(pos_o, np.zeros_like(pos_o))
            pos_u, _ = ctx.download_particles()
    if prec == E.ECS_PREC_FP64:
        assert np.array_equal(pos, pos_o)
    else:
        assert np.array_equal(pos, pos_u)


def test_velocities_maxwellian(built):
    p = params(16)
    N = 1_000_000
    with E.Context(p, E.ECS_PREC_FP64, np_capacity=N) as ctx:
        ctx.init_particles(E.ECS_INIT_RANDOM, N, seed=5)
        pos, vel = ctx.download_particles()
    vT = np.array([p.viTx, p.viTy, p.viTz])
    v0 = np.array([p.vi0x, p.vi0y, p.vi0z])
    assert np.all(np.abs(vel.mean(0) - v0) < 5 * vT / math.sqrt(N))
    assert np.all(np.abs(vel.std(0) - vT) < 5 * vT / math.sqrt(2 * N))
    for d in range(3):
        assert stats.kstest((vel[:, d] - v0[d]) / vT[d], "norm").pvalue > 1e-4
    ref = orc.normal_velocities(vT, v0, 200_000)  # the reference's gasdev stream
    for d in range(3):
        assert stats.ks_2samp(vel[:200_000, d], ref[:, d]).pvalue > 1e-4
    L = np.array([p.Lx, p.Ly, p.Lz])
    assert np.all(pos >= 0) and np.all(pos < L)
    for d in range(3):
        assert stats.kstest(pos[:, d] / L[d], "uniform").pvalue > 1e-4


def test_sinusoidal_rejection(built):
    """Density 1 + 0.25 sin(2 pi x/Lx) (src/positions.c:236-251): the x
    fractions follow F(s) = s + 0.25 (1 - cos 2 pi s) / (2 pi)."""
    p = params(32)
    N = 1_000_000
    with E.Context(p, E.ECS_PREC_FP64, np_capacity=N) as ctx:
        ctx.init_particles(E.ECS_INIT_SINUSOIDAL, N, seed=6)
        pos, _ = ctx.download_particles()
    s = pos[:, 0] / p.Lx
    cdf = lambda x: x + 0.25 * (1.0 - np.cos(2 * np.pi * x)) / (2 * np.pi)
    assert stats.kstest(s, cdf).pvalue > 1e-4
    assert stats.kstest(pos[:, 1] / p.Ly, "uniform").pvalue > 1e-4


def test_mode_density_and_determinism(built):
    p = params(32)
    N = 2_000_000
    modes = [(1, 0, 0, 0.2, 0.3), (0, 2, -1, 0.15, -1.0)]
    with E.Context(p, E.ECS_PREC_FP64, np_capacity=N) as ctx:
        ctx.init_particles(E.ECS_INIT_MODES, N, seed=7, modes=modes)
        pos, vel = ctx.download_particles()
        ctx.init_particles(E.ECS_INIT_MODES, N, seed=7, modes=modes)
        pos2, vel2 = ctx.download_particles()
        ctx.init_particles(E.ECS_INIT_MODES, N, seed=8, modes=modes)
        pos3, _ = ctx.download_particles()
    assert np.array_equal(pos, pos2) and np.array_equal(vel, vel2)
    assert not np.array_equal(pos, pos3)
    s = pos / np.array([p.Lx, p.Ly, p.Lz])
    for kx, ky, kz, a, ph in modes:
        th = 2 * np.pi * (kx * s[:, 0] + ky * s[:, 1] + kz * s[:, 2]) + ph
        # E_w[cos th] = a/2 and E_w[sin th] = 0 for w = 1 + a cos th (+ orthogonal modes)
        se = math.sqrt(0.5 / N)
        assert abs(np.cos(th).mean() - a / 2) < 5 * se
        assert abs(np.sin(th).mean()) < 5 * se


def test_init_errors(built):
    p = params(16)
    with E.Context(p, E.ECS_PREC_MIXED, np_capacity=1000) as ctx:
        with pytest.raises(E.EcsError) as ei:
            ctx.init_particles(E.ECS_INIT_MODES, 1000, modes=[(1, 0, 0, 0.6, 0), (0, 1, 0, 0.5, 0)])
        assert ei.value.code == E._lib.ECS_ERR_INVALID
        with pytest.raises(E.EcsError) as ei:
            ctx.init_particles(3, 1000)  # the reference's "uniform" lattice: not on the device
        assert ei.value.code == E._lib.ECS_ERR_UNSUPPORTED
        with pytest.raises(E.EcsError) as ei:
            ctx.init_particles(E.ECS_INIT_SOBOL, 1001)
        assert ei.value.code == E._lib.ECS_ERR_INVALID


def test_full_size_256x256x128_reflecting_z(built):
    """The 256 x 256 x 128 workload (periodic x/y, reflecting z, 32 ions per
    cell = 268,435,456 ions, density 1 + 8 Fourier modes of amplitude 0.02,
    mixed precision, cell sort every 4 steps) at full size: a few steps
    keep every ion, lose only the density a reflecting z drops, and each
    solve reaches 1e-8."""
    p = E.params_from_options("-Nx 256 -Ny 256 -Nz 128 -dx 1 -dy 1 -dz 1 -qi 1 -mi 1 -B0 0.1 -viT 1 -vi0x 0.5 "
                              "-nui 0.02 -nue 8.79e9 -Te 11604.5 -E0 0 -zBC inject-reflect")
    N = 256 * 256 * 128 * 32
    with E.Context(p, E.ECS_PREC_MIXED, np_capacity=N) as ctx:
        ctx.set_sort_every(4)
        ctx.init_particles(E.ECS_INIT_MODES, N, seed=W.C3_SEED, modes=W.c3_modes())
        ctx.collect()
        st0 = ctx.compute_potential(rtol=1e-8, max_it=400)
        assert st0.relres <= 1e-8
        import time
        for q in range(4):
            t0 = time.perf_counter()
            st = ctx.step(0.1, 1e-8, 400)
            t1 = time.perf_counter()
            assert st.solve.relres <= 1e-8
            print(f"step {q}: {1e3 * (t1 - t0):.2f} ms wall, particles {1e3 * st.particle_seconds:.2f} ms, "
                  f"sort {1e3 * st.sort_seconds:.2f} ms, solve {1e3 * st.solve.seconds:.2f} ms "
                  f"({st.solve.iterations} its), {N / (t1 - t0):.3e} particle-steps/s")
        assert ctx.launches > 0
        m = ctx.moments
        assert int(E._lib.gpu().ecs_particles_count(ctx.handle)) == N
    dropped = N - m[..., 0].sum()
    assert 0 < dropped < 1.2 * N / 128, dropped / N
    assert abs(dropped / N - 1 / 256) < 0.1 / 256
    assert m[..., 0].min() > 0
