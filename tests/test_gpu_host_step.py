"""ecs_step_host: the time step through host buffers (the reference's DMSwarm
arrays live on the host), against the device-resident ecs_step.

After its first call the host arrays hold the ions in the device's order,
and the next call pipelines the upload, the particle pass and the download
by ranges of tiles.  Without collisions every step is deterministic and
order-free (fixed-point deposit), so both paths must give the same moments
and potential bit for bit, and the same ions as a set, over steps with and
without a cell sort.  Ions reordered by the caller between calls are still
stepped correctly (only the tile staging loses its locality).
"""
import numpy as np
import pytest

import ecsprt_gb300 as E

pytestmark = pytest.mark.gpu


def setup(n=16, ppc=16, seed=3, mn=False):
    opts = (f"-Nx {n} -Ny {n} -Nz {n} -dx 1 -dy 1 -dz 1 -qi 1 -mi 1 -B0 0.1 -viT 1 -vi0x 0.7 "
            f"-nui 0.5 -nue 8.79e9 -Te 11604.5 -E0 0" + ("" if mn else " -mn 0"))
    p = E.params_from_options(opts)
    rng = np.random.default_rng(seed)
    N = ppc * n ** 3
    pos = rng.uniform(0, n, (N, 3))
    vel = rng.standard_normal((N, 3)) + [0.7, 0, 0]
    return p, pos, vel


def as_set(pos, vel):
    rows = np.hstack([pos, vel])
    return rows[np.lexsort(rows.T[::-1])]


def host_buffers(pos, vel, shape):
    hp = E.pinned_empty(pos.shape)
    hv = E.pinned_empty(vel.shape)
    hp[:] = pos
    hv[:] = vel
    hm = E.pinned_empty(shape + (4,))
    hphi = E.pinned_empty(shape)
    return hp, hv, hm, hphi


@pytest.mark.parametrize("sort_every", [2, 3])
def test_host_step_matches_device_step(built, sort_every):
    p, pos, vel = setup()
    steps = 6
    with E.Context(p, E.ECS_PREC_MIXED, np_capacity=pos.shape[0]) as ctx:
        ctx.set_sort_every(sort_every)
        ctx.upload_particles(pos, vel)
        ctx.collect()
        ctx.compute_potential(rtol=1e-8, max_it=400)
        phi0 = ctx.phi
        ref = []
        for _ in range(steps):
            st = ctx.step(0.1, 1e-8, 400)
            gp, gv = ctx.download_particles()
            ref.append((ctx.moments, ctx.phi, as_set(gp, gv), st.sorted))
    with E.Context(p, E.ECS_PREC_MIXED, np_capacity=pos.shape[0]) as ctx:
        ctx.set_sort_every(sort_every)
        ctx.upload_particles(pos, vel)
        ctx.collect()
        ctx.compute_potential(rtol=1e-8, max_it=400)
        assert np.array_equal(ctx.phi, phi0)
        hp, hv, hm, hphi = host_buffers(*ctx.download_particles(), ctx.shape)
        nsorted = 0
        for s in range(steps):
            st = ctx.step_host(hp, hv, 0.1, 1e-8, 400, hm, hphi)
            m, phi, ions, sorted_ = ref[s]
            nsorted += st.sorted
            assert st.sorted == sorted_
            assert np.array_equal(hm, m), s
            assert np.array_equal(hphi, phi), s
            assert np.array_equal(as_set(hp, hv), ions), s
    assert nsorted >= 2


@pytest.mark.parametrize("shift", [(1, 0), (0, 5), (3, 30)])
def test_host_step_unaligned_host_arrays(built, shift):
    """The host copies run on 256-byte host boundaries, read a little past
    each chunk and write the few ions before a boundary with the next chunk:
    with the position and velocity arrays at different offsets from those
    boundaries (views `shift` doubles into pinned buffers), the ions, moments
    and potential still equal the device-resident step's, over steps with and
    without a sort, and no double outside the arrays changes."""
    p, pos, vel = setup(n=24, ppc=20, seed=11)
    N = pos.shape[0]
    steps = 5
    with E.Context(p, E.ECS_PREC_MIXED, np_capacity=N) as ctx:
        ctx.set_sort_every(2)
        ctx.upload_particles(pos, vel)
        ctx.collect()
        ctx.compute_potential(rtol=1e-8, max_it=400)
        ref = []
        for _ in range(steps):
            ctx.step(0.1, 1e-8, 400)
            ref.append((ctx.moments, ctx.phi, as_set(*ctx.download_particles())))
    with E.Context(p, E.ECS_PREC_MIXED, np_capacity=N) as ctx:
        ctx.set_sort_every(2)
        ctx.upload_particles(pos, vel)
        ctx.collect()
        ctx.compute_potential(rtol=1e-8, max_it=400)
        gp, gv = ctx.download_particles()
        sp, sv = shift
        bp = E.pinned_empty((3 * N + sp + 40,))
        bv = E.pinned_empty((3 * N + sv + 40,))
        bp[:] = -7.0
        bv[:] = -7.0
        hp = bp[sp:sp + 3 * N].reshape(N, 3)
        hv = bv[sv:sv + 3 * N].reshape(N, 3)
        hp[:] = gp
        hv[:] = gv
        hm = E.pinned_empty(ctx.shape + (4,))
        hphi = E.pinned_empty(ctx.shape)
        for s in range(steps):
            ctx.step_host(hp, hv, 0.1, 1e-8, 400, hm, hphi)
            m, phi, ions = ref[s]
            assert np.array_equal(hm, m), s
            assert np.array_equal(hphi, phi), s
            assert np.array_equal(as_set(hp, hv), ions), s
        assert (bp[:sp] == -7.0).all() and (bp[sp + 3 * N:] == -7.0).all()
        assert (bv[:sv] == -7.0).all() and (bv[sv + 3 * N:] == -7.0).all()


def test_host_step_reordered_between_calls(built):
    p, pos, vel = setup(seed=5)
    with E.Context(p, E.ECS_PREC_MIXED, np_capacity=pos.shape[0]) as ctx:
        ctx.upload_particles(pos, vel)
        ctx.collect()
        ctx.compute_potential(rtol=1e-8, max_it=400)
        for _ in range(3):
            ctx.step(0.1, 1e-8, 400)
        m_ref, ions_ref = ctx.moments, as_set(*ctx.download_particles())
    with E.Context(p, E.ECS_PREC_MIXED, np_capacity=pos.shape[0]) as ctx:
        ctx.upload_particles(pos, vel)
        ctx.collect()
        ctx.compute_potential(rtol=1e-8, max_it=400)
        hp, hv, hm, hphi = host_buffers(*ctx.download_particles(), ctx.shape)
        rng = np.random.default_rng(9)
        for s in range(3):
            if s == 1:  # the caller shuffles its arrays: the hand-off order no longer holds
                perm = rng.permutation(hp.shape[0])
                hp[:] = hp[perm]
                hv[:] = hv[perm]
            ctx.step_host(hp, hv, 0.1, 1e-8, 400, hm, hphi)
        assert np.array_equal(hm, m_ref)
        assert np.array_equal(as_set(hp, hv), ions_ref)


def test_host_step_with_collisions(built):
    """With collisions the host path draws each ion's numbers from its
    position in the host arrays (its identity there), so it is compared as a
    physical system: the ion count, the density sum and the collision count
    per step against the device-resident path's."""
    p, pos, vel = setup(mn=True, seed=7)
    N = pos.shape[0]
    counts = {}
    for path in ("device", "host"):
        with E.Context(p, E.ECS_PREC_MIXED, np_capacity=N) as ctx:
            ctx.upload_particles(pos, vel)
            ctx.collect()
            ctx.compute_potential(rtol=1e-8, max_it=400)
            hp, hv, hm, hphi = host_buffers(pos, vel, ctx.shape)
            c = []
            for _ in range(4):
                st = ctx.step(0.1, 1e-8, 400) if path == "device" else ctx.step_host(hp, hv, 0.1, 1e-8, 400, hm,
                                                                                         hphi)
                assert st.solve.relres <= 1e-8
                c.append(st.collisions)
            m = ctx.moments if path == "device" else hm
            assert m[..., 0].sum() == pytest.approx(N, rel=1e-9)
            counts[path] = np.array(c)
    Nc = counts["device"].mean()
    assert Nc > 1000
    assert abs(counts["host"].mean() - Nc) <= 5 * np.sqrt(Nc)
