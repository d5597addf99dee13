"""Parity over the reference's full time loop (src/pic.c:238-258): many steps
of push, move, deposit, RHS and solve against the FP64 oracle, at the
benchmarked configurations.

test_fp64_c1_hundred_steps
    The plain FP64 path on the 32^3, 16 ions/cell workload (524,288 ions;
    the reference's own Sobol positions and NormalVelocities; drift 0.5,
    gyrofrequency 0.1, collisions off so that both sides are deterministic)
    for 100 steps of dt = 0.1.  Tolerance, stated before measuring: positions
    and velocities after 100 steps <= 1e-10 relative (max |dv| / max |v|;
    periodic distance / L), density <= 1e-12 relative, potential relative
    L2 <= 1e-8.  The oracle solves to a true FP64 relative residual of 1e-13
    (FFT-preconditioned GMRES on the oracle operator) and the GPU to 1e-13.

test_mixed_bench_path_hundred_steps
    The mixed path exactly as the benchmark runs it (FP32 ions counting-
    sorted every 2 steps, so the tile kernel does the work; FP32 multigrid
    inside FP64 refinement to 1e-8) on a 32^3 grid with the benchmark's
    physics: 64 ions/cell, density 1 + 0.05 sin(2 pi x / Lx), drift 1.0,
    kappa_e ~ 2, collisions off.  100 steps side by side with the oracle;
    ions are matched through their identities (ecs_particles_ids).

    The reference's gathered field is discontinuous across cell faces: it
    interpolates along z with the x weight and along x with the z weight
    (quirk Q3, src/vector-math.c:645-651), so at an x or z face the two
    cells give different fields, and at the periodic seams the last cell
    uses the backward difference stored at node N (quirk Q2,
    src/vector-math.c:632-644).  An ion that starts a step with its FP32
    position in another cell than the oracle's FP64 one (an ion within the
    rounding error of a face) receives a kick that differs by the field
    jump, not by the rounding, and its trajectory departs from the oracle's
    by that much.  The test downloads the ions after every step, marks every
    ion that ever started a step in a cell other than the oracle's ("face
    ions"), and checks the others against the
    rounding model.  Tolerances:
      relative residual of every solve       <= 1e-8 (FP64-measured)
      deposit of the GPU's own ions           <= 1e-6 relative (L-infinity /
                                                 max) against the oracle's
                                                 FP64 deposit of those ions
      solve of the GPU's own moments          <= 1e-5 relative L2 against the
                                                 oracle's FP64 solve of them
                                                 (1e-8 relative residual times
                                                 the operator's conditioning)
      face ions                               <= 0.5 % of the ions
      velocity after N steps (other ions)     <= 2e-6 N max|v|: the single-
                                                 step push tolerance,
                                                 accumulated
      position after N steps (other ions)     <= 2e-6 N + 1e-6 N^2 max|v| dt
                                                 cells: the single-step move
                                                 tolerance plus the velocity
                                                 error carried
      density after N steps, per node        <= the change that the ions'
                                                 measured position differences
                                                 can make (each weight moves
                                                 by at most |dx|+|dy|+|dz|)
                                                 plus the deposit tolerance
    The velocity and position errors of all ions and the potential's
    difference from the oracle's trajectory are printed against N.

test_tile_window_chunks
    Above 125 ions a cell a 4x4x2-cell tile holds more than the 4000 ions
    its shared-memory window takes between flushes, so the tile kernel
    works through the tile in several chunks.  At 200 ions/cell (two chunks
    a tile) the tile kernel's deposit and full steps with collisions equal
    the order-free kernel's bit for bit.
"""
import numpy as np
import pytest

import ecsprt_gb300 as E
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

PHYS = "-qi 1 -mi 1 -B0 0.1 -viT 1 -nue 8.79e9 -Te 11604.5 -E0 0"


def rel_inf(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


def periodic_dist(a, b, L):
    d = np.abs(a - b)
    return np.minimum(d, L - d)


def bit_equal(a, b):
    a, b = np.asarray(a), np.asarray(b)
    bad = np.flatnonzero(a.ravel() != b.ravel())
    assert bad.size == 0, f"{bad.size}/{a.size} differ"


def oracle_step(O, pos, vel, phi, dt, rtol=1e-13):
    vel = O.push(pos, vel, phi, dt)
    pos, vel = O.move(pos, vel, dt)
    m = O.collect(pos, vel)
    b = O.rhs(m)
    phi, _, rel = O.solve_fft(m[..., 0], b, rtol=rtol)
    assert rel <= rtol
    return pos, vel, m, phi


def test_fp64_c1_hundred_steps(built):
    n, ppc, steps, dt = 32, 16, 100, 0.1
    opts = f"-Nx {n} -Ny {n} -Nz {n} -dx 1 -dy 1 -dz 1 {PHYS} -vi0x 0.5 -mn 0"
    p = E.params_from_options(opts)
    O = orc.Oracle(p)
    npart = ppc * n ** 3
    pos = O.sobol(npart)  # the reference's SobolDistribution (src/positions.c:139-233)
    vel = orc.normal_velocities([p.viTx, p.viTy, p.viTz], [p.vi0x, p.vi0y, p.vi0z], npart)
    op, ov = pos.copy(), vel.copy()
    m0 = O.collect(op, ov)
    ophi, _, _ = O.solve_fft(m0[..., 0], O.rhs(m0), rtol=1e-13)
    L = n * 1.0
    rows = []
    with E.Context(p, E.ECS_PREC_FP64, np_capacity=npart) as ctx:
        ctx.upload_particles(pos, vel)
        ctx.phi = ophi
        for step in range(1, steps + 1):
            st = ctx.step(dt, rtol=1e-13, max_it=400)
            assert st.solve.relres <= 1e-13
            op, ov, om, ophi = oracle_step(O, op, ov, ophi, dt)
            if step in (1, 10, 25, 50, 75, 100):
                gp, gv = ctx.download_particles()
                gm, gphi = ctx.moments, ctx.phi
                rows.append((step, rel_inf(gv, ov), periodic_dist(gp, op, L).max() / L,
                             rel_inf(gm[..., 0], om[..., 0]), rel_inf(gm, om),
                             np.linalg.norm(gphi - ophi) / np.linalg.norm(ophi)))
    print("\n  N   velocity   position   density    moments    potential")
    for r in rows:
        print("%3d  %.2e   %.2e   %.2e   %.2e   %.2e" % r)
    for step, ev, ex, en, em, ephi in rows:
        assert ev <= 1e-10, (step, ev)
        assert ex <= 1e-10, (step, ex)
        assert en <= 1e-12, (step, en)
        assert em <= 1e-10, (step, em)
        assert ephi <= 1e-8, (step, ephi)


def sinusoidal_ions(n, ppc, drift, seed):
    """Rejection-sampled density 1 + 0.05 sin(2 pi x / Lx) on an n^3 box,
    Maxwellian velocities (sigma 1) with a drift along x."""
    rng = np.random.default_rng(seed)
    npart = ppc * n ** 3
    xs = np.empty(0)
    while xs.size < npart:
        x = rng.uniform(0, n, 2 * npart)
        keep = rng.uniform(0, 1.05, x.size) < 1.0 + 0.05 * np.sin(2 * np.pi * x / n)
        xs = np.concatenate([xs, x[keep]])
    pos = np.empty((npart, 3))
    pos[:, 0] = xs[:npart]
    pos[:, 1:] = rng.uniform(0, n, (npart, 2))
    vel = rng.standard_normal((npart, 3))
    vel[:, 0] += drift
    return pos, vel


def node_error_bound(pos, dpos, n):
    """Per node, |dx| + |dy| + |dz| of dpos (cells) summed over the ions at
    `pos` in the eight cells that touch the node (periodic n^3 grid): the
    most that an ion's CIC weight on that node moves when it moves by dpos."""
    c = np.floor(pos).astype(np.int64) % n
    cell = (c[:, 2] * n + c[:, 1]) * n + c[:, 0]
    h = np.bincount(cell, weights=np.abs(dpos).sum(axis=1), minlength=n ** 3).reshape(n, n, n)
    return sum(np.roll(h, (dz, dy, dx), axis=(0, 1, 2)) for dz in (0, 1) for dy in (0, 1) for dx in (0, 1))


MIXED_REPORT = (1, 2, 5, 10, 20, 50, 100)


def test_mixed_bench_path_hundred_steps(built):
    n, ppc, steps, dt, drift = 32, 64, 100, 0.1, 1.0
    opts = f"-Nx {n} -Ny {n} -Nz {n} -dx 1 -dy 1 -dz 1 {PHYS} -vi0x {drift} -mn 0"
    p = E.params_from_options(opts)
    O = orc.Oracle(p)
    pos, vel = sinusoidal_ions(n, ppc, drift, seed=20261205)
    op, ov = pos.copy(), vel.copy()
    m0 = O.collect(op, ov)
    ophi, _, _ = O.solve_fft(m0[..., 0], O.rhs(m0), rtol=1e-13)
    L = float(n)
    face = np.zeros(pos.shape[0], dtype=bool)
    rows = []
    sorted_steps = 0
    with E.Context(p, E.ECS_PREC_MIXED, np_capacity=pos.shape[0]) as ctx:
        ctx.set_sort_every(2)  # as the benchmark: the tile kernel runs every step
        ctx.upload_particles(pos, vel)
        gp, gv = ctx.download_particles_in_upload_order()
        assert periodic_dist(gp, pos, L).max() <= 1e-6  # identities survive the upload's sort
        ctx.phi = ophi
        for step in range(1, steps + 1):
            face |= (np.floor(gp) != np.floor(op)).any(axis=1)  # cells at the start of this step
            st = ctx.step(dt, rtol=1e-8, max_it=400)
            assert st.solve.relres <= 1e-8, (step, st.solve.relres)
            sorted_steps += st.sorted
            op, ov, om, ophi = oracle_step(O, op, ov, ophi, dt)
            gp, gv = ctx.download_particles_in_upload_order()
            if step in MIXED_REPORT:
                gm, gphi = ctx.moments, ctx.phi
                own = O.collect(gp, gv)  # the oracle's FP64 deposit of the GPU's own ions
                # the oracle's FP64 solve of the GPU's own moments
                phi_own, _, _ = O.solve_fft(gm[..., 0], O.rhs(gm), rtol=1e-13)
                dpos = np.where(np.abs(gp - op) > L / 2, L - np.abs(gp - op), np.abs(gp - op))
                vmax = np.abs(ov).max()
                dv = np.abs(gv - ov).max(axis=1) / vmax
                dx = dpos.max(axis=1)
                bulk = ~face
                # the ion's weights sit on the nodes of its oracle cell and of its GPU cell
                dn_bound = (node_error_bound(op, dpos, n) + node_error_bound(gp, dpos, n) +
                            1e-6 * np.abs(om[..., 0]).max())
                rows.append(dict(
                    N=step, dep=rel_inf(gm[..., 0], own[..., 0]),
                    solve=np.linalg.norm(gphi - phi_own) / np.linalg.norm(phi_own),
                    face=int(face.sum()), vel=dv[bulk].max(), pos=dx[bulk].max(),
                    vel_all=dv.max(), pos_all=dx.max(), vmax=vmax,
                    dens=rel_inf(gm[..., 0], om[..., 0]),
                    dens_ok=bool((np.abs(gm[..., 0] - om[..., 0]) <= dn_bound).all()),
                    phi=np.linalg.norm(gphi - ophi) / np.linalg.norm(ophi)))
    assert sorted_steps == steps // 2
    print("\n  N   deposit  solve    | face ions  velocity  position | all ions: velocity position"
          " | density  potential")
    for r in rows:
        print("%3d  %.1e  %.1e  | %8d   %.2e  %.2e |           %.2e %.2e | %.2e %.2e" % (
            r["N"], r["dep"], r["solve"], r["face"], r["vel"], r["pos"], r["vel_all"], r["pos_all"],
            r["dens"], r["phi"]))
    for r in rows:
        N = r["N"]
        assert r["dep"] <= 1e-6, r
        assert r["solve"] <= 1e-5, r
        assert r["face"] <= 0.005 * pos.shape[0], r
        assert r["vel"] <= 2e-6 * N, r
        assert r["pos"] <= 2e-6 * N + 1e-6 * N * N * r["vmax"] * dt, r
        assert r["dens_ok"], r


def test_tile_window_chunks(built):
    n, ppc = 8, 200
    opts = f"-Nx {n} -Ny {n} -Nz {n} -dx 1 -dy 1 -dz 1 {PHYS} -vi0x 0.5 -nui 0.05"
    p = E.params_from_options(opts)
    rng = np.random.RandomState(5)
    npart = ppc * n ** 3
    assert npart // (n ** 3 // 32) > 4000  # ions a tile: more than one window's worth
    pos = rng.uniform(0, n, (npart, 3))
    vel = rng.standard_normal((npart, 3)) + [0.5, 0, 0]
    out = []
    for every in (1, 0):
        with E.Context(p, E.ECS_PREC_MIXED, np_capacity=npart) as ctx:
            ctx.set_sort_every(every)
            ctx.upload_particles(pos, vel)
            ctx.collect()
            m0 = ctx.moments
            ctx.compute_potential(rtol=1e-8, max_it=400)
            ncoll = 0
            for _ in range(3):
                ncoll += ctx.step(0.1, rtol=1e-8, max_it=400).collisions
            gp, gv = ctx.download_particles_in_upload_order()
            out.append((m0, ncoll, ctx.moments, gp, gv))
    assert out[0][1] == out[1][1] and out[0][1] > 0
    for a, b in zip(out[0], out[1]):
        bit_equal(a, b)
    assert out[0][0][..., 0].sum() == pytest.approx(npart, rel=1e-9)
