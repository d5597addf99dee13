"""Generate the golden vectors in tests/golden/ from the reference itself.

The reference publishes no golden data and its tests pin no numbers, so the
vectors are produced by the reference's own hot-path C sources, compiled
unmodified against the PETSc-API shim (oracle/_ref/libecsref.so, built by
oracle/ref_shim/Makefile).  Each case runs in a fresh process: the reference
keeps process-global RNG and Sobol state (src/random.c).

    python tests/golden/make_golden.py            # all cases
    python tests/golden/make_golden.py --case c1  # one case, prints nothing

Cases:
  c1   8^3 periodic grid, dx = 1, normalised C1 physics (qi = mi = 1,
       B0 = 0.1, viT = 1, vi0x = 0.5, kappa_e ~ 2), 4 ions/cell from the
       reference's Sobol + Maxwellian initialisation, nui = 2 (so that ~900
       collisions happen per call).
  edge 8x6x5 grid, dx = 0.5, dy = 1, dz = 2, hand-placed ions in the last
       cell (backward-difference branch), on cell faces, and crossing both
       periodic bounds during the move.
  fb   the reference's own test physics (tests/fb-physics.ini, SI units,
       kappa_e ~ 88) on tests/grid3D.ini spacing (dx = 0.5) at 16^3, one ion
       per cell, dt = 1e-5 as in tests/test_all.sh.
  rng  ran1 / ran3 / gasdev streams and Sobol points from a fresh process.
  twod -ndim 2 on an 8x6 grid (dx = 0.5, dy = 1), collisions off, 4 Sobol
       ions per cell plus hand-placed ions in the last cells (backward
       differences) and on the bounds: push, move, deposit, RHS and the
       9-point operator (dense), and the 5-point Laplacian with the
       sinusoidal RHS.
  ops  the other operator options on a 6x5x4 grid (dx = 0.1, dy = 0.125,
       dz = 0.2, n0 = 2.5): RHS and dense LHS of -lhs laplacian -rhs
       sinusoidal, of -lhs laplacian -rhs constant with a reflecting z, of
       -lhs identity -rhs constant, and of -lhs full -rhs sinusoidal.
"""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle import ref as refmod  # noqa: E402

C1_PHYS = ("-qi 1 -mi 1 -B0 0.1 -viT 1 -vi0x 0.5 -nue 8.79e9 -Te 11604.5 -E0 0 ")
FB_PHYS = ("-nue 5e4 -nui 3e3 -B0 2.5e-5 -E0 5e-2 -mi 5.0e-26 -mn 4.6e-26 -Te 300.0 -Ti 300.0 -Tn 300.0 ")


def smooth_phi(shape, seed, amp=1.0):
    """Seeded sum of Fourier modes on the node grid [Nz][Ny][Nx]."""
    rng = np.random.RandomState(seed)
    nz, ny, nx = shape
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    phi = np.zeros(shape)
    for _ in range(6):
        mx, my, mz = rng.randint(0, 3, size=3)
        ph = rng.uniform(0, 2 * np.pi)
        a = rng.uniform(0.2, 1.0)
        phi += a * np.cos(2 * np.pi * (mx * i / nx + my * j / ny + mz * k / nz) + ph)
    phi += 0.05 * rng.standard_normal(shape)
    return amp * phi


def lhs_rows(A, shape):
    """The 11 stencil coefficients of every row, in the reference's order."""
    nz, ny, nx = shape
    offs = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1),
            (1, 1, 0), (1, -1, 0), (-1, 1, 0), (-1, -1, 0), (0, 0, 0)]
    rows = np.zeros((nz * ny * nx, 11))
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                r = (k * ny + j) * nx + i
                for e, (di, dj, dk) in enumerate(offs):
                    c = (((k + dk) % nz) * ny + (j + dj) % ny) * nx + (i + di) % nx
                    rows[r, e] = A[r, c]
    return rows


def run_pipeline(R, pos, vel, phi, dt, ncollide):
    out = {"pos0": pos.copy(), "vel0": vel.copy(), "phi": phi.copy(), "dt": np.float64(dt)}
    R.set_particles(pos, vel)
    R.set_phi(phi)
    R.push(dt)
    _, vpush = R.get_particles()
    out["vel_push"] = vpush.copy()
    for c in range(ncollide):
        rc = R.collide(dt)
        _, vc = R.get_particles()
        out[f"vel_collide{c + 1}"] = vc.copy()
        out[f"collide_rc{c + 1}"] = np.int64(rc)
    R.set_particles(pos, vpush)
    R.update_positions(dt)
    pmove, vmove = R.get_particles()
    out["pos_move"] = pmove.copy()
    out["vel_move"] = vmove.copy()
    R.collect()
    m = R.get_moments()
    out["moments"] = m.copy()
    out["rhs"] = R.rhs()
    A = R.lhs_dense()
    out["lhs_rows"] = lhs_rows(A, R.shape)
    return out


def case_c1():
    opts = "-Nx 8 -Ny 8 -Nz 8 -dx 1 -dy 1 -dz 1 -nui 2.0 " + C1_PHYS
    Np = 4 * 512
    R = refmod.Ref(opts, Np)
    R.init_positions(0)
    R.init_velocities()
    pos, vel = R.get_particles()
    phi = smooth_phi(R.shape, 11, amp=2.0)
    out = run_pipeline(R, pos, vel, phi, 0.1, 2)
    out["opts"] = opts
    out["params"] = json.dumps(R.params)
    out["init_pos"] = pos
    out["init_vel"] = vel
    return out


def case_edge():
    opts = "-Nx 8 -Ny 6 -Nz 5 -dx 0.5 -dy 1.0 -dz 2.0 -mn 0 " + C1_PHYS
    R = refmod.Ref(opts, 16)
    Lx, Ly, Lz = 4.0, 6.0, 10.0
    pos = np.array([
        [3.99, 5.5, 9.9],      # last cell in every axis: backward differences
        [0.0, 0.0, 0.0],       # the origin
        [0.5, 1.0, 2.0],       # exactly on interior faces
        [3.75, 0.25, 1.0],
        [0.01, 3.3, 9.99],     # will cross x = 0 going left
        [3.999, 5.999, 0.001], # will cross the upper x and y bounds
        [2.0, 3.0, 5.0],
        [1.234, 4.567, 7.891],
    ] * 2)
    rng = np.random.RandomState(5)
    vel = rng.normal(0, 1.0, pos.shape)
    vel[4] = [-0.5, 0.1, 0.3]
    vel[5] = [0.5, 0.4, -0.3]
    pos[8:] = rng.uniform(0, 1, (8, 3)) * [Lx, Ly, Lz]
    phi = smooth_phi(R.shape, 12, amp=3.0)
    out = run_pipeline(R, pos, vel, phi, 0.1, 0)
    out["opts"] = opts
    out["params"] = json.dumps(R.params)
    return out


def case_fb():
    opts = "-Nx 16 -Ny 16 -Nz 16 -dx 0.5 -dy 0.5 -dz 0.5 " + FB_PHYS
    R = refmod.Ref(opts, 16 ** 3)
    R.init_positions(0)
    R.init_velocities()
    pos, vel = R.get_particles()
    phi = smooth_phi(R.shape, 13, amp=1e-3)
    out = run_pipeline(R, pos, vel, phi, 1e-5, 1)
    out["opts"] = opts
    out["params"] = json.dumps(R.params)
    out["init_pos"] = pos
    out["init_vel"] = vel
    return out


def case_rng():
    R = refmod.Ref("-Nx 4 -Ny 4 -Nz 4", 64)
    out = {}
    a, s = R.ran3(-12345, 2000)
    out["ran3_m12345"] = a
    out["ran3_m12345_state"] = np.int64(s)
    b, s = R.ran3(s, 500)
    out["ran3_continue"] = b
    c, s = R.gasdev(-12345, 2001)
    out["gasdev_m12345"] = c
    d, s = R.ran1(-777, 1000)
    out["ran1_m777"] = d
    R2 = refmod.Ref("-Nx 8 -Ny 8 -Nz 8 -dx 1 -dy 1 -dz 1", 1000)
    R2.init_positions(0)
    out["sobol_8cube_1000"], _ = R2.get_particles()
    return out


def case_twod():
    opts = "-ndim 2 -Nx 8 -Ny 6 -dx 0.5 -dy 1.0 -mn 0 " + C1_PHYS
    R = refmod.Ref(opts, 4 * 48)
    R.init_positions(0)
    R.init_velocities()
    pos, vel = R.get_particles()
    out = {"init_pos": pos.copy(), "init_vel": vel.copy()}
    extra = np.array([[3.99, 5.5], [0.0, 0.0], [0.5, 1.0], [3.999, 5.999], [0.01, 3.3], [3.75, 0.25]])
    pos = np.concatenate([pos[: pos.shape[0] - extra.shape[0]], extra])
    vel = vel.copy()
    vel[-3] = [0.5, 0.4]    # crosses both upper bounds
    vel[-2] = [-0.5, 0.1]   # crosses x = 0
    phi = smooth_phi(R.shape, 31, amp=2.0)
    out.update({"pos0": pos.copy(), "vel0": vel.copy(), "phi": phi.copy(), "dt": np.float64(0.1)})
    R.set_particles(pos, vel)
    R.set_phi(phi)
    R.push(0.1)
    _, vpush = R.get_particles()
    out["vel_push"] = vpush.copy()
    R.update_positions(0.1)
    pmove, vmove = R.get_particles()
    out["pos_move"] = pmove.copy()
    out["vel_move"] = vmove.copy()
    R.collect()
    out["moments"] = R.get_moments()
    out["rhs"] = R.rhs()
    out["lhs"] = R.lhs_dense()
    out["opts"] = opts
    out["params"] = json.dumps(R.params)
    opts_lap = "-ndim 2 -Nx 8 -Ny 6 -dx 0.1 -dy 0.125 -n0 2.5 -mn 0 -lhs laplacian -rhs sinusoidal " + C1_PHYS
    R2 = refmod.Ref(opts_lap, 8)
    out["lap_rhs"] = R2.rhs()
    out["lap_lhs"] = R2.lhs_dense()
    out["lap_opts"] = opts_lap
    out["lap_params"] = json.dumps(R2.params)
    return out


OPS_BASE = "-Nx 6 -Ny 5 -Nz 4 -dx 0.1 -dy 0.125 -dz 0.2 -n0 2.5 " + C1_PHYS
OPS_VARIANTS = {
    "lap_sin": "-lhs laplacian -rhs sinusoidal",
    "lap_const_zrefl": "-lhs laplacian -rhs constant -zBC inject-reflect",
    "id_const": "-lhs identity -rhs constant",
    "full_sin": "-lhs full -rhs sinusoidal",
}


def case_ops():
    out = {"opts_base": OPS_BASE, "variants": json.dumps(OPS_VARIANTS)}
    for name, extra in OPS_VARIANTS.items():
        R = refmod.Ref(OPS_BASE + extra, 8)
        if name == "full_sin":  # a density for the variable-coefficient operator
            m = np.zeros(R.shape + (4,))
            m[..., 0] = 2.0 + smooth_phi(R.shape, 21, amp=0.3)
            R.set_moments(m)
            out["full_sin_density"] = m[..., 0]
        out[f"{name}_rhs"] = R.rhs()
        out[f"{name}_lhs"] = R.lhs_dense()
        out[f"{name}_params"] = json.dumps(R.params)
    return out


CASES = {"c1": case_c1, "edge": case_edge, "fb": case_fb, "rng": case_rng, "ops": case_ops, "twod": case_twod}


def main():
    if len(sys.argv) == 3 and sys.argv[1] == "--case":
        name = sys.argv[2]
        data = CASES[name]()
        np.savez_compressed(HERE / f"{name}.npz", **data)
        return
    if not refmod.LIB_PATH.exists():
        refmod.build()
    for name in CASES:
        subprocess.run([sys.executable, __file__, "--case", name], check=True)
        print("wrote", HERE / f"{name}.npz", (HERE / f"{name}.npz").stat().st_size, "bytes")


if __name__ == "__main__":
    main()
