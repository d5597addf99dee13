"""Seeded synthetic inputs of the serving workloads.

The reference has no generator for these fields (its only built-in density is
the fixed 1 + 0.25 sin of src/positions.c:246-247, and its stand-alone solver
reads a density from an HDF5 file, src/file-io.c:45), so the same arrays are
generated here for the GPU path and for any CPU check:

* stand-alone solves: grids N^3 with N uniform over {32, 48, 64, 96, 128},
  density = lognormal(0, 0.1) x (1 + sum of 12 random Fourier modes of
  amplitude 0.05), Poisson arrivals;
* simulation ensembles: grids N^3 with N uniform over {32, 48, 64}, 16 ions
  per cell, drift uniform in [0.2, 1.5] (thermal speed 1), collision
  frequency log-uniform in [0.005, 0.1].

Fourier modes have integer wavevectors (kx, ky, kz) with 0 < |k| <= kmax in
units of 2 pi / L and phases uniform in [0, 2 pi).
"""
from __future__ import annotations

import numpy as np

SOLVE_SIZES = (32, 48, 64, 96, 128)
SIM_SIZES = (32, 48, 64)


def solver_options(n: int) -> str:
    """Options of a stand-alone solve on an n^3 periodic grid (unit spacing,
    the electron parameters of the particle workload: kappa_e about 2)."""
    return (f"-Nx {n} -Ny {n} -Nz {n} -dx 1 -dy 1 -dz 1 -qi 1 -mi 1 -B0 0.1 -viT 1 "
            f"-nue 8.79e9 -Te 11604.5 -E0 0")


def sim_options(n: int, ppc: int, drift: float, nu: float, dt: float = 0.1) -> str:
    return (f"-Nx {n} -Ny {n} -Nz {n} -dx 1 -dy 1 -dz 1 -qi 1 -mi 1 -B0 0.1 -viT 1 -vi0x {drift} "
            f"-nui {nu} -nue 8.79e9 -Te 11604.5 -E0 0 -Np -{ppc} -dt {dt}")


def random_modes(nmodes: int, amplitude: float, rng: np.random.Generator, kmax: int = 4):
    """[(kx, ky, kz, amplitude, phase)]: integer wavevectors with
    0 < |k| <= kmax, phases uniform in [0, 2 pi)."""
    ks = []
    while len(ks) < nmodes:
        k = rng.integers(-kmax, kmax + 1, size=3)
        if 0 < float(np.sqrt((k * k).sum())) <= kmax:
            ks.append(k)
    phases = rng.uniform(0.0, 2.0 * np.pi, nmodes)
    return [(int(k[0]), int(k[1]), int(k[2]), float(amplitude), float(ph)) for k, ph in zip(ks, phases)]


# the 256 x 256 x 128 workload's initial density: 1 + 8 modes of amplitude 0.02
C3_SEED = 20261208


def c3_modes():
    return random_modes(8, 0.02, np.random.default_rng(C3_SEED))


def fourier_modes(shape, nmodes: int, amplitude: float, rng: np.random.Generator, kmax: int = 4) -> np.ndarray:
    """sum_m amplitude cos(k_m . r + phi_m) on a [Nz][Ny][Nx] grid of unit
    cells (r at the nodes, L = the grid extent)."""
    nz, ny, nx = shape
    modes = random_modes(nmodes, amplitude, rng, kmax)
    ks = [np.array(m[:3]) for m in modes]
    phases = [m[4] for m in modes]
    x = 2.0 * np.pi * np.arange(nx) / nx
    y = 2.0 * np.pi * np.arange(ny) / ny
    z = 2.0 * np.pi * np.arange(nz) / nz
    out = np.zeros(shape)
    for k, ph in zip(ks, phases):
        # separable: cos(a + b + c) through complex exponentials
        e = (np.exp(1j * k[2] * z)[:, None, None] * np.exp(1j * k[1] * y)[None, :, None] *
             np.exp(1j * (k[0] * x + ph))[None, None, :])
        out += amplitude * e.real
    return out


def solve_density(n: int, rng: np.random.Generator) -> np.ndarray:
    """lognormal(0, 0.1) x (1 + 12 Fourier modes of amplitude 0.05), n^3."""
    shape = (n, n, n)
    return rng.lognormal(0.0, 0.1, shape) * (1.0 + fourier_modes(shape, 12, 0.05, rng))


def solve_requests(count: int, rate: float, seed: int, sizes=SOLVE_SIZES):
    """(arrival time in seconds, grid edge) of `count` Poisson arrivals at
    `rate` per second, grid edges uniform over `sizes`."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, count)
    gaps[0] = 0.0
    return np.cumsum(gaps), rng.choice(np.asarray(sizes), count)


def sim_instances(count: int, seed: int, sizes=SIM_SIZES):
    """Per instance: grid edge, drift (x, in thermal speeds), collision frequency."""
    rng = np.random.default_rng(seed)
    n = rng.choice(np.asarray(sizes), count)
    drift = rng.uniform(0.2, 1.5, count)
    nu = np.exp(rng.uniform(np.log(0.005), np.log(0.1), count))
    return [(int(a), float(b), float(c)) for a, b, c in zip(n, drift, nu)]


def uniform_ions(n: int, ppc: int, drift: float, rng: np.random.Generator):
    """Uniform positions on an n^3 box, Maxwellian velocities (thermal speed
    1 per component) plus the drift along x: pos, vel as [np][3] FP64."""
    N = n ** 3 * ppc
    pos = rng.uniform(0.0, float(n), (N, 3))
    vel = rng.standard_normal((N, 3))
    vel[:, 0] += drift
    return pos, vel
