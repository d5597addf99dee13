"""The reference's programs and loop order on the GPU library, through C.

test_slot_order_matches_step
    tests/c/slot_order.c, compiled here against include/ and libecsgpu, runs
    src/pic.c:244-258 through the operator slots the reference binds
    (EcsGpuBindOperatorsFor -> EcsGpuUpdateVelocities -> EcsGpuUpdatePositions
    -> ops.collect -> EcsGpuComputePotential) on one context and the fused
    ecs_step on another: moments, potential and ions (matched by identity)
    must agree bit for bit after every step, collisions included.

test_pic_program
    The re-hosted pic program (ecsprt_gb300/host/ecs_pic_main.c) reads
    petsc.ini plus the command line, writes options.log and the fluid and
    particle files under the reference's names, and its final fluid output
    equals, bit for bit, the same sequence run through the Python mirror of
    the operator interface.

test_solver_program
    The re-hosted solver program reads a density (PETSc binary Vec in place
    of the HDF5 dataset density-kji), scales the fluxes by --flux-scale and
    writes fluid.bin; its potential equals Context.solve_density's bit for
    bit.
"""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import ecsprt_gb300 as E
from ecsprt_gb300 import build as B

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent


def read_vecs(path, count):
    """`count` consecutive PETSc binary Vecs (class id 1211214, big-endian)."""
    raw = Path(path).read_bytes()
    out, off = [], 0
    for _ in range(count):
        cid, n = np.frombuffer(raw, dtype=">i4", count=2, offset=off)
        assert cid == 1211214
        out.append(np.frombuffer(raw, dtype=">f8", count=int(n), offset=off + 8).astype(np.float64))
        off += 8 + 8 * int(n)
    assert off == len(raw)
    return out


def write_vec(path, v):
    v = np.ascontiguousarray(v, dtype=np.float64).ravel()
    Path(path).write_bytes(np.array([1211214, v.size], dtype=">i4").tobytes() + v.astype(">f8").tobytes())


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_slot_order_matches_step(built, tmp_path, prec):
    cc = shutil.which("gcc") or "cc"
    exe = tmp_path / "slot_order"
    subprocess.run([cc, "-O2", "-std=gnu11", "-Wall", "-Wextra", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "c" / "slot_order.c"), "-o", str(exe), f"-L{B.OUT}", "-lecsgpu",
                    "-lecshost", "-lm", f"-Wl,-rpath,{B.OUT}"], check=True)
    r = subprocess.run([str(exe), prec, "6"], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bit-identical" in r.stdout
    assert " 0 collisions" not in r.stdout


PIC_INI = """# options file, as run.sh writes petsc.ini
-Nx 16 -Ny 16 -Nz 16 -dx 1 -dy 1 -dz 1
-qi 1 -mi 1 -B0 0.1 -viT 1 -vi0x 0.5 -nui 0.5 -nue 8.79e9 -Te 11604.5 -E0 0
-Np -8 -Nt 2 -dt 0.1 --every 2 --output-particles
-ksp_rtol 1e-9
"""


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_pic_program(built, tmp_path, prec):
    (tmp_path / "petsc.ini").write_text(PIC_INI)
    exe = Path(B.OUT) / "pic"
    # the command line overrides the options file
    r = subprocess.run([str(exe), "-Nt", "3", "--precision", prec, "--seed", "11", "--log-level", "2"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=300)
    print(r.stdout[-2000:])
    assert r.returncode == 0, r.stdout + r.stderr
    names = sorted(f.name for f in tmp_path.iterdir())
    for want in ("options.log", "fluid-initial.bin", "fluid-0.bin", "fluid-2.bin", "fluid-final.bin",
                 "position-initial.bin", "velocity-0.bin", "position-final.bin"):
        assert want in names, names
    assert "fluid-1.bin" not in names  # --every 2
    assert "-Nt 3" in (tmp_path / "options.log").read_text()
    n = 16 ** 3
    dens, gx, gy, gz, rhs, phi = read_vecs(tmp_path / "fluid-final.bin", 6)
    pos = read_vecs(tmp_path / "position-final.bin", 1)[0].reshape(-1, 3)
    assert pos.shape == (8 * n, 3) and (pos >= 0).all() and (pos < 16).all()
    assert abs(dens.sum() - 8 * n) <= 1e-6 * 8 * n

    # the same sequence through the Python mirror of the operator interface
    p = E.params_from_options(" ".join(ln for ln in PIC_INI.splitlines() if not ln.startswith("#")) + " -Nt 3")
    with E.Context(p, E.ECS_PREC_FP64 if prec == "fp64" else E.ECS_PREC_MIXED, np_capacity=8 * n) as ctx:
        ctx.set_seed(11)
        ctx.init_particles(E.ECS_INIT_SOBOL, 8 * n, seed=11)
        ctx.collect()
        ctx.compute_potential(rtol=1e-9, max_it=10000)
        for _ in range(3):
            ctx.update_velocities(0.1)
            ctx.update_positions(0.1)
            ctx.collect()
            ctx.compute_potential(rtol=1e-9, max_it=10000)
        m, ref_phi, ref_rhs = ctx.moments, ctx.phi, ctx.rhs
    assert np.array_equal(dens, m[..., 0].ravel())
    assert np.array_equal(np.stack([gx, gy, gz], -1), m[..., 1:].reshape(-1, 3))
    assert np.array_equal(rhs, ref_rhs.ravel())
    assert np.array_equal(phi, ref_phi.ravel())


def test_solver_program(built, tmp_path):
    from ecsprt_gb300 import workloads as W

    n = 32
    dens = W.solve_density(n, np.random.default_rng(5))
    write_vec(tmp_path / "density.bin", dens)
    opts = W.solver_options(n)
    (tmp_path / "petsc.ini").write_text(opts + "\n-ksp_rtol 1e-8\n")
    exe = Path(B.OUT) / "solver"
    r = subprocess.run([str(exe), "--input", "density.bin", "--flux-scale", "0.5", "--y-flux-scale", "0.25"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=300)
    print(r.stdout[-1500:])
    assert r.returncode == 0, r.stdout + r.stderr
    d, gx, gy, gz, rhs, phi = read_vecs(tmp_path / "fluid.bin", 6)
    assert np.array_equal(d, dens.ravel())
    assert np.array_equal(gx, 0.5 * dens.ravel()) and np.array_equal(gy, 0.25 * dens.ravel())
    p = E.params_from_options(opts)
    with E.Context(p, E.ECS_PREC_MIXED) as ctx:
        ref, st = ctx.solve_density(dens, flux_scale=(0.5, 0.25, 0.5), rtol=1e-8, max_it=10000)
    assert st.relres <= 1e-8
    assert np.array_equal(phi, ref.ravel())
    # an option the reference's solver has and this build cannot honour is refused
    r = subprocess.run([str(exe), "--input", "density.bin", "--view-lhs"], cwd=tmp_path, capture_output=True,
                       text=True, timeout=120)
    assert r.returncode != 0 and "not available" in r.stderr
