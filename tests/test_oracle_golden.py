"""Pin the oracle restatement against the reference's own outputs.

The golden vectors (tests/golden/*.npz) were produced by the reference's
unmodified hot-path sources compiled against the PETSc-API shim
(tests/golden/make_golden.py).  Every stage is fed the reference's input and
must reproduce the reference's output bit for bit: all of it is FP64 arithmetic
evaluated in the same order, and the oracle is compiled without FMA
contraction.
"""
import numpy as np
import pytest

from oracle import oracle as orc


def eq(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape
    diff = np.flatnonzero(a.ravel() != b.ravel())
    assert diff.size == 0, f"{diff.size} of {a.size} values differ; first at {diff[:5]}: {a.ravel()[diff[:5]]} vs {b.ravel()[diff[:5]]}"


@pytest.fixture(scope="module")
def O(built, golden):
    return {k: orc.Oracle(golden[k]["params"]) for k in ("c1", "edge", "fb")}


@pytest.mark.parametrize("case", ["c1", "edge", "fb"])
def test_push_bit_exact(O, golden, case):
    g = golden[case]
    eq(O[case].push(g["pos0"], g["vel0"], g["phi"], float(g["dt"])), g["vel_push"])


@pytest.mark.parametrize("case", ["c1", "edge", "fb"])
def test_move_bit_exact(O, golden, case):
    g = golden[case]
    pos, vel = O[case].move(g["pos0"], g["vel_push"], float(g["dt"]))
    eq(pos, g["pos_move"])
    eq(vel, g["vel_move"])


@pytest.mark.parametrize("case", ["c1", "edge", "fb"])
def test_collect_bit_exact(O, golden, case):
    g = golden[case]
    eq(O[case].collect(g["pos_move"], g["vel_move"]), g["moments"])


@pytest.mark.parametrize("case", ["c1", "edge", "fb"])
def test_rhs_bit_exact(O, golden, case):
    g = golden[case]
    eq(O[case].rhs(g["moments"]), g["rhs"])


@pytest.mark.parametrize("case", ["c1", "edge", "fb"])
def test_lhs_bit_exact(O, golden, case):
    g = golden[case]
    A = O[case].lhs_dense(g["moments"][..., 0])
    nz, ny, nx = O[case].shape
    offs = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1),
            (1, 1, 0), (1, -1, 0), (-1, 1, 0), (-1, -1, 0), (0, 0, 0)]
    rows = np.zeros_like(g["lhs_rows"])
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                r = (k * ny + j) * nx + i
                for e, (di, dj, dk) in enumerate(offs):
                    c = (((k + dk) % nz) * ny + (j + dj) % ny) * nx + (i + di) % nx
                    rows[r, e] = A[r, c]
    eq(rows, g["lhs_rows"])
    # the operator has zero row and column sums (constant null space on both sides)
    assert np.abs(A.sum(axis=1)).max() < 1e-12 * np.abs(A).max()
    assert np.abs(A.sum(axis=0)).max() < 1e-12 * np.abs(A).max()


def test_rng_streams(built, golden):
    g = golden["rng"]
    orc.rng_reset()
    a, s = orc.ran3(-12345, 2000)
    eq(a, g["ran3_m12345"])
    assert s == int(g["ran3_m12345_state"])
    b, s = orc.ran3(s, 500)
    eq(b, g["ran3_continue"])
    c, _ = orc.gasdev(-12345, 2001)
    eq(c, g["gasdev_m12345"])
    d, _ = orc.ran1(-777, 1000)
    eq(d, g["ran1_m777"])


def test_sobol(O, golden):
    g = golden["rng"]
    P = dict(golden["c1"]["params"])
    eq(orc.Oracle(P).sobol(1000), g["sobol_8cube_1000"])


@pytest.mark.parametrize("case", ["c1", "fb"])
def test_initial_state(O, golden, case):
    g = golden[case]
    P = g["params"]
    eq(O[case].sobol(g["init_pos"].shape[0]), g["init_pos"])
    orc.rng_reset()
    vel = orc.normal_velocities([P["viTx"], P["viTy"], P["viTz"]], [P["vi0x"], P["vi0y"], P["vi0z"]],
                                g["init_vel"].shape[0])
    eq(vel, g["init_vel"])


@pytest.mark.parametrize("case", ["c1", "fb"])
def test_collisions_bit_exact(O, golden, case):
    """ScatterElastic with the reference's RNG state sequence: initial
    velocities (gasdev on ran1), then successive collision calls (ran3 is
    re-seeded every call, src/collisions.c:41 with src/random.c:103)."""
    g = golden[case]
    P = g["params"]
    orc.rng_reset()
    orc.normal_velocities([P["viTx"], P["viTy"], P["viTz"]], [P["vi0x"], P["vi0y"], P["vi0z"]],
                          g["init_vel"].shape[0])
    v = g["vel_push"]
    c = 1
    while f"vel_collide{c}" in g:
        v, ns, stats = O[case].collide(v, float(g["dt"]))
        eq(v, g[f"vel_collide{c}"])
        assert ns == O[case].collision_count(v.shape[0], float(g["dt"]))
        c += 1
    assert c > 1


OPS_VARIANTS = ("lap_sin", "lap_const_zrefl", "id_const", "full_sin")


@pytest.mark.parametrize("variant", OPS_VARIANTS)
def test_operator_options_bit_exact(built, variant):
    """-lhs identity / laplacian and -rhs constant / sinusoidal (src/lhs.c:11-191,
    src/rhs.c:6-148) against the reference's own RHS vectors and assembled
    matrices, bit for bit."""
    import json

    from conftest import GOLDEN
    d = np.load(GOLDEN / "ops.npz")
    params = json.loads(str(d[f"{variant}_params"]))
    O = orc.Oracle(params)
    dens = d["full_sin_density"] if variant == "full_sin" else np.zeros(O.shape)
    m = np.zeros(O.shape + (4,))
    m[..., 0] = dens
    eq(O.rhs(m), d[f"{variant}_rhs"])
    eq(O.lhs_dense(dens), d[f"{variant}_lhs"])


def test_two_d_bit_exact(built):
    """-ndim 2 (BorisMoverBz2D + DifferenceVector2D, UpdatePositions +
    Apply2DBC, Collect2DFluidMoments, ComputeFullRHS2D, ComputeFullLHS2D,
    ComputeLaplacianLHS2D, ComputeSinusoidalRHS2D) against the reference."""
    import json

    from conftest import GOLDEN
    d = np.load(GOLDEN / "twod.npz")
    O = orc.Oracle(json.loads(str(d["params"])))
    vel = O.push(d["pos0"], d["vel0"], d["phi"], float(d["dt"]))
    eq(vel, d["vel_push"])
    pos, vel = O.move(d["pos0"], d["vel_push"], float(d["dt"]))
    eq(pos, d["pos_move"])
    eq(vel, d["vel_move"])
    m = O.collect(d["pos_move"], d["vel_move"])
    eq(m, d["moments"])
    eq(O.rhs(d["moments"]), d["rhs"])
    eq(O.lhs_dense(d["moments"][..., 0]), d["lhs"])
    O2 = orc.Oracle(json.loads(str(d["lap_params"])))
    eq(O2.rhs(np.zeros(O2.shape + (4,))), d["lap_rhs"])
    eq(O2.lhs_dense(np.zeros(O2.shape)), d["lap_lhs"])


@pytest.mark.parametrize("zbc", ["periodic", "reflect"])
def test_multithreaded_deposit_matches_serial(zbc):
    """The slab-decomposed deposit that times the CPU baseline sums the same
    CIC weights as the reference-order deposit, in another order."""
    import ecsprt_gb300 as E
    opts = "-Nx 12 -Ny 10 -Nz 9 -dx 1 -dy 1 -dz 1 -qi 1 -mi 1 -B0 0.1 -viT 1 -vi0x 0.5"
    if zbc == "reflect":
        opts += " -zBC inject-reflect"
    p = E.params_from_options(opts)
    O = orc.Oracle(p)
    rng = np.random.default_rng(5)
    n = 20000
    pos = rng.uniform(0, 1, (n, 3)) * [12, 10, 9]
    vel = rng.standard_normal((n, 3))
    a = O.collect(pos, vel)
    b = O.collect_mt(pos, vel)
    assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max()
    assert abs(b[..., 0].sum() - (n if zbc == "periodic" else a[..., 0].sum())) <= 1e-9 * n
