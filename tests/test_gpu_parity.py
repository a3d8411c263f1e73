"""GPU parity: the CUDA engine through its C ABI (libqsg.so) against the oracle.

The bar (complex128 "plain" form): relative L2 error <= 1e-12 against the
reference's own CPU evolution on the same inputs (golden fixtures made by the
reference; the C oracle, bit-exact with the reference on every fixture, for
shapes computed live).  The complex64 "mixed" form is held to relative L2
<= 1e-5 against the same FP64 result.
"""
import numpy as np
import pytest

from tests.conftest import load_golden
from tests.workloads import gauss_packet_1d, gauss_packet_2d, gaussian_bumps_2d

pytestmark = pytest.mark.gpu

PLAIN_TOL = 1e-12
MIXED_TOL = 1e-5


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.fixture(scope="module")
def qsg():
    import qusim_gb300 as q
    q.load()
    return q


@pytest.fixture(scope="module")
def ctx(qsg):
    return qsg.Context(0)


def mass_hbar(g):
    """(mass, hbar) of a fixture; 1, 1 where it stores none."""
    return float(g.get("mass", 1.0)), float(g.get("hbar", 1.0))


def run_1d(qsg, ctx, g, precision):
    n, x0, x1, order, wall, batch, calls, fnes = g["params"]
    n, order, batch, calls = int(n), int(order), int(batch), int(calls)
    dx = (x1 - x0) / n
    mass, hbar = mass_hbar(g)
    bc = qsg.BoundaryCondition.InfiniteWall if int(wall) else qsg.BoundaryCondition.Period
    inst = qsg.Instance.create_1d(ctx, g["psi0"], g["V"], dx, complex(g["dt"]), order=order,
                                  precision=precision, mass=mass, hbar=hbar, boundary=bc)
    for _ in range(calls):
        inst.step(batch, renormalize=bool(fnes))
    return inst, dx


# hbar07_m2: hbar = 0.7, mass = 2; their kinetic energies pin the reference's
# two KinEn formulas (the periodic 1D one omits hbar^2,
# src/SplittingMethod1D.cpp:101-102; the wall and 2D ones use (Dk hbar)^2 / 2m)
GOLDEN_1D = ["evolve1d_n4096_o2_2000", "evolve1d_n4096_o4_200", "evolve1d_n256_o2_b7x3_fnes",
             "evolve1d_n1024_o4_imag", "evolve1d_n512_o2_wall", "evolve1d_n1024_o2_hbar07_m2",
             "evolve1d_n512_o4_wall_hbar07_m2", "evolve1d_n1000_o2", "evolve1d_n600_o4_wall",
             "evolve1d_n5000_o4", "evolve1d_n4099_o2_b5x2_fnes", "evolve1d_n3000_o4_wall"]
GOLDEN_2D = ["evolve2d_128x256_o2_50", "evolve2d_256x128_o4_20", "evolve2d_128x128_o4_b5x2_fnes",
             "evolve2d_128x256_o4_hbar07_m2", "evolve2d_45x70_o2_30",
             "evolve2d_96x50_o4_10"]


@pytest.mark.parametrize("name", GOLDEN_1D)
def test_evolve1d_plain_matches_reference(qsg, ctx, name):
    g = load_golden(name)
    inst, dx = run_1d(qsg, ctx, g, "fp64")
    psi = inst.get_psi()
    assert rel_l2(psi, g["psi"]) <= PLAIN_TOL
    assert abs(inst.norm2() - g["norm2"]) <= 1e-12 * abs(g["norm2"])
    kin, pot = inst.energies()
    assert abs(kin - g["kin"]) <= 1e-11 * max(1.0, abs(g["kin"]))
    assert abs(pot - g["pot"]) <= 1e-11 * max(1.0, abs(g["pot"]))


@pytest.mark.parametrize("name", GOLDEN_1D)
def test_evolve1d_mixed_close_to_reference(qsg, ctx, name):
    g = load_golden(name)
    inst, dx = run_1d(qsg, ctx, g, "mixed")
    assert rel_l2(inst.get_psi(), g["psi"]) <= MIXED_TOL
    assert abs(inst.norm2() - g["norm2"]) <= 1e-5


@pytest.mark.parametrize("name", GOLDEN_2D)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_evolve2d_matches_reference(qsg, ctx, name, precision):
    g = load_golden(name)
    nx, ny, x0, x1, y0, y1, order, batch, calls, fnes = g["params"]
    nx, ny, order, batch, calls = int(nx), int(ny), int(order), int(batch), int(calls)
    dx, dy = (x1 - x0) / nx, (y1 - y0) / ny
    mass, hbar = mass_hbar(g)
    inst = qsg.Instance.create_2d(ctx, g["psi0"], g["V"], dx, dy, complex(g["dt"]), order=order,
                                  precision=precision, mass=mass, hbar=hbar)
    for _ in range(calls):
        inst.step(batch, renormalize=bool(fnes))
    tol = PLAIN_TOL if precision == "fp64" else MIXED_TOL
    assert rel_l2(inst.get_psi(), g["psi"]) <= tol
    assert abs(inst.norm2() - g["norm2"]) <= (1e-12 if precision == "fp64" else 1e-5)
    kin, pot = inst.energies()
    etol = 1e-10 if precision == "fp64" else 1e-4
    assert abs(kin - g["kin"]) <= etol * max(1.0, abs(g["kin"]))
    assert abs(pot - g["pot"]) <= etol * max(1.0, abs(g["pot"]))


# shapes that exercise every x-split (G = 1, 2, 4) and row/column tile shape
SPLIT_SHAPES = [(4096, 128, 4), (2048, 256, 2), (128, 4096, 4), (512, 512, 2), (1024, 128, 2)]


@pytest.mark.parametrize("nx,ny,order", SPLIT_SHAPES)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_evolve2d_shapes_vs_oracle(qsg, ctx, oracle, nx, ny, order, precision):
    hx, hy = 0.05 * nx, 0.05 * ny
    psi0, dx, dy = gauss_packet_2d(nx, ny, -hx, hx, -hy, hy, kx=1.0, ky=0.5, xc=-0.2 * hx, yc=0.1 * hy,
                                   s=0.08 * min(hx, hy))
    V = gaussian_bumps_2d(nx, ny, -hx, hx, -hy, hy, nbumps=8, seed=1, spread=0.5 * min(hx, hy))
    nsteps = 3
    ref = oracle.evolve2d(psi0, V, dx, dy, 0.01, nsteps, order=order)
    inst = qsg.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=order, precision=precision)
    inst.step(nsteps)
    tol = PLAIN_TOL if precision == "fp64" else MIXED_TOL
    assert rel_l2(inst.get_psi(), ref) <= tol


@pytest.mark.parametrize("nx,ny,precision", [(8192, 128, "fp64"), (8192, 128, "mixed"), (8192, 2048, "fp64"),
                                             (8192, 4096, "mixed")])
def test_evolve2d_8192_columns_vs_oracle(qsg, ctx, oracle, nx, ny, precision):
    """Grids with 8192 sites along x (the columns): the x split (G = 4) leaves
    2048-point column transforms.  Two O2 steps in two calls against the oracle,
    with Norm2, KinEn and PotEn."""
    hx, hy = 0.0125 * nx, 0.05 * ny
    psi0, dx, dy = gauss_packet_2d(nx, ny, -hx, hx, -hy, hy, kx=1.0, ky=0.5, xc=-0.2 * hx, yc=0.1 * hy,
                                   s=0.08 * min(hx, hy))
    V = gaussian_bumps_2d(nx, ny, -hx, hx, -hy, hy, nbumps=8, seed=2, spread=0.5 * min(hx, hy))
    ref = oracle.evolve2d(psi0, V, dx, dy, 0.01, 2, order=2)
    inst = qsg.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=2, precision=precision)
    inst.step(1)
    inst.step(1)
    tol = PLAIN_TOL if precision == "fp64" else MIXED_TOL
    assert rel_l2(inst.get_psi(), ref) <= tol
    etol = 1e-10 if precision == "fp64" else 1e-4
    kin, pot = inst.energies()
    assert abs(kin - oracle.kinen2d(ref, dx, dy)) <= etol * abs(kin)
    assert abs(pot - oracle.poten(ref, V, dx * dy)) <= etol * max(1.0, abs(pot))
    # sums of up to 33.5 M terms in another order than the reference's: 1e-11 for complex128
    assert abs(inst.norm2() - oracle.norm2(ref, dx * dy)) <= (1e-11 if precision == "fp64" else 1e-5)
    inst.close()


@pytest.mark.parametrize("nx,form", [(128, "momentum"), (1024, "direct"), (4096, "momentum")])
def test_evolve2d_8192_rows_vs_oracle(qsg, ctx, oracle, nx, form):
    """complex64 grids with rows of 8192 sites (y), one or two rows per unit of
    the row pass.  Two O2 steps in two calls against the oracle, with the
    energies; complex128 has no row pass of that length and refuses the grid."""
    ny = 8192
    hx, hy = 0.05 * nx, 0.0125 * ny
    psi0, dx, dy = gauss_packet_2d(nx, ny, -hx, hx, -hy, hy, kx=1.0, ky=0.5, xc=-0.2 * hx, yc=0.1 * hy,
                                   s=0.08 * min(hx, hy))
    V = gaussian_bumps_2d(nx, ny, -hx, hx, -hy, hy, nbumps=8, seed=3, spread=0.5 * min(hx, hy))
    ref = oracle.evolve2d(psi0, V, dx, dy, 0.01, 2, order=2)
    inst = qsg.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=2, precision="mixed")
    inst.form = form
    inst.step(1)
    inst.step(1)
    assert rel_l2(inst.get_psi(), ref) <= MIXED_TOL
    kin, pot = inst.energies()
    assert abs(kin - oracle.kinen2d(ref, dx, dy)) <= 1e-4 * abs(kin)
    assert abs(pot - oracle.poten(ref, V, dx * dy)) <= 1e-4 * max(1.0, abs(pot))
    inst.close()
    if nx == 128:
        with pytest.raises(qsg.QsgError) as e:
            qsg.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=2, precision="fp64")
        assert e.value.code == 5


@pytest.mark.parametrize("n", [64, 128, 512, 2048, 4096])
@pytest.mark.parametrize("order", [2, 4])
def test_evolve1d_sizes_vs_oracle(qsg, ctx, oracle, n, order):
    psi0, V, dx = gauss_packet_1d(n, -0.05 * n, 0.05 * n, 1.5, -0.01 * n, 0.01 * n + 1, barrier=0.7)
    ref = oracle.evolve1d(psi0, V, dx, 0.02, 25, order=order)
    for precision, tol in (("fp64", PLAIN_TOL), ("mixed", MIXED_TOL)):
        inst = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.02, order=order, precision=precision)
        inst.step(25)
        assert rel_l2(inst.get_psi(), ref) <= tol, precision


def test_batch_equals_repeated_steps(qsg, ctx):
    psi0, V, dx = gauss_packet_1d(1024, -50, 50, 1.0, -10, 3.0)
    a = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.02, order=4)
    b = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.02, order=4)
    a.step(10)
    for _ in range(10):
        b.step(1)
    assert rel_l2(a.get_psi(), b.get_psi()) <= 1e-13
    assert a.steps_taken() == b.steps_taken() == 10


def test_tunnelling_known_answer_gpu(qsg, ctx):
    """QuSimPrecision.cpp:82: transmission 0.15937744085 at t=64."""
    ref = (0.1593774409 + 0.1593774408) / 2
    n, x0, x1, dt = 2048, -100.0, 100.0, 0.02
    dx = (x1 - x0) / n
    xs = x0 + dx * np.arange(n)
    psi = np.exp(-0.5 * ((xs + 20) / 5) ** 2) * np.exp(1j * xs)
    psi /= np.sqrt(np.sum(np.abs(psi) ** 2) * dx)
    for precision, tol in (("fp64", 1e-9), ("mixed", 2e-6)):
        inst = qsg.Instance.create_1d(ctx, psi, np.exp(-xs * xs), dx, dt, order=4, precision=precision)
        inst.step(3200)
        assert abs(inst.norm2_range(x0, 0.0, x1) - ref) < tol, precision


def test_unsupported_sizes_are_reported(qsg, ctx):
    # periodic lengths that are not powers of two: up to 4194304 (2n - 1 <= 8388608)
    psi0, V, dx = gauss_packet_1d(4194305, -5000, 5000, 1.0, -10, 3.0)
    for precision in ("mixed", "fp64"):
        with pytest.raises(qsg.QsgError) as e:
            qsg.Instance.create_1d(ctx, psi0, V, dx, 0.02, precision=precision)
        assert e.value.code == 5
    # batches take powers of two
    with pytest.raises(qsg.QsgError) as e:
        qsg.Batch(ctx, [psi0[:5000]], [V[:5000]], [dx], [0.01], order=2, precision="mixed")
    assert e.value.code == 5
    with pytest.raises(qsg.QsgError) as e:
        qsg.Instance.create_1d(ctx, psi0[:512], V[:512], dx, 0.02, order=3)
    assert e.value.code == 1
    # 2D sides that are not powers of two: up to 4096
    z = np.zeros((5000, 128), np.complex128)
    with pytest.raises(qsg.QsgError) as e:
        qsg.Instance.create_2d(ctx, z, z.real, 0.1, 0.1, 0.02, precision="mixed")
    assert e.value.code == 5


def test_budget_rejects_oversize(qsg):
    c = qsg.Context(0, hbm_budget=1 << 20)
    psi0, V, dx = gauss_packet_1d(4096, -50, 50, 1.0, -10, 3.0)
    qsg.Instance.create_1d(c, psi0, V, dx, 0.02)  # ~ 0.3 MB, fits
    z = np.zeros((1024, 1024), np.complex128)
    with pytest.raises(qsg.QsgError) as e:
        qsg.Instance.create_2d(c, z, z.real, 0.1, 0.1, 0.02)
    assert e.value.code == 2


def test_evolver_api_mirror(qsg):
    """The Evolver1D API mirror: init with functors, batch, force-normalise."""
    from qusim_gb300 import BoundaryCondition, Evolver1D, Options, SolverMethod
    e = Evolver1D()
    opts = Options().Gb300().Batch(10)
    e.init(lambda x: np.exp(-0.5 * ((x + 20) / 5) ** 2) * np.exp(1j * x), True, 0.02, False,
           lambda x: np.exp(-x * x), -100.0, 100.0, 2048, BoundaryCondition.Period,
           SolverMethod.SplittingMethodO2, 1.0, 1.0, opts)
    assert abs(e.Norm2() - 1) < 1e-13
    x0 = e.Xavg()
    e.step()
    assert abs(e.Time() - 0.2) < 1e-15
    assert e.GetPsi().shape == (2048,)
    assert e.Xavg() > x0
    with pytest.raises(ValueError):
        Evolver1D().init(lambda x: 0j, True, 0.02, False, lambda x: 0.0, -1, 1, 64,
                         BoundaryCondition.Period, SolverMethod.SplittingMethodO2, 1, 1, Options())


@pytest.mark.parametrize("nx,ny", [(4096, 128), (2048, 256), (256, 1024), (512, 2048), (1024, 4096)])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_every_plan_matches_oracle(qsg, ctx, oracle, nx, ny, precision):
    hx, hy = 0.05 * nx, 0.05 * ny
    psi0, dx, dy = gauss_packet_2d(nx, ny, -hx, hx, -hy, hy, kx=1.0, ky=0.5, xc=-0.2 * hx, yc=0.1 * hy,
                                   s=0.08 * min(hx, hy))
    V = gaussian_bumps_2d(nx, ny, -hx, hx, -hy, hy, nbumps=8, seed=2, spread=0.5 * min(hx, hy))
    ref = oracle.evolve2d(psi0, V, dx, dy, 0.01, 2, order=4)
    inst = qsg.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=4, precision=precision)
    plans = inst.candidate_plans()
    assert len(plans) >= 1
    tol = PLAIN_TOL if precision == "fp64" else MIXED_TOL
    for p in plans:
        inst.set_psi(psi0)
        inst.set_plan(p)
        inst.step(2)
        err = rel_l2(inst.get_psi(), ref)
        assert err <= tol, (p, err)


def test_autotune_keeps_state(qsg, ctx):
    nx = ny = 1024
    psi0, dx, dy = gauss_packet_2d(nx, ny, -50, 50, -50, 50, 1.0, 0.0, -10.0, 0.0, 4.0)
    V = gaussian_bumps_2d(nx, ny, -50, 50, -50, 50, nbumps=8, seed=3, spread=20.0)
    inst = qsg.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=4, precision="mixed")
    inst.step(3)
    before = inst.get_psi().copy()
    plan, ms = inst.autotune(trial_steps=2, persist=False)
    assert ms > 0
    assert plan.as_tuple() in [p.as_tuple() for p in inst.candidate_plans()]
    assert inst.plan().as_tuple() == plan.as_tuple()
    assert np.array_equal(inst.get_psi(), before)
    assert inst.steps_taken() == 3


@pytest.mark.parametrize("n", [8192, 16384, 32768, 65536, 131072, 262144, 524288, 1048576])
@pytest.mark.parametrize("order", [2, 4])
def test_evolve1d_fourstep_vs_oracle(qsg, ctx, oracle, n, order):
    """Sizes above one CTA run as four-step column / row passes."""
    psi0, V, dx = gauss_packet_1d(n, -0.05 * n, 0.05 * n, 1.5, -0.01 * n, 0.005 * n, barrier=0.7)
    nsteps = 4
    ref = oracle.evolve1d(psi0, V, dx, 0.01, nsteps, order=order)
    for precision, tol in (("fp64", PLAIN_TOL), ("mixed", MIXED_TOL)):
        inst = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.01, order=order, precision=precision)
        inst.step(nsteps)
        assert rel_l2(inst.get_psi(), ref) <= tol, precision
        if precision == "fp64":
            kin, pot = inst.energies()
            assert abs(kin - oracle.kinen1d(ref, dx)) <= 1e-10 * abs(kin)
            assert abs(pot - oracle.poten(ref, V, dx)) <= 1e-10 * max(1, abs(pot))


@pytest.mark.parametrize("n,wall", [(1 << 22, False), (1 << 23, False), (2000000, False), (4000000, False),
                                    (1 << 21, True), (1 << 22, True), (1000000, True), (2000000, True)])
def test_largest_1d_lengths_vs_oracle(qsg, ctx, oracle, n, wall):
    """The largest 1D lengths: 2^22 sites (4096 x 1024 four-step passes) and 2^23
    (4096 x 2048), periodic 2,000,000 and 4,000,000 through Bluestein (M = 2^22,
    2^23), walls of 2^21 and 2^22 (their 2^22 and 2^23 extensions) and of
    1,000,000 and 2,000,000 (Bluestein of the extension, M = 2^22, 2^23).
    Three O2 steps in two calls against the oracle: complex128 <= 1e-12 with
    KinEn and PotEn at 1e-10, complex64 <= 1e-5."""
    bc = qsg.BoundaryCondition.InfiniteWall if wall else qsg.BoundaryCondition.Period
    L = 0.01 * n
    psi0, V, dx = gauss_packet_1d(n, -L, L, 1.5, -0.2 * L, 0.02 * L, barrier=0.7)
    ref = oracle.evolve1d(psi0, V, dx, 0.01, 3, order=2, wall=wall)
    for precision, tol in (("fp64", PLAIN_TOL), ("mixed", MIXED_TOL)):
        inst = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.01, order=2, precision=precision, boundary=bc)
        assert inst.plan().as_tuple()[0] == 1
        inst.step(1)
        inst.step(2)
        assert rel_l2(inst.get_psi(), ref) <= tol, (precision, rel_l2(inst.get_psi(), ref))
        if precision == "fp64":
            kin, pot = inst.energies()
            assert abs(kin - oracle.kinen1d(ref, dx, wall=wall)) <= 1e-10 * abs(kin)
            assert abs(pot - oracle.poten(ref, V, dx)) <= 1e-10 * max(1, abs(pot))
        inst.close()


def test_fourstep_renormalize(qsg, ctx, oracle):
    n = 65536
    psi0, V, dx = gauss_packet_1d(n, -0.05 * n, 0.05 * n, 1.0, -100.0, 40.0, barrier=0.5)
    ref = oracle.evolve1d(psi0 * 1.5, V, dx, 0.01 - 0.002j, 3, order=2, renormalize=True)
    inst = qsg.Instance.create_1d(ctx, psi0 * 1.5, V, dx, 0.01 - 0.002j, order=2)
    inst.step(3, renormalize=True)
    assert rel_l2(inst.get_psi(), ref) <= PLAIN_TOL
    assert abs(inst.norm2() - 1) < 1e-13


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_matches_solo_runs(qsg, ctx, precision):
    """Each member of a mixed-size batch evolves exactly as it does alone."""
    rng = np.random.default_rng(7)
    sizes = [1024, 2048, 1024, 8192, 4096, 16384, 65536, 16384, 512]
    psis, Vs, dxs, dts = [], [], [], []
    for n in sizes:
        box = 0.05 * n
        p, v, dx = gauss_packet_1d(n, -box, box, rng.uniform(0.5, 3), -0.25 * box, rng.uniform(2, 20), barrier=0.8)
        psis.append(p), Vs.append(v), dxs.append(dx), dts.append(0.01)
    b = qsg.Batch(ctx, psis, Vs, dxs, dts, order=2, precision=precision)
    # step calls of a repeated count (replayed graphs when QSG_BATCH_GRAPHS=1)
    b.step(7)
    b.step(5)
    b.step(5)
    assert b.sites() == sum(sizes)
    for i, n in enumerate(sizes):
        solo = qsg.Instance.create_1d(ctx, psis[i], Vs[i], dxs[i], dts[i], order=2, precision=precision)
        solo.step(7)
        solo.step(5)
        solo.step(5)
        got = b.instance(i).get_psi()
        assert np.array_equal(got, solo.get_psi()), (i, n)
        assert b.instance(i).steps_taken() == 17
    b.close()



@pytest.mark.parametrize("n", [64, 256, 1024, 2048, 4096])
@pytest.mark.parametrize("order", [2, 4])
def test_wall_vs_oracle(qsg, ctx, oracle, n, order):
    """InfiniteWall (odd extension to 2n) against the oracle's wall path."""
    wall = qsg.BoundaryCondition.InfiniteWall
    psi0, V, dx = gauss_packet_1d(n, -0.05 * n, 0.05 * n, 1.5, -0.01 * n, 0.01 * n + 1, barrier=0.7)
    ref = oracle.evolve1d(psi0, V, dx, 0.02, 25, order=order, wall=True)
    cases = (("fp64", PLAIN_TOL), ("mixed", MIXED_TOL)) if n <= 2048 else (("mixed", MIXED_TOL),)
    for precision, tol in cases:
        inst = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.02, order=order, precision=precision, boundary=wall)
        inst.step(25)
        assert rel_l2(inst.get_psi(), ref) <= tol, precision
        kin, pot = inst.energies()
        ktol = 1e-11 if precision == "fp64" else 1e-5
        assert abs(kin - oracle.kinen1d(ref, dx, wall=True)) <= ktol * abs(kin), precision
        assert abs(pot - oracle.poten(ref, V, dx)) <= ktol * max(1, abs(pot)), precision


def test_wall_imaginary_time_renormalized(qsg, ctx, oracle):
    n = 512
    wall = qsg.BoundaryCondition.InfiniteWall
    psi0, V, dx = gauss_packet_1d(n, -20.0, 20.0, 1.0, -5.0, 3.0, barrier=0.5)
    ref = oracle.evolve1d(psi0 * 2.0, V, dx, 0.01 - 0.003j, 40, order=4, wall=True, renormalize=True)
    inst = qsg.Instance.create_1d(ctx, psi0 * 2.0, V, dx, 0.01 - 0.003j, order=4, boundary=wall)
    inst.step(40, renormalize=True)
    assert rel_l2(inst.get_psi(), ref) <= PLAIN_TOL
    assert abs(inst.norm2() - 1) < 1e-13


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_wall_box_eigenstate(qsg, ctx, precision):
    """A sine mode of the box is stationary: psi(t) = psi(0) exp(-i E t / hbar), E = (pi hbar k / L)^2 / 2m."""
    n, L, k, dt, steps = 1024, 30.0, 3, 0.01, 300
    dx = L / n
    i = np.arange(n)
    psi0 = np.sin(np.pi * k * i / n).astype(np.complex128)
    psi0 /= np.sqrt(np.sum(np.abs(psi0) ** 2) * dx)
    E = (np.pi * k / L) ** 2 / 2
    inst = qsg.Instance.create_1d(ctx, psi0, np.zeros(n), dx, dt, order=2, precision=precision,
                                  boundary=qsg.BoundaryCondition.InfiniteWall)
    inst.step(steps)
    want = psi0 * np.exp(-1j * E * dt * steps)
    tol = 1e-11 if precision == "fp64" else 5e-5
    assert rel_l2(inst.get_psi(), want) <= tol
    kin, _ = inst.energies()
    assert abs(kin - E) <= tol * E


def test_wall_limits_are_reported(qsg, ctx):
    """InfiniteWall: powers of two up to 4194304 (the 2n extension of the largest
    fits the four-step passes' 8388608 sites) and any other length up to 2097152,
    whose Bluestein transforms of the 2n extension take 4n - 1 <= 8388608 sites."""
    wall = qsg.BoundaryCondition.InfiniteWall
    psi0, V, dx = gauss_packet_1d(1 << 23, -5000, 5000, 1.0, -10, 3.0)
    with pytest.raises(qsg.QsgError) as e:
        qsg.Instance.create_1d(ctx, psi0, V, dx, 0.02, boundary=wall)
    assert e.value.code == 5
    for precision in ("mixed", "fp64"):
        with pytest.raises(qsg.QsgError) as e:
            qsg.Instance.create_1d(ctx, psi0[:2097153], V[:2097153], dx, 0.02, boundary=wall, precision=precision)
        assert e.value.code == 5
    with pytest.raises(qsg.QsgError) as e:
        qsg.Instance.create_1d(ctx, psi0[:1], V[:1], dx, 0.02, boundary=wall)
    assert e.value.code == 5


@pytest.mark.parametrize("n", [2, 3, 10, 32, 100, 600, 1000, 2047])
@pytest.mark.parametrize("order", [2, 4])
def test_wall_any_length_vs_oracle(qsg, ctx, oracle, n, order):
    """InfiniteWall at lengths that are not powers of two (and powers of two below
    64): the reference's wall ExpT (src/SplittingMethod1D.cpp:61-81) on its KISS
    transforms of length 2n, here the 2n odd extension in one Bluestein kernel.
    Against the oracle: complex128 <= 1e-12 with the wall KinEn and PotEn at 1e-11,
    complex64 <= 1e-5; hbar = 0.7, m = 2."""
    wall = qsg.BoundaryCondition.InfiniteWall
    L = max(6.0, 0.1 * n)
    psi0, V, dx = gauss_packet_1d(n, -L, L, 1.2, -0.2 * L, max(0.1 * L, 2 * 2 * L / n), barrier=0.6)
    ref = oracle.evolve1d(psi0, V, dx, 0.02, 12, order=order, mass=2.0, hbar=0.7, wall=True)
    for precision, tol in (("fp64", PLAIN_TOL), ("mixed", MIXED_TOL)):
        inst = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.02, order=order, precision=precision, boundary=wall,
                                      mass=2.0, hbar=0.7)
        assert inst.plan().as_tuple() == (0, 0, 0)
        inst.step(5)
        inst.step(7)
        got = inst.get_psi()
        assert got.shape == (n,)
        assert rel_l2(got, ref) <= tol, (precision, rel_l2(got, ref))
        if precision == "fp64":
            kin, pot = inst.energies()
            kr = oracle.kinen1d(ref, dx, mass=2.0, hbar=0.7, wall=True)
            assert abs(kin - kr) <= 1e-11 * abs(kr)
            assert abs(pot - oracle.poten(ref, V, dx)) <= 1e-11 * max(1.0, abs(pot))
            assert abs(inst.norm2() - oracle.norm2(ref, dx)) <= 1e-12
        inst.close()


@pytest.mark.parametrize("n,order", [(2049, 4), (3000, 2), (20000, 4), (65535, 2), (250000, 4)])
def test_wall_long_any_length_vs_oracle(qsg, ctx, oracle, n, order):
    """InfiniteWall at lengths above 2048 that are not powers of two: Bluestein
    transforms of the 2n odd extension on the four-step passes (the two sites the
    reference's wall ExpT discards, src/SplittingMethod1D.cpp:63-65, zeroed by the
    factors that open each transform).  Against the oracle (KISS transforms of
    length 2n): complex128 <= 1e-12 with the wall KinEn and PotEn at 1e-11,
    complex64 <= 1e-5; hbar = 0.7, m = 2."""
    wall = qsg.BoundaryCondition.InfiniteWall
    L = 0.02 * n
    psi0, V, dx = gauss_packet_1d(n, -L, L, 1.2, -0.2 * L, 0.05 * L, barrier=0.6)
    ref = oracle.evolve1d(psi0, V, dx, 0.02, 6, order=order, mass=2.0, hbar=0.7, wall=True)
    for precision, tol in (("fp64", PLAIN_TOL), ("mixed", MIXED_TOL)):
        inst = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.02, order=order, precision=precision, boundary=wall,
                                      mass=2.0, hbar=0.7)
        assert inst.plan().as_tuple()[0] == 1
        inst.step(4)
        inst.step(2)
        got = inst.get_psi()
        assert got.shape == (n,)
        assert rel_l2(got, ref) <= tol, (precision, rel_l2(got, ref))
        kin, pot = inst.energies()
        kr = oracle.kinen1d(ref, dx, mass=2.0, hbar=0.7, wall=True)
        etol = 1e-11 if precision == "fp64" else 1e-4
        assert abs(kin - kr) <= etol * abs(kr), (precision, kin, kr)
        assert abs(pot - oracle.poten(ref, V, dx)) <= etol * max(1.0, abs(pot))
        inst.close()


@pytest.mark.parametrize("n", [1000, 2048, 5000, 8192])
def test_wall_imaginary_time_o4_fine_grid_vs_oracle(qsg, ctx, oracle, n):
    """A wall under a complex dt with O4 on a fine grid (dx = 0.04): the middle
    kinetic substep's negative coefficient d2 amplifies the highest modes by
    exp(|d2| Im(dt) k^2 DT) ~ 3.6e4, so rounding noise fed back at the wall sites
    each transform would grow step after step.  Every wall path (one CTA on the
    2n extension for 2048; Bluestein on it for 1000, in one CTA, and 5000, on the
    four-step passes; the four-step 2n extension for 8192) matches the oracle's
    transforms of the odd extension (src/SplittingMethod1D.cpp:61-81) after 9
    steps in two calls: complex128 <= 1e-12, complex64 <= 1e-5 (zeroing the two
    sites before every transform instead left 4e-3 .. 2e-2 here)."""
    wall = qsg.BoundaryCondition.InfiniteWall
    L = 0.02 * n
    psi0, V, dx = gauss_packet_1d(n, -L, L, 1.0, -0.2 * L, 0.05 * L, barrier=0.5)
    dt = 0.01 - 0.002j
    ref = oracle.evolve1d(psi0, V, dx, dt, 9, order=4, wall=True)
    for precision, tol in (("fp64", PLAIN_TOL), ("mixed", MIXED_TOL)):
        inst = qsg.Instance.create_1d(ctx, psi0, V, dx, dt, order=4, precision=precision, boundary=wall)
        inst.step(4)
        inst.step(5)
        err = rel_l2(inst.get_psi(), ref)
        assert err <= tol, (precision, err)
        inst.close()


@pytest.mark.parametrize("n", [1000, 2048, 8192])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_wall_split_calls_equal_one_call(qsg, ctx, oracle, n, precision):
    """A wall keeps the caller's psi_0 until the first step discards it (as the
    reference's first wall ExpT does, src/SplittingMethod1D.cpp:63-65); the state
    then stays odd to rounding, so 9 steps in one call equal 4 + 5 in two, bit for
    bit, on the one-CTA Bluestein, one-CTA and four-step wall paths."""
    wall = qsg.BoundaryCondition.InfiniteWall
    L = 0.02 * n
    psi0, V, dx = gauss_packet_1d(n, -L, L, 1.0, -0.2 * L, 0.05 * L, barrier=0.5)
    psi0 = psi0.copy()
    psi0[0] = 0.3
    a = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.01 - 0.002j, order=4, precision=precision, boundary=wall)
    b = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.01 - 0.002j, order=4, precision=precision, boundary=wall)
    assert abs(a.get_psi()[0] - 0.3) <= 1e-7
    a.step(9)
    b.step(4)
    b.step(5)
    got = a.get_psi()
    assert np.array_equal(got, b.get_psi())
    ref = oracle.evolve1d(psi0, V, dx, 0.01 - 0.002j, 9, order=4, wall=True)
    assert rel_l2(got, ref) <= (PLAIN_TOL if precision == "fp64" else MIXED_TOL)
    a.close()
    b.close()


def test_wall_long_renormalising_and_set_psi(qsg, ctx, oracle):
    """A renormalising Bluestein four-step wall and its set_psi (the odd
    extension rebuilt, zero above it)."""
    wall = qsg.BoundaryCondition.InfiniteWall
    n = 5001
    psi0, V, dx = gauss_packet_1d(n, -100, 100, 1.0, -20.0, 5.0, barrier=0.5)
    ref = oracle.evolve1d(psi0 * 1.3, V, dx, 0.01 - 0.002j, 9, order=4, wall=True, renormalize=True)
    inst = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.01 - 0.002j, order=4, precision="fp64", boundary=wall)
    inst.step(3)
    inst.set_psi(psi0 * 1.3)
    inst.step(9, renormalize=True)
    assert rel_l2(inst.get_psi(), ref) <= PLAIN_TOL
    assert abs(inst.norm2() - 1.0) <= 1e-13


def test_wall_any_length_renormalising_and_set_psi(qsg, ctx, oracle):
    """A renormalising wall of odd length and its set_psi (the extension rebuilt)."""
    wall = qsg.BoundaryCondition.InfiniteWall
    n = 777
    psi0, V, dx = gauss_packet_1d(n, -40, 40, 1.0, -8.0, 3.0, barrier=0.5)
    ref = oracle.evolve1d(psi0 * 1.3, V, dx, 0.01 - 0.002j, 9, order=2, wall=True, renormalize=True)
    inst = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.01 - 0.002j, order=2, precision="fp64", boundary=wall)
    inst.step(3)
    inst.set_psi(psi0 * 1.3)
    inst.step(9, renormalize=True)
    assert rel_l2(inst.get_psi(), ref) <= PLAIN_TOL
    assert abs(inst.norm2() - 1.0) <= 1e-13


@pytest.mark.parametrize("n,order", [(4097, 4), (4099, 2), (6000, 4), (10007, 2), (100000, 4), (131070, 2),
                                     (200000, 4), (500000, 2)])
def test_periodic_long_any_length_vs_oracle(qsg, ctx, oracle, n, order):
    """Periodic lengths above 4096 that are not powers of two: the reference's
    ExpT/ExpV (src/SplittingMethod1D.cpp:48-57, 83-90) on its KISS transforms of
    length n; here Bluestein's two circular convolutions of length M (the
    smallest power of two >= 2n - 1) per kinetic factor, on the four-step passes.
    Against the oracle: complex128 <= 1e-12 with KinEn and PotEn at 1e-11,
    complex64 <= 1e-5; hbar = 0.7, m = 2, a complex time step."""
    L = 0.02 * n
    psi0, V, dx = gauss_packet_1d(n, -L, L, 1.3, -0.2 * L, 0.05 * L, barrier=0.6)
    dt = 0.02 - 0.001j
    ref = oracle.evolve1d(psi0, V, dx, dt, 6, order=order, mass=2.0, hbar=0.7)
    m = 1 << (2 * n - 2).bit_length()
    for precision, tol in (("fp64", PLAIN_TOL), ("mixed", MIXED_TOL)):
        inst = qsg.Instance.create_1d(ctx, psi0, V, dx, dt, order=order, precision=precision, mass=2.0, hbar=0.7)
        plan = inst.plan().as_tuple()
        assert plan[0] == 1 and plan[2] == 0 and m % plan[1] == 0
        inst.step(2)
        inst.step(4)
        got = inst.get_psi()
        assert got.shape == (n,)
        assert rel_l2(got, ref) <= tol, (precision, rel_l2(got, ref))
        kin, pot = inst.energies()
        kr = oracle.kinen1d(ref, dx, mass=2.0, hbar=0.7)
        etol = 1e-11 if precision == "fp64" else 1e-4
        assert abs(kin - kr) <= etol * abs(kr), (precision, kin, kr)
        assert abs(pot - oracle.poten(ref, V, dx)) <= etol * max(1.0, abs(pot))
        assert abs(inst.norm2() - oracle.norm2(ref, dx)) <= (1e-12 if precision == "fp64" else 1e-5)
        inst.close()


def test_periodic_long_any_length_renormalising_set_psi_and_tune(qsg, ctx, oracle):
    """A renormalising Bluestein four-step instance, its set_psi (the buffer above
    n stays zero) and its tuner (one plan: the state is kept and the plan too)."""
    n = 7777
    psi0, V, dx = gauss_packet_1d(n, -150, 150, 1.0, -30.0, 6.0, barrier=0.5)
    ref = oracle.evolve1d(psi0 * 1.3, V, dx, 0.01 - 0.002j, 9, order=4, renormalize=True)
    inst = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.01 - 0.002j, order=4, precision="fp64")
    inst.step(3)
    inst.set_psi(psi0 * 1.3)
    plan = inst.plan().as_tuple()
    best, ms = inst.autotune(trial_steps=2)
    assert best.as_tuple() == plan and ms > 0
    assert np.array_equal(inst.get_psi(), psi0 * 1.3)
    inst.step(9, renormalize=True)
    assert rel_l2(inst.get_psi(), ref) <= PLAIN_TOL
    assert abs(inst.norm2() - 1.0) <= 1e-13


@pytest.mark.parametrize("nx,ny", [(512, 4096), (1024, 2048)])
def test_tmem_row_pass_equals_shared_memory_row_pass(qsg, ctx, nx, ny):
    """The row pass that parks waiting rows in tensor memory does the same
    arithmetic in the same order as the shared-memory one: bitwise equal."""
    hx, hy = 0.05 * nx, 0.05 * ny
    psi0, dx, dy = gauss_packet_2d(nx, ny, -hx, hx, -hy, hy, kx=1.0, ky=0.5, xc=-0.2 * hx, yc=0.1 * hy,
                                   s=0.08 * min(hx, hy))
    V = gaussian_bumps_2d(nx, ny, -hx, hx, -hy, hy, nbumps=8, seed=4, spread=0.5 * min(hx, hy))
    inst = qsg.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=4, precision="mixed")
    plans = {p.as_tuple(): p for p in inst.candidate_plans()}
    tm = [p for t, p in plans.items() if t[5] == 1]
    assert tm, "no tensor-memory row plan for this grid"
    key = tm[0].as_tuple()
    shared = [p for t, p in plans.items() if t[5] == 0 and (t[0], t[1], t[3], t[4]) == (key[0], key[1], key[3], key[4])]
    assert shared
    out = []
    for p in (tm[0], shared[0]):
        inst.set_psi(psi0)
        inst.set_plan(p)
        inst.step(3)
        inst.step(2, renormalize=True)
        out.append((inst.get_psi(), inst.norm2(), inst.energies()))
    assert np.array_equal(out[0][0], out[1][0])
    assert out[0][1] == out[1][1]
    assert out[0][2] == out[1][2]


def test_batch_graph_replay_equals_direct(qsg, monkeypatch):
    """QSG_BATCH_GRAPHS=1: step calls replayed from a captured CUDA graph give the
    same states as the same launches queued directly."""
    rng = np.random.default_rng(11)
    sizes = [2048, 16384, 1024, 32768]
    psis, Vs, dxs, dts = [], [], [], []
    for n in sizes:
        box = 0.05 * n
        p, v, dx = gauss_packet_1d(n, -box, box, rng.uniform(0.5, 3), -0.25 * box, rng.uniform(2, 20), barrier=0.8)
        psis.append(p), Vs.append(v), dxs.append(dx), dts.append(0.01)
    out = []
    for graphs in ("0", "1"):
        monkeypatch.setenv("QSG_BATCH_GRAPHS", graphs)
        c = qsg.Context(0)
        b = qsg.Batch(c, psis, Vs, dxs, dts, order=4, precision="mixed")
        for _ in range(3):
            b.step(4)
        out.append([b.instance(i).get_psi() for i in range(len(sizes))])
        assert b.instance(0).steps_taken() == 12
        b.close()
        c.close()
    for a, g in zip(*out):
        assert np.array_equal(a, g)


def test_fourstep_tensor_copy_pass_is_bitwise_the_plain_one(qsg, monkeypatch):
    """The complex64 four-step column pass fed by tensor copies (QSG_FS_TMA=1;
    off by default, measured slower) computes exactly what the load-instruction
    pass computes: a mixed-size batch and a single large instance."""
    rng = np.random.default_rng(21)
    sizes = [16384, 32768, 65536, 131072, 262144, 8192, 1024]
    psis, Vs, dxs, dts = [], [], [], []
    for n in sizes:
        box = 0.05 * n
        p, v, dx = gauss_packet_1d(n, -box, box, rng.uniform(0.5, 3), -0.25 * box, rng.uniform(2, 20), barrier=0.8)
        psis.append(p), Vs.append(v), dxs.append(dx), dts.append(0.01)
    out = []
    for tma in ("1", "0"):
        monkeypatch.setenv("QSG_FS_TMA", tma)
        c = qsg.Context(0)
        b = qsg.Batch(c, psis, Vs, dxs, dts, order=4, precision="mixed")
        b.step(3)
        b.step(2)
        got = [b.instance(i).get_psi() for i in range(len(sizes))]
        b.close()
        solo = qsg.Instance.create_1d(c, psis[3], Vs[3], dxs[3], 0.01, order=2, precision="mixed")
        solo.step(4)
        got.append(solo.get_psi())
        got.append(solo.step_norm2())
        solo.close()
        c.close()
        out.append(got)
    for x, y in zip(*out):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("order", [2, 4])
def test_batch_tile_queue_is_bitwise_the_per_class_launches(qsg, monkeypatch, order):
    """complex64 batches step their resident classes of length 1024 .. 8192 in
    one persistent launch fed by a tile queue (8192-site tiles).  Members get
    exactly the states the per-class launches (QSG_BATCH_QUEUE=0) give.  The
    batch has more tiles than the launch has CTAs (so CTAs take several tiles
    and the queue counter is reused by the next call), classes whose last tile
    is partial, sizes below 1024 and four-step sizes beside the queue."""
    rng = np.random.default_rng(33)
    sizes = [1024] * 700 + [2048] * 301 + [4096] * 75 + [8192] * 40 + [512] * 5 + [16384] * 3
    rng.shuffle(sizes)
    psis, Vs, dxs, dts = [], [], [], []
    for n in sizes:
        box = 0.05 * n
        p, v, dx = gauss_packet_1d(n, -box, box, rng.uniform(0.5, 3), -0.25 * box, rng.uniform(2, 20), barrier=0.8)
        psis.append(p), Vs.append(v), dxs.append(dx), dts.append(0.01)
    out = []
    for queue in ("1", "0"):
        monkeypatch.setenv("QSG_BATCH_QUEUE", queue)
        c = qsg.Context(0)
        c.profile(2)
        b = qsg.Batch(c, psis, Vs, dxs, dts, order=order, precision="mixed")
        b.step(3)
        b.step(2)
        out.append([b.instance(i).get_psi() for i in range(len(sizes))])
        kernels = {name: v[0] for name, v in c.profile_read().items()}
        if queue == "1":
            assert kernels.get("evolve1d_queue") == 2
            assert kernels.get("evolve1d_resident") == 2  # the 512-site class
        else:
            assert "evolve1d_queue" not in kernels
        b.close()
        c.close()
    for i, (a, g) in enumerate(zip(*out)):
        assert np.array_equal(a, g), (i, sizes[i])
    c = qsg.Context(0)
    for i in (0, 1, sizes.index(8192), sizes.index(4096)):
        solo = qsg.Instance.create_1d(c, psis[i], Vs[i], dxs[i], 0.01, order=order, precision="mixed")
        solo.step(5)
        assert np.array_equal(solo.get_psi(), out[0][i]), i
        solo.close()
    c.close()


def wall_packet(n):
    """A packet 30 sites from the left wall moving into it (k0 = -2) plus the
    barrier 0.7 exp(-x^2/2), on [-0.05 n, 0.05 n) (dx = 0.1)."""
    x0, x1 = -0.05 * n, 0.05 * n
    xs = x0 + 0.1 * np.arange(n)
    psi = np.exp(-2j * xs) * np.exp(-((xs - (x0 + 3.0)) ** 2) / 4.0)
    psi /= np.sqrt(np.sum(np.abs(psi) ** 2) * 0.1)
    return psi.astype(np.complex128), 0.7 * np.exp(-xs * xs / 2), 0.1


@pytest.mark.parametrize("n", [4096, 8192, 32768, 131072, 524288])
@pytest.mark.parametrize("order", [2, 4])
def test_wall_beyond_one_cta_vs_oracle(qsg, ctx, oracle, n, order):
    """InfiniteWall above the one-CTA sizes (n > 4096 complex64, > 2048
    complex128) runs as a four-step periodic instance of the 2n odd extension
    (src/SplittingMethod1D.cpp:61-81).  The packet reflects off the wall within
    the run; hbar = 0.7 and m = 2 pin the wall KinEn, which keeps hbar^2
    (:117-119).  complex128 <= 1e-12, complex64 <= 1e-5, with Norm2, KinEn,
    PotEn, <x> and a renormalising call."""
    psi0, V, dx = wall_packet(n)
    mass, hbar, dt, steps = 2.0, 0.7, 0.2, 30
    ref = oracle.evolve1d(psi0, V, dx, dt, steps, order=order, mass=mass, hbar=hbar, wall=True)
    ref2 = oracle.evolve1d(ref, V, dx, dt, 3, order=order, mass=mass, hbar=hbar, wall=True, renormalize=True)
    kin_ref = oracle.kinen1d(ref, dx, mass=mass, hbar=hbar, wall=True)
    for precision, tol, otol in (("fp64", PLAIN_TOL, 1e-11), ("mixed", MIXED_TOL, 1e-5)):
        inst = qsg.Instance.create_1d(ctx, psi0, V, dx, dt, order=order, precision=precision, mass=mass,
                                      hbar=hbar, boundary=qsg.BoundaryCondition.InfiniteWall)
        inst.step(steps)
        got = inst.get_psi()
        assert got.shape == (n,)
        assert rel_l2(got, ref) <= tol, (precision, rel_l2(got, ref))
        kin, pot = inst.energies()
        assert abs(kin - kin_ref) <= otol * abs(kin_ref), (precision, kin, kin_ref)
        assert abs(pot - oracle.poten(ref, V, dx)) <= otol, precision
        assert abs(inst.norm2() - oracle.norm2(ref, dx)) <= otol, precision
        assert abs(inst.xavg(-0.05 * n) - oracle.xavg(ref, -0.05 * n, dx)) <= otol * 0.05 * n, precision
        inst.step(3, renormalize=True)
        assert rel_l2(inst.get_psi(), ref2) <= tol, precision
        assert abs(inst.norm2() - 1.0) <= (1e-12 if precision == "fp64" else 1e-6)
        inst.close()


def test_wall_extension_set_psi_round_trip(qsg, ctx, oracle):
    """qsg_set_psi on a wall extension takes n sites and rebuilds the odd
    extension: stepping from it equals stepping a fresh instance."""
    n = 16384
    psi0, V, dx = wall_packet(n)
    a = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.2, order=4, precision="fp64",
                               boundary=qsg.BoundaryCondition.InfiniteWall)
    a.step(5)
    mid = a.get_psi()
    b = qsg.Instance.create_1d(ctx, mid, V, dx, 0.2, order=4, precision="fp64",
                               boundary=qsg.BoundaryCondition.InfiniteWall)
    a.set_psi(mid)
    a.step(4)
    b.step(4)
    assert np.array_equal(a.get_psi(), b.get_psi())
    ref = oracle.evolve1d(oracle.evolve1d(psi0, V, dx, 0.2, 5, order=4, wall=True), V, dx, 0.2, 4, order=4, wall=True)
    assert rel_l2(b.get_psi(), ref) <= PLAIN_TOL
    a.close()
    b.close()


@pytest.mark.parametrize("n", [3, 5, 8, 32, 100, 1000, 1234, 2047, 4095])
@pytest.mark.parametrize("order", [2, 4])
def test_lengths_not_powers_of_two_vs_oracle(qsg, ctx, oracle, n, order):
    """Periodic 1D grids of any length (the reference transforms them with KISS's
    mixed radix, src/kissfft.hh:26-45; 1234 is its FFT test's length,
    applications/QuSimTest/TestFFT.cpp:89-99): Bluestein transforms of a
    power-of-two length (also for the powers of two 8 and 32, below the one-CTA
    kernels' 64).  Against the oracle (bit-exact with the reference's
    KISS evolution): complex128 <= 1e-12 with Norm2, KinEn and PotEn to 1e-11,
    complex64 <= 1e-5."""
    L = max(10.0, 0.1 * n)
    psi0, V, dx = gauss_packet_1d(n, -L, L, 1.5, -0.2 * L, max(0.08 * L, 2 * 2 * L / n), barrier=0.7)
    ref = oracle.evolve1d(psi0, V, dx, 0.02, 25, order=order)
    for precision, tol in (("fp64", PLAIN_TOL), ("mixed", MIXED_TOL)):
        inst = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.02, order=order, precision=precision)
        inst.step(20)
        inst.step(5)
        got = inst.get_psi()
        assert rel_l2(got, ref) <= tol, (precision, rel_l2(got, ref))
        if precision == "fp64":
            kin, pot = inst.energies()
            kr = oracle.kinen1d(ref, dx)
            assert abs(kin - kr) <= 1e-11 * max(1.0, abs(kr))
            assert abs(pot - oracle.poten(ref, V, dx)) <= 1e-11
            assert abs(inst.norm2() - oracle.norm2(ref, dx)) <= 1e-12
            assert abs(inst.step_norm2() - oracle.norm2(ref, dx)) <= 1e-12
        inst.close()


def test_length_not_power_of_two_renormalising_and_batches(qsg, ctx, oracle):
    """Renormalising calls on a Bluestein instance; a batch refuses such lengths."""
    n = 1234
    psi0, V, dx = gauss_packet_1d(n, -60, 60, 1.0, -10, 3.0)
    inst = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.02 - 0.004j, order=4, precision="fp64")
    inst.step(7, renormalize=True)
    ref = oracle.evolve1d(psi0, V, dx, 0.02 - 0.004j, 7, order=4, renormalize=True)
    assert rel_l2(inst.get_psi(), ref) <= PLAIN_TOL
    assert abs(inst.norm2() - 1.0) <= 1e-13
    inst.close()
    with pytest.raises(qsg.QsgError) as e:
        qsg.Batch(ctx, [psi0, psi0[:1024]], [V, V[:1024]], [dx, dx], [0.02, 0.02])
    assert e.value.code == 5


@pytest.mark.parametrize("nx,ny", [(123, 234), (100, 128), (64, 96), (5, 3), (2048, 100), (96, 4095)])
@pytest.mark.parametrize("order", [2, 4])
def test_2d_grids_not_powers_of_two_vs_oracle(qsg, ctx, oracle, nx, ny, order):
    """SplittingMethod2D on grids with a side that is not a power of two (the
    reference's own FFT test uses 123 x 234, applications/QuSimTest/TestFFT.cpp:
    89-99) and on power-of-two sides without a compiled plan (64): Bluestein
    row and column passes in natural layout.  Against the oracle: complex128
    <= 1e-12 with Norm2, KinEn and PotEn to 1e-11; complex64 <= 1e-5 (sides up
    to 4096)."""
    hx, hy = 0.1 * max(nx, 20), 0.1 * max(ny, 20)
    psi0, dx, dy = gauss_packet_2d(nx, ny, -hx, hx, -hy, hy, kx=1.0, ky=0.5, xc=-0.2 * hx, yc=0.1 * hy,
                                   s=max(0.1 * min(hx, hy), 2 * max(2 * hx / nx, 2 * hy / ny)))
    V = gaussian_bumps_2d(nx, ny, -hx, hx, -hy, hy, nbumps=6, seed=4, spread=0.5 * min(hx, hy))
    ref = oracle.evolve2d(psi0, V, dx, dy, 0.02, 6, order=order)
    for precision, tol in (("fp64", PLAIN_TOL), ("mixed", MIXED_TOL)):
        inst = qsg.Instance.create_2d(ctx, psi0, V, dx, dy, 0.02, order=order, precision=precision)
        inst.step(4)
        inst.step(2)
        got = inst.get_psi()
        assert rel_l2(got, ref) <= tol, (precision, rel_l2(got, ref))
        if precision == "fp64":
            kin, pot = inst.energies()
            kr = oracle.kinen2d(ref, dx, dy)
            assert abs(kin - kr) <= 1e-11 * max(1.0, abs(kr))
            assert abs(pot - oracle.poten(ref, V, dx * dy)) <= 1e-11
            assert abs(inst.norm2() - oracle.norm2(ref, dx * dy)) <= 1e-12
        inst.close()


def test_2d_grid_not_power_of_two_renormalising(qsg, ctx, oracle):
    nx, ny = 123, 234
    psi0, dx, dy = gauss_packet_2d(nx, ny, -12, 12, -20, 20, 1.0, 0.0, -3.0, 0.0, 2.0)
    V = gaussian_bumps_2d(nx, ny, -12, 12, -20, 20, nbumps=6, seed=2, spread=6.0)
    inst = qsg.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01 - 0.003j, order=4, precision="fp64")
    inst.step(5, renormalize=True)
    ref = oracle.evolve2d(psi0, V, dx, dy, 0.01 - 0.003j, 5, order=4, renormalize=True)
    assert rel_l2(inst.get_psi(), ref) <= PLAIN_TOL
    assert abs(inst.norm2() - 1.0) <= 1e-13
    with pytest.raises(qsg.QsgError) as e:
        inst.set_plan((2, 8, 256, 8, 4, 0))
    assert e.value.code == 5
    inst.close()
