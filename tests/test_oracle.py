"""The oracle (C restatement) against the reference's golden vectors and known answers.

CPU only.  The fixtures in tests/golden/ were produced by the reference's own
sources compiled as they lie (tests/golden/make_golden.py); the oracle must
reproduce them to the last bit (same algorithm, same operation order): psi is
compared with np.array_equal and Norm2, KinEn and PotEn with ==.
"""
import numpy as np
import pytest

from tests.conftest import load_golden

EVOLVE_1D = ["evolve1d_n4096_o2_2000", "evolve1d_n4096_o4_200", "evolve1d_n256_o2_b7x3_fnes",
             "evolve1d_n1024_o4_imag", "evolve1d_n512_o2_wall", "evolve1d_n1000_o2",
             "evolve1d_n1024_o2_hbar07_m2", "evolve1d_n512_o4_wall_hbar07_m2", "evolve1d_n600_o4_wall",
             "evolve1d_n5000_o4", "evolve1d_n4099_o2_b5x2_fnes", "evolve1d_n3000_o4_wall"]
EVOLVE_2D = ["evolve2d_128x256_o2_50", "evolve2d_256x128_o4_20", "evolve2d_128x128_o4_b5x2_fnes",
             "evolve2d_128x256_o4_hbar07_m2", "evolve2d_45x70_o2_30",
             "evolve2d_96x50_o4_10"]


def mass_hbar(g):
    """(mass, hbar) of a fixture; 1, 1 where it stores none."""
    return float(g.get("mass", 1.0)), float(g.get("hbar", 1.0))


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.mark.parametrize("n", [1234, 4096])
def test_fft1d_ramp_matches_reference(oracle, n):
    g = load_golden(f"fft1d_ramp_{n}")
    x = np.arange(n, dtype=np.complex128)
    assert np.array_equal(oracle.fft1d(x), g["fwd"])
    assert np.array_equal(oracle.fft1d(x, inverse=True), g["inv"])
    # applications/QuSimTest/TestFFT.cpp:71-81: round trip, sum |a-b|^2 < 1e-8
    rt = oracle.fft1d(oracle.fft1d(x), inverse=True) / n
    assert np.sum(np.abs(rt - x) ** 2) < 1e-8


@pytest.mark.parametrize("shape", [(123, 234), (64, 128)])
def test_fft2d_ramp_matches_reference(oracle, shape):
    nx, ny = shape
    g = load_golden(f"fft2d_ramp_{nx}x{ny}")
    x = np.arange(nx * ny, dtype=np.complex128).reshape(nx, ny)
    assert np.array_equal(oracle.fft2d(x), g["fwd"])
    assert np.array_equal(oracle.fft2d(x, inverse=True), g["inv"])
    assert rel_l2(oracle.fft2d(x), np.fft.fft2(x)) < 1e-13


@pytest.mark.parametrize("name", EVOLVE_1D)
def test_evolve1d_matches_reference(oracle, name):
    g = load_golden(name)
    n, x0, x1, order, wall, batch, calls, fnes = g["params"]
    n, order, batch, calls = int(n), int(order), int(batch), int(calls)
    dx = (x1 - x0) / n
    mass, hbar = mass_hbar(g)
    psi = g["psi0"]
    for _ in range(calls):
        psi = oracle.evolve1d(psi, g["V"], dx, complex(g["dt"]), batch, order=order, mass=mass,
                              hbar=hbar, wall=bool(wall), renormalize=bool(fnes))
    assert np.array_equal(psi, g["psi"])
    assert oracle.norm2(psi, dx) == g["norm2"]
    assert oracle.kinen1d(psi, dx, mass=mass, hbar=hbar, wall=bool(wall)) == g["kin"]
    assert oracle.poten(psi, g["V"], dx) == g["pot"]


@pytest.mark.parametrize("name", EVOLVE_2D)
def test_evolve2d_matches_reference(oracle, name):
    g = load_golden(name)
    nx, ny, x0, x1, y0, y1, order, batch, calls, fnes = g["params"]
    nx, ny, order, batch, calls = int(nx), int(ny), int(order), int(batch), int(calls)
    dx, dy = (x1 - x0) / nx, (y1 - y0) / ny
    mass, hbar = mass_hbar(g)
    psi = g["psi0"]
    for _ in range(calls):
        psi = oracle.evolve2d(psi, g["V"], dx, dy, complex(g["dt"]), batch, order=order, mass=mass,
                              hbar=hbar, renormalize=bool(fnes))
    assert np.array_equal(psi, g["psi"])
    assert oracle.norm2(psi, dx * dy) == g["norm2"]
    assert oracle.kinen2d(psi, dx, dy, mass=mass, hbar=hbar) == g["kin"]
    assert oracle.poten(psi, g["V"], dx * dy) == g["pot"]


def test_splitting_constants(oracle):
    c1, c2, d1, d2 = oracle.splitting_constants()
    # SplittingUtils.cpp:3-8; consistency: 2 C1 + 2 C2 = 1, 2 D1 + D2 = 1
    assert abs(2 * c1 + 2 * c2 - 1) < 1e-15
    assert abs(2 * d1 + d2 - 1) < 1e-15
    assert abs(c1 - 0.6756035959798288) < 1e-15


def test_tunnelling_known_answer(oracle):
    """applications/QuEvol1DPrecision/QuSimPrecision.cpp:82,106-120: the
    transmitted probability of gauss(x,-20,5)*exp(I*x) through exp(-x*x) on
    [-100,100) at t=64 is 0.15937744085."""
    ref = (0.1593774409 + 0.1593774408) / 2
    n, dt = 2048, 0.02
    x0, x1 = -100.0, 100.0
    dx = (x1 - x0) / n
    xs = x0 + dx * np.arange(n)
    psi = np.exp(-0.5 * ((xs + 20) / 5) ** 2) * np.exp(1j * xs)
    psi /= np.sqrt(np.sum(np.abs(psi) ** 2) * dx)
    p = oracle.evolve1d(psi, np.exp(-xs * xs), dx, dt, 3200, order=4)
    assert abs(oracle.norm2_range(p, x0, dx, 0.0, x1) - ref) < 1e-9


def test_group_velocity(oracle):
    """QuSimPrecision.cpp:206-218: a free packet gauss(x,0,5)*exp(I*x) moves at 1."""
    n, dt, x0, x1 = 1024, 0.01, -100.0, 100.0
    dx = (x1 - x0) / n
    xs = x0 + dx * np.arange(n)
    psi = np.exp(-0.5 * (xs / 5) ** 2) * np.exp(1j * xs)
    psi /= np.sqrt(np.sum(np.abs(psi) ** 2) * dx)
    xa = oracle.xavg(psi, x0, dx)
    p = oracle.evolve1d(psi, np.zeros(n), dx, dt, 11, order=2)
    assert abs((oracle.xavg(p, x0, dx) - xa) / (11 * dt) - 1) < 1e-10


# --- Born-series scattering solvers -------------------------------------------

from tests.workloads import (BORN_1D_CASES, BORN_2D_CASES, BORN_XSEC_TOTAL,  # noqa: E402
                             born_potential_1d, born_potential_2d, xsec_cosines)


@pytest.mark.parametrize("case", BORN_1D_CASES, ids=[c[0] for c in BORN_1D_CASES])
def test_born1d_matches_reference(oracle, case):
    """QuPerturbation1D: naive and preconditioned series (each preconditioner),
    several Compute() calls, a left-going wave and a grid that is not a power
    of two."""
    name, n, x0, x1, v0, en, eps, direction, order, pre, precer, slow, computes = case
    g = load_golden(name)
    V = g["V"]
    r = oracle.born1d(V, x0, x1, en, eps, direction=direction, order=order, preconditional=pre,
                      preconditioner=precer, slow=slow, computes=computes)
    assert np.array_equal(r["psi0"], g["psi0"])
    assert np.array_equal(r["v"], g["v"])
    assert abs(r["epsilon"] - g["epsilon"]) <= 1e-15 * abs(g["epsilon"])
    assert rel_l2(r["dpsi"], g["dpsi"]) <= 1e-14
    assert abs(r["R"] - g["R"]) <= 1e-14 and abs(r["T"] - g["T"]) <= 1e-14


@pytest.mark.parametrize("case", BORN_2D_CASES, ids=[c[0] for c in BORN_2D_CASES])
def test_born2d_matches_reference(oracle, case):
    name, nx, ny, hx, hy, en, eps, dirx, diry, order, pre, precer, slow, computes = case
    g = load_golden(name)
    V, _, _ = born_potential_2d(nx, ny, -hx, hx, -hy, hy)
    r = oracle.born2d(V, -hx, hx, -hy, hy, en, eps, dirx=dirx, diry=diry, order=order,
                      preconditional=pre, preconditioner=precer, slow=slow, computes=computes,
                      cosxy=xsec_cosines(), ntot=BORN_XSEC_TOTAL)
    assert r["psi0"].sum() == g["psi0_sum"] and r["v"].sum() == g["v_sum"]
    assert abs(r["epsilon"] - g["epsilon"]) <= 1e-15 * abs(g["epsilon"])
    assert rel_l2(r["dpsi"], g["dpsi"]) <= 1e-14
    assert abs(r["delta_norm"] - g["delta_norm"]) <= 1e-13 * g["delta_norm"]
    assert np.allclose(r["xsec"], g["xsec"], rtol=1e-13, atol=0)
    assert abs(r["total"] - g["total"]) <= 1e-13 * g["total"]


def test_born_layer_refuses_small_world(oracle):
    """The preconditioned series needs a box of at least 24 wavelengths
    (src/Perturbation1DImpl.cpp:24-27, src/Perturbation2DImpl.cpp:25-31)."""
    V, _ = born_potential_1d(256, -10.0, 10.0, 0.5)
    with pytest.raises(ValueError):
        oracle.born1d(V, -10.0, 10.0, 0.5, 0.0, order=1, preconditional=True)


# --- 3D ------------------------------------------------------------------------

@pytest.mark.parametrize("shape", [(6, 10, 14), (16, 8, 32)])
def test_fft3d_matches_reference(oracle, shape):
    g = load_golden("fft3d_ramp_%dx%dx%d" % shape)
    x = np.arange(int(np.prod(shape)), dtype=np.complex128).reshape(shape) * (1 + 0.5j)
    assert np.array_equal(oracle.fft3d(x), g["fwd"])
    assert np.array_equal(oracle.fft3d(x, inverse=True), g["inv"])


def test_evolve3d_matches_numpy_restatement(oracle):
    """The 3D split-operator step against an independent numpy restatement of
    the same formulas (np.fft.fftn), and its norm conservation.  The reference
    has no 3D evolver to pin against; its transform is pinned above."""
    nx, ny, nz = 16, 12, 20
    dx, dy, dz = 0.5, 0.6, 0.4
    rng = np.random.default_rng(7)
    psi = rng.normal(size=(nx, ny, nz)) + 1j * rng.normal(size=(nx, ny, nz))
    V = rng.uniform(-1, 1, size=(nx, ny, nz))
    dt, steps = 0.01, 5
    got = oracle.evolve3d(psi, V, dx, dy, dz, dt, steps, order=4)
    t = 2 ** (1 / 3)
    c1, c2 = 1 / (2 * (2 - t)), (1 - t) / (2 * (2 - t))
    d1, d2 = 1 / (2 - t), -t / (2 - t)

    def fold(n):
        i = np.arange(n)
        return np.where(i > n // 2, n - i, i).astype(float)

    kk = ((fold(nx) * 2 * np.pi / (dx * nx)) ** 2 / 2)[:, None, None] + \
         ((fold(ny) * 2 * np.pi / (dy * ny)) ** 2 / 2)[None, :, None] + \
         ((fold(nz) * 2 * np.pi / (dz * nz)) ** 2 / 2)[None, None, :]
    p = psi.copy()
    for _ in range(steps):
        for c, d in ((c1, d1), (c2, d2), (c2, d1)):
            p = p * np.exp(-1j * dt * c * V)
            p = np.fft.ifftn(np.fft.fftn(p) * np.exp(-1j * dt * d * kk))
        p = p * np.exp(-1j * dt * c1 * V)
    assert rel_l2(got, p) <= 1e-12
    assert abs(np.sum(np.abs(got) ** 2) / np.sum(np.abs(psi) ** 2) - 1) <= 1e-12
