"""Born-series scattering solvers on the GPU against the oracle and the
reference's golden vectors (QuPerturbation1D / QuPerturbation2D,
src/Perturbation1DImpl.cpp, src/Perturbation2DImpl.cpp, src/Perburbation.h).

complex128: relative L2 <= 1e-12 on the scattered wave, 1e-12 on R, T, the
delta-psi norm and the cross sections.  complex64 ("mixed"): the FP32
transforms and updates carry ~1e-7 relative rounding per update; the bar is
relative L2 <= 2e-5 on the wave and 2e-5 (relative) on R, T and cross sections.
"""
import numpy as np
import pytest

from tests.conftest import load_golden
from tests.workloads import (BORN_1D_CASES, BORN_2D_CASES, BORN_XSEC_TOTAL, born_potential_1d,
                             born_potential_2d, xsec_cosines)

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 2e-5


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.fixture(scope="module")
def q():
    import qusim_gb300 as m
    m.load()
    return m


def opts_for(q, order, pre, precer, slow, precision="fp64"):
    o = q.Options().Gb300().Order(order).Slow(slow).Precision(precision)
    if pre:
        o.Preconditional(True)
        o.SetString("preconditioner", ("BornIndentity", "Vellekoop", "Hao1", "Hao2")[precer])
    return o


def run_1d(q, V, x0, x1, en, eps, direction, order, pre, precer, slow, computes, precision="fp64"):
    per = q.QuPerturbation1D()
    per.init(V, x0, x1, V.size, en, eps, direction, q.SolverMethod.BornSerise, 1.0, 1.0,
             opts_for(q, order, pre, precer, slow, precision))
    for _ in range(computes):
        per.Compute()
    return per


POW2_1D = [c for c in BORN_1D_CASES if (c[1] & (c[1] - 1)) == 0]


@pytest.mark.parametrize("case", POW2_1D, ids=[c[0] for c in POW2_1D])
def test_born1d_matches_reference_golden(q, case):
    name, n, x0, x1, v0, en, eps, direction, order, pre, precer, slow, computes = case
    g = load_golden(name)
    per = run_1d(q, g["V"], x0, x1, en, eps, direction, order, pre, precer, slow, computes)
    # psi0 and the absorbing layer come from the host's libm (exp): equal to
    # the last bit on the machine that made the fixtures, within it elsewhere
    assert np.max(np.abs(per.GetPsi0() - g["psi0"])) <= 1e-15
    assert np.max(np.abs(per.GetV() - g["v"])) <= 1e-15
    assert abs(per.GetEpsilon() - g["epsilon"]) <= 1e-15 * abs(g["epsilon"])
    assert rel_l2(per.GetPsi(), g["dpsi"]) <= TOL64
    assert abs(per.GetR() - g["R"]) <= TOL64 and abs(per.GetT() - g["T"]) <= TOL64


@pytest.mark.parametrize("case", BORN_2D_CASES, ids=[c[0] for c in BORN_2D_CASES])
def test_born2d_matches_reference_golden(q, case):
    name, nx, ny, hx, hy, en, eps, dirx, diry, order, pre, precer, slow, computes = case
    g = load_golden(name)
    V, _, _ = born_potential_2d(nx, ny, -hx, hx, -hy, hy)
    per = q.QuPerturbation2D()
    per.init(V, -hx, hx, nx, -hy, hy, ny, en, eps, dirx, diry, q.SolverMethod.BornSerise, 1.0, 1.0,
             opts_for(q, order, pre, precer, slow))
    for _ in range(computes):
        per.Compute()
    assert abs(per.GetPsi0().sum() - g["psi0_sum"]) <= 1e-12 * nx * ny
    assert abs(per.GetV().sum() - g["v_sum"]) <= 1e-13 * abs(g["v_sum"])
    assert abs(per.GetEpsilon() - g["epsilon"]) <= 1e-14 * abs(g["epsilon"])
    assert rel_l2(per.GetPsi(), g["dpsi"]) <= TOL64
    assert abs(per.GetDeltaPsiNorm() - g["delta_norm"]) <= TOL64 * g["delta_norm"]
    xs = per.ComputeXSections(xsec_cosines())
    assert np.allclose(xs, g["xsec"], rtol=1e-11, atol=0)
    assert abs(per.ComputeTotalXSection(BORN_XSEC_TOTAL) - g["total"]) <= 1e-11 * g["total"]


# four-step sizes (complex128 from 8192, complex64 from 16384) and the
# resident ones, every post-update kind
CASES_1D_SIZES = [
    # n, half-box, v0, en, eps, order, pre, precer, slow
    (128, 12.0, 0.5, 2.0, 0.05, 3, False, 1, 1.0),
    (4096, 150.0, 0.5, 0.5, 0.0, 6, True, 1, 1.0),
    (8192, 300.0, 1.0, 0.5, 0.02, 4, False, 1, 1.0),
    (16384, 400.0, 0.5, 0.5, 0.0, 5, True, 2, 0.6),
    (65536, 1000.0, 0.5, 0.5, 0.0, 4, True, 3, 0.7),
    (262144, 4000.0, 0.5, 0.5, 0.0, 3, True, 0, 0.5),
    (1 << 20, 20000.0, 0.5, 0.5, 0.0, 2, True, 0, 1.0),
]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", CASES_1D_SIZES, ids=[str(c[0]) for c in CASES_1D_SIZES])
def test_born1d_sizes_against_oracle(q, oracle, case, precision):
    n, h, v0, en, eps, order, pre, precer, slow = case
    V, _ = born_potential_1d(n, -h, h, v0)
    ref = oracle.born1d(V, -h, h, en, eps, order=order, preconditional=pre, preconditioner=precer,
                        slow=slow, computes=2)
    per = run_1d(q, V, -h, h, en, eps, 1.0, order, pre, precer, slow, 2, precision)
    tol = TOL64 if precision == "fp64" else TOL32
    assert rel_l2(per.GetPsi(), ref["dpsi"]) <= tol
    assert abs(per.GetR() - ref["R"]) <= tol * max(1.0, ref["R"])
    assert abs(per.GetT() - ref["T"]) <= tol * max(1.0, ref["T"])


CASES_2D_SIZES = [
    # nx, ny, hx, hy, en, eps, dir, order, pre, precer, slow
    (256, 512, 60.0, 90.0, 2.0, 0.0, (1.0, 0.3), 4, True, 1, 1.0),
    (1024, 256, 120.0, 60.0, 2.0, 0.0, (0.0, 1.0), 3, True, 3, 0.5),
    (512, 512, 80.0, 80.0, 0.5, 0.05, (1.0, 0.0), 3, False, 1, 1.0),
    (2048, 128, 200.0, 40.0, 2.0, 0.0, (1.0, -1.0), 2, True, 0, 0.8),
    (128, 4096, 40.0, 300.0, 2.0, 0.0, (1.0, 1.0), 2, True, 2, 1.0),
]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", CASES_2D_SIZES, ids=[f"{c[0]}x{c[1]}" for c in CASES_2D_SIZES])
def test_born2d_sizes_against_oracle(q, oracle, case, precision):
    nx, ny, hx, hy, en, eps, (dx_, dy_), order, pre, precer, slow = case
    V, _, _ = born_potential_2d(nx, ny, -hx, hx, -hy, hy)
    cs = xsec_cosines(12)
    ref = oracle.born2d(V, -hx, hx, -hy, hy, en, eps, dirx=dx_, diry=dy_, order=order, preconditional=pre,
                        preconditioner=precer, slow=slow, computes=2, cosxy=cs)
    per = q.QuPerturbation2D()
    per.init(V, -hx, hx, nx, -hy, hy, ny, en, eps, dx_, dy_, q.SolverMethod.BornSerise, 1.0, 1.0,
             opts_for(q, order, pre, precer, slow, precision))
    per.Compute()
    per.Compute()
    tol = TOL64 if precision == "fp64" else TOL32
    assert rel_l2(per.GetPsi(), ref["dpsi"]) <= tol
    assert abs(per.GetDeltaPsiNorm() - ref["delta_norm"]) <= tol * ref["delta_norm"] * 10
    xs = per.ComputeXSections(cs)
    assert np.allclose(xs, ref["xsec"], rtol=10 * tol, atol=1e-14 * max(ref["xsec"]))


def test_born_python_functor_equals_array(q):
    """init with a callable V(x) samples the same grid as an array."""
    n, h = 2048, 100.0
    V, _ = born_potential_1d(n, -h, h, 0.5)
    a = run_1d(q, V, -h, h, 0.5, 0.51, 1.0, 5, True, 1, 1.0, 1)
    b = q.QuPerturbation1D()
    b.init(lambda x: 0.5 * np.exp(-x * x), -h, h, n, 0.5, 0.51, 1.0, q.SolverMethod.BornSerise, 1.0, 1.0,
           q.Options().Gb300().Order(5).Preconditional(True))
    b.Compute()
    assert np.array_equal(a.GetPsi(), b.GetPsi())
    assert a.GetR() == b.GetR() and a.GetT() == b.GetT()


def test_born_errors(q):
    V, _ = born_potential_1d(1000, -100.0, 100.0, 0.5)
    with pytest.raises(q.QsgError) as e:  # not a power of two
        run_1d(q, V, -100.0, 100.0, 0.5, 0.1, 1.0, 1, False, 1, 1.0, 1)
    assert e.value.code == 5
    V, _ = born_potential_1d(256, -10.0, 10.0, 0.5)
    with pytest.raises(q.QsgError) as e:  # box below 24 wavelengths
        run_1d(q, V, -10.0, 10.0, 0.5, 0.0, 1.0, 1, True, 1, 1.0, 1)
    assert e.value.code == 1
    with pytest.raises(q.QsgError) as e:
        run_1d(q, V, -10.0, 10.0, 0.5, 0.1, 1.0, 0, False, 1, 1.0, 1)
    assert e.value.code == 1
    per = q.QuPerturbation1D()
    per.init(V, -10.0, 10.0, 256, 0.5, 0.1, 1.0, q.SolverMethod.BornSerise, 1.0, 1.0, q.Options().Gb300())
    with pytest.raises(q.QsgError) as e:  # R / T before any Compute
        per.GetR()
    assert e.value.code == 6
