"""Expressions in the language of the reference's calculator (src/Cal.cpp):
the host evaluator of libqsg.so (qsg_expr_eval, behind Calculator /
FunctorWrapper / Functor2DWrapper) against values the reference's own Cal
computed (tests/golden/cal_exprs.npz, tests/golden/make_golden.py).  CPU only:
no CUDA call is made."""
import numpy as np
import pytest

from tests.conftest import load_golden
from tests.workloads import CAL_BAD, CAL_EXPRESSIONS, CAL_POINTS


@pytest.fixture(scope="module")
def q():
    import qusim_gb300 as q
    q.load()
    return q


def test_expressions_match_the_reference_calculator(q):
    g = load_golden("cal_exprs")
    vals = g["values"]
    for i, e in enumerate(CAL_EXPRESSIONS):
        f = q.Functor2DWrapper(e)
        for j, (x, y) in enumerate(CAL_POINTS):
            got, want = f(x, y), vals[i, j]
            assert abs(got - want) <= 1e-14 * max(1.0, abs(want)), (e, x, y, got, want)


def test_bad_expressions_are_refused_like_the_reference(q):
    g = load_golden("cal_exprs")
    assert g["bad_fail"].all()
    for e in CAL_BAD:
        with pytest.raises(q.QsgError) as err:
            c = q.Calculator(e)
            c.SetVaraible("x", 1.0)
            c.SetVaraible("y", 2.0)
            c.Evaluate()
        assert err.value.code == 1, e


def test_calculator_variables_and_functor_wrapper(q):
    c = q.Calculator("a*x + I")
    c.SetVaraible("a", 2.0)
    c.SetVaraible("x", 1.5 + 0.5j)
    assert c.Evaluate() == 2.0 * (1.5 + 0.5j) + 1j
    assert c.GetVaraible("a") == 2.0
    f = q.FunctorWrapper("gauss(x,-20,5)*exp(I*x)")
    x = -18.0
    want = np.exp(-0.5 * ((x + 20) / 5) ** 2) / (np.sqrt(2 * np.pi) * 5) * np.exp(1j * x)
    assert abs(f(x) - want) < 1e-16
    # "==" and sign parse here (the reference's parser cannot accept either)
    assert q.FunctorWrapper("x == 1")(1.0) == 1.0
    assert q.FunctorWrapper("sign(x)")(-2.0) == -1.0
