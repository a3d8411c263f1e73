"""The deferred closing row pass of a 2D qsg_step call.

Stepping in many small calls must give the same state as one long call (the
next call merges the deferred pass into its first one), every read settles
the state first, and qsg_step_norm2 -- the norm the step's last column pass
summed -- equals qsg_norm2 (1e-12 in complex128, rounding level in complex64).
"""
import numpy as np
import pytest

from tests.workloads import gauss_packet_2d, gaussian_bumps_2d

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def q():
    import qusim_gb300 as m
    m.load()
    return m


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("order", [2, 4])
def test_small_calls_equal_one_call(q, precision, order):
    ctx = q.Context(0)
    n = 512
    psi0, dx, dy = gauss_packet_2d(n, n, -40, 40, -40, 40, 1.5, 0.3, -10.0, 0.0, 4.0)
    V = gaussian_bumps_2d(n, n, -40, 40, -40, 40, nbumps=8, seed=4, spread=20.0)
    a = q.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=order, precision=precision)
    b = q.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=order, precision=precision)
    a.step(12)
    for _ in range(12):
        b.step(1)
        nb = b.step_norm2()
        assert abs(nb - 1.0) < (1e-10 if precision == "fp64" else 1e-4)
    assert np.array_equal(a.get_psi(), b.get_psi())
    # a read in the middle (settles), then more small steps
    a.step(5)
    b.step(2)
    b.get_psi()
    b.step(3)
    assert np.max(np.abs(a.get_psi() - b.get_psi())) <= (1e-13 if precision == "fp64" else 1e-5)
    a.close()
    b.close()
    ctx.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_step_norm2_equals_norm2(q, precision):
    ctx = q.Context(0)
    n = 1024
    psi0, dx, dy = gauss_packet_2d(n, n, -60, 60, -60, 60, 1.0, 0.0, -20.0, 0.0, 6.0)
    V = gaussian_bumps_2d(n, n, -60, 60, -60, 60, nbumps=8, seed=5, spread=30.0)
    a = q.Instance.create_2d(ctx, psi0 * 1.3, V, dx, dy, 0.01, order=4, precision=precision)
    a.step(7)
    fast = a.step_norm2()
    exact = a.norm2()
    assert abs(fast - exact) <= (1e-12 if precision == "fp64" else 1e-6) * exact
    assert abs(exact - 1.69) <= (1e-10 if precision == "fp64" else 1e-4)
    a.close()
    ctx.close()


def test_plan_change_and_energies_settle(q):
    ctx = q.Context(0)
    n = 512
    psi0, dx, dy = gauss_packet_2d(n, n, -40, 40, -40, 40, 1.5, 0.0, -10.0, 0.0, 4.0)
    V = gaussian_bumps_2d(n, n, -40, 40, -40, 40, nbumps=8, seed=6, spread=20.0)
    a = q.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=4, precision="fp64")
    b = q.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=4, precision="fp64")
    a.step(4)
    b.step(4)
    ka, pa = a.energies()
    plans = b.candidate_plans()
    other = [p for p in plans if p.as_tuple() != b.plan().as_tuple()][0]
    b.set_plan(other)       # settles under the old plan first
    kb, pb = b.energies()
    assert abs(ka - kb) <= 1e-12 * abs(ka) and abs(pa - pb) <= 1e-12 * abs(pa)
    a.step(3)
    b.step(3)
    assert np.max(np.abs(a.get_psi() - b.get_psi())) <= 1e-12
    a.close()
    b.close()
    ctx.close()
