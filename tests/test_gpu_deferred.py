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


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_plan_change_and_energies_settle(q, precision):
    """A plan change settles the state under the old plan (in the complex64
    momentum form also the stored momentum-space state and its split-k copy)."""
    ctx = q.Context(0)
    n = 512
    psi0, dx, dy = gauss_packet_2d(n, n, -40, 40, -40, 40, 1.5, 0.0, -10.0, 0.0, 4.0)
    V = gaussian_bumps_2d(n, n, -40, 40, -40, 40, nbumps=8, seed=6, spread=20.0)
    a = q.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=4, precision=precision)
    b = q.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=4, precision=precision)
    a.step(4)
    b.step(4)
    ka, pa = a.energies()
    plans = b.candidate_plans()
    # a plan with another x split, so that the split-k layouts differ
    other = [p for p in plans if p.as_tuple()[0] != b.plan().as_tuple()[0]][0]
    b.set_plan(other)       # settles under the old plan first
    kb, pb = b.energies()
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert abs(ka - kb) <= tol * abs(ka) and abs(pa - pb) <= tol * abs(pa)
    a.step(3)
    b.step(3)
    assert np.max(np.abs(a.get_psi() - b.get_psi())) <= (1e-12 if precision == "fp64" else 1e-5)
    a.close()
    b.close()
    ctx.close()


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_posted_step_norms(q, dim):
    """post / get returns each step's norm while later steps run; equals step_norm2."""
    ctx = q.Context(0)
    if dim == 2:
        psi0, dx, dy = gauss_packet_2d(256, 256, -30, 30, -30, 30, 1.0, 0.0, -5.0, 0.0, 3.0)
        V = gaussian_bumps_2d(256, 256, -30, 30, -30, 30, nbumps=4, seed=7, spread=10.0)
        a = q.Instance.create_2d(ctx, psi0 * 0.9, V, dx, dy, 0.01, order=4, precision="fp64")
    elif dim == 1:
        from tests.workloads import gauss_packet_1d
        psi0, V, dx = gauss_packet_1d(4096, -200.0, 200.0, 1.0, -50.0, 10.0)
        a = q.Instance.create_1d(ctx, psi0 * 0.9, V, dx, 0.05, order=2, precision="fp64")
    else:
        rng = np.random.default_rng(3)
        psi0 = (rng.normal(size=(16, 16, 32)) + 1j * rng.normal(size=(16, 16, 32))) * 0.1
        V = rng.uniform(0, 1, size=psi0.shape)
        a = q.Instance.create_3d(ctx, psi0, V, 0.5, 0.5, 0.5, 0.01, order=4, precision="fp64")
    want = a.norm2()
    tickets, got = [], []
    for _ in range(5):
        a.step(1)
        tickets.append(a.post_step_norm2())
        if len(tickets) > 1:
            got.append(a.get_step_norm2(tickets[-2]))
    got.append(a.get_step_norm2(tickets[-1]))
    assert len(got) == 5
    for g in got:
        assert abs(g - want) <= 1e-12 * want
    assert abs(a.step_norm2() - got[-1]) <= 1e-13 * want
    with pytest.raises(q.QsgError) as e:
        a.get_step_norm2(tickets[-1] + 1)
    assert e.value.code == 1
    for _ in range(64):
        a.post_step_norm2()
    with pytest.raises(q.QsgError) as e:
        a.get_step_norm2(tickets[0])
    assert e.value.code == 6
    a.close()
    ctx.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_1d_step_norm2_from_the_step_kernel(q, precision):
    """1D one-CTA instances: qsg_step_norm2 is the kernel's own sum of the state
    it ended in; after renormalisation or a new state it is summed afresh."""
    from tests.workloads import gauss_packet_1d
    ctx = q.Context(0)
    psi0, V, dx = gauss_packet_1d(2048, -100.0, 100.0, 1.0, -30.0, 8.0)
    a = q.Instance.create_1d(ctx, psi0 * 1.2, V, dx, 0.02, order=4, precision=precision)
    tol = 1e-12 if precision == "fp64" else 1e-7
    a.step(3)
    assert abs(a.step_norm2() - a.norm2()) <= tol * a.norm2()
    a.step(2, renormalize=True)
    assert abs(a.step_norm2() - 1.0) <= tol
    a.set_psi(psi0 * 0.5)
    assert abs(a.step_norm2() - a.norm2()) <= 1e-13 * a.norm2()
    a.step(1)
    t = a.post_step_norm2()
    assert abs(a.get_step_norm2(t) - a.norm2()) <= tol * a.norm2()
    a.close()
    ctx.close()
