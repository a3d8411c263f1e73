"""psi0 and V from a packet-plus-bumps spec, sampled on the device.

The reference samples its psi / V functors on the host at x0 + i*dx
(src/EvolverImpl1D.cpp:33-81, src/EvolverImpl2D.cpp:39-98); the spec entry
points sample the same formula on the device in FP64.  Checked against the
host-sampled arrays of tests/workloads.py, against array-created instances,
and through the server.
"""
import numpy as np
import pytest

from tests.workloads import gauss_packet_1d, gauss_packet_2d, gaussian_bumps_2d, grid

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.fixture(scope="module")
def q():
    import qusim_gb300 as m
    m.load()
    return m


@pytest.fixture(scope="module")
def ctx(q):
    return q.Context(0)


def bumps_2d(nbumps, seed, spread):
    """The bumps of gaussian_bumps_2d(..., nbumps, seed, spread) as spec rows (h, cx, cy, w)."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-spread, spread, size=(nbumps, 2))
    h = rng.uniform(-1.0, 1.0, size=nbumps)
    w = rng.uniform(1.0, 5.0, size=nbumps)
    return [(h[i], c[i, 0], c[i, 1], w[i]) for i in range(nbumps)]


def test_spec_1d_samples_and_evolves_like_host_arrays(q, ctx):
    n, x0, x1 = 4096, -200.0, 200.0
    psi0, V, dx = gauss_packet_1d(n, x0, x1, 1.0, -50.0, 10.0, barrier=0.5)
    spec = q.Spec.make(x0=x0, s=10.0, kx=1.0, cx=-50.0, bumps=[(0.5, 0.0, 0.0, 1.0)])
    for precision, tol in (("fp64", 1e-12), ("mixed", 1e-6)):
        a = q.Instance.create_1d_spec(ctx, spec, n, dx, 0.05, order=2, precision=precision)
        b = q.Instance.create_1d(ctx, psi0, V, dx, 0.05, order=2, precision=precision)
        if precision == "fp64":
            assert rel_l2(a.get_psi(), psi0) <= 1e-14
        a.step(50)
        b.step(50)
        assert rel_l2(a.get_psi(), b.get_psi()) <= tol, precision
        _, pa = a.energies()
        _, pb = b.energies()
        assert abs(pa - pb) <= tol * max(1.0, abs(pb)), precision


def test_spec_2d_samples_and_evolves_like_host_arrays(q, ctx):
    nx, ny, h = 512, 256, 40.0
    psi0, dx, dy = gauss_packet_2d(nx, ny, -h, h, -h, h, 1.5, 0.5, -10.0, 3.0, 4.0)
    V = gaussian_bumps_2d(nx, ny, -h, h, -h, h, nbumps=8, seed=5, spread=20.0)
    spec = q.Spec.make(x0=-h, y0=-h, s=4.0, kx=1.5, ky=0.5, cx=-10.0, cy=3.0, bumps=bumps_2d(8, 5, 20.0))
    a = q.Instance.create_2d_spec(ctx, spec, nx, ny, dx, dy, 0.01, order=4, precision="fp64")
    b = q.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=4, precision="fp64")
    assert rel_l2(a.get_psi(), psi0) <= 1e-14
    a.step(10)
    b.step(10)
    assert rel_l2(a.get_psi(), b.get_psi()) <= 1e-12
    _, pa = a.energies()
    _, pb = b.energies()
    assert abs(pa - pb) <= 1e-12 * max(1.0, abs(pb))


def test_spec_requests_served_equal_solo(q):
    """Served results of spec requests equal the same specs evolved alone."""
    srv = q.Server(0, hbm_budget=2 << 30)
    ctx = q.Context(0)
    rng = np.random.default_rng(11)
    reqs = []
    for k in range(6):
        if k % 2 == 0:
            n = int(2 ** rng.integers(10, 15))
            half = 0.05 * n
            _, dx = grid(n, -half, half)
            spec = q.Spec.make(x0=-half, s=rng.uniform(2, 20), kx=rng.uniform(0.5, 3), cx=-0.25 * half,
                               bumps=[(rng.uniform(-1, 1), rng.uniform(-half, half), 0.0, rng.uniform(1, 5))
                                      for _ in range(8)])
            reqs.append((srv.submit_spec(spec, (n,), dx, 0.01, 37, order=2), ("1d", spec, n, dx)))
        else:
            side = int(2 ** rng.integers(8, 10))
            h = 0.05 * side
            _, dx = grid(side, -h, h)
            spec = q.Spec.make(x0=-h, y0=-h, s=rng.uniform(2, 8), kx=rng.uniform(0.5, 3), cx=-0.25 * h,
                               bumps=bumps_2d(8, int(rng.integers(1 << 20)), 0.8 * h))
            reqs.append((srv.submit_spec(spec, (side, side), dx, 0.01, 21, order=4), ("2d", spec, side, dx)))
    for rid, (kind, spec, n, dx) in reqs:
        assert srv.wait(rid) == 2
        got = srv.take(rid)[0]
        if kind == "1d":
            solo = q.Instance.create_1d_spec(ctx, spec, n, dx, 0.01, order=2, precision="mixed")
            solo.step(37)
        else:
            solo = q.Instance.create_2d_spec(ctx, spec, n, n, dx, dx, 0.01, order=4, precision="mixed")
            solo.step(21)
        assert np.array_equal(got, solo.get_psi()), kind
        solo.close()
    srv.close()


def test_spec_arguments_are_checked(q, ctx):
    bad = q.Spec.make(x0=0.0, s=0.0)
    with pytest.raises(q.QsgError) as e:
        q.Instance.create_1d_spec(ctx, bad, 1024, 0.1, 0.01)
    assert e.value.code == 1
    with pytest.raises(ValueError):
        q.Spec.make(x0=0.0, s=1.0, bumps=[(1, 0, 0, 1)] * 33)
    worse = q.Spec.make(x0=0.0, s=1.0, bumps=[(1.0, 0.0, 0.0, -1.0)])
    with pytest.raises(q.QsgError) as e:
        q.Instance.create_2d_spec(ctx, worse, 256, 256, 0.1, 0.1, 0.01)
    assert e.value.code == 1
