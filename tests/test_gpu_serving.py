"""Serving (continuous batching): results equal solo runs, the HBM budget
holds under load, bad requests are refused.  GPU."""
import numpy as np
import pytest

from tests.workloads import gauss_packet_1d, gauss_packet_2d, gaussian_bumps_2d

pytestmark = pytest.mark.gpu


def make_requests(seed=3):
    rng = np.random.default_rng(seed)
    reqs = []
    for n, steps, order in [(1024, 300, 2), (1024, 300, 2), (8192, 120, 4), (2048, 77, 2), (65536, 9, 2),
                            (16384, 13, 4), (512, 1000, 4)]:
        box = 0.05 * n
        p, v, dx = gauss_packet_1d(n, -box, box, rng.uniform(0.5, 3), -0.25 * box, rng.uniform(2, 20), barrier=0.8)
        reqs.append(dict(psi0=p, V=v, dx=dx, dt=0.01, nsteps=steps, order=order))
    for side, steps, order in [(256, 40, 4), (512, 7, 2), (256, 25, 2)]:
        h = 0.05 * side
        p, dx, dy = gauss_packet_2d(side, side, -h, h, -h, h, 1.0, 0.3, -0.2 * h, 0.0, 0.08 * h)
        v = gaussian_bumps_2d(side, side, -h, h, -h, h, nbumps=8, seed=int(rng.integers(100)), spread=0.5 * h)
        reqs.append(dict(psi0=p, V=v, dx=dx, dy=dy, dt=0.01, nsteps=steps, order=order))
    return reqs


def solo(q, ctx, r, precision):
    if r["psi0"].ndim == 1:
        inst = q.Instance.create_1d(ctx, r["psi0"], r["V"], r["dx"], r["dt"], order=r["order"], precision=precision)
    else:
        inst = q.Instance.create_2d(ctx, r["psi0"], r["V"], r["dx"], r["dy"], r["dt"], order=r["order"],
                                    precision=precision)
    inst.step(r["nsteps"])
    out = inst.get_psi()
    inst.close()
    return out


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_served_results_equal_solo_runs(precision):
    import qusim_gb300 as q
    reqs = make_requests()
    srv = q.Server(0, max_running=64)
    ids = [srv.submit(r["psi0"], r["V"], r["dx"], r["dt"], r["nsteps"], order=r["order"], precision=precision,
                      dy=r.get("dy")) for r in reqs]
    results = []
    for i in ids:
        assert srv.wait(i, 300) == q.Server.DONE
        results.append(srv.take(i))
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    ctx = q.Context(0)
    for r, (psi, lat) in zip(reqs, results):
        assert lat > 0
        # alone, in one qsg_step call: bitwise the same as served in chunks and in the mix
        assert np.array_equal(psi, solo(q, ctx, r, precision))


def test_budget_holds_under_load():
    import qusim_gb300 as q
    reqs = make_requests(seed=5) * 3
    budget = 96 << 20
    srv = q.Server(0, hbm_budget=budget)
    ids = [srv.submit(r["psi0"], r["V"], r["dx"], r["dt"], r["nsteps"], order=r["order"], dy=r.get("dy"))
           for r in reqs]
    for i in ids:
        assert srv.wait(i, 300) == q.Server.DONE
        srv.take(i)
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs)
    assert 0 < st["peak_device_bytes"] <= budget


def test_bad_requests_are_refused():
    import qusim_gb300 as q
    srv = q.Server(0, hbm_budget=32 << 20)
    big = np.zeros((2048, 2048), np.complex128)
    with pytest.raises(q.QsgError) as e:
        srv.submit(big, big.real, 0.1, 0.01, 10, dy=0.1)
    assert e.value.code == 2
    odd = np.ones(1000, np.complex128)
    rid = srv.submit(odd, odd.real, 0.1, 0.01, 10)
    assert srv.wait(rid, 60) == q.Server.FAILED
    with pytest.raises(q.QsgError) as e:
        srv.take(rid)
    assert e.value.code == 5
    ok = np.ones(1024, np.complex128)
    rid = srv.submit(ok, ok.real, 0.1, 0.01, 10)
    assert srv.wait(rid, 60) == q.Server.DONE
    srv.close()
