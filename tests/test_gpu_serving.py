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
    odd = np.ones((4097, 2), np.complex128)  # a 2D side above 4096 that is not a power of two
    rid = srv.submit(odd, odd.real, 0.1, 0.01, 10, dy=0.1)
    assert srv.wait(rid, 60) == q.Server.FAILED
    with pytest.raises(q.QsgError) as e:
        srv.take(rid)
    assert e.value.code == 5
    ok = np.ones(1024, np.complex128)
    rid = srv.submit(ok, ok.real, 0.1, 0.01, 10)
    assert srv.wait(rid, 60) == q.Server.DONE
    srv.close()


@pytest.mark.parametrize("bad", [8, 4])
def test_failed_dispatch_fails_only_its_request(monkeypatch, bad):
    """A dispatch that fails ends its request FAILED with the failure's status
    and message; the other requests finish DONE, bitwise equal to solo runs.
    The failure is injected on the host (QSG_SERVER_FAIL_REQUEST): request 8
    is the first 2D request (a chunked, stepped dispatch), request 4 the only
    2048-site 1D request (a batched resident launch with one member).  No device
    work faults."""
    import qusim_gb300 as q
    monkeypatch.setenv("QSG_SERVER_FAIL_REQUEST", str(bad))
    reqs = make_requests()
    srv = q.Server(0, max_running=64)
    ids = [srv.submit(r["psi0"], r["V"], r["dx"], r["dt"], r["nsteps"], order=r["order"], precision="mixed",
                      dy=r.get("dy")) for r in reqs]
    assert ids == list(range(1, len(reqs) + 1))
    results = {}
    for i in ids:
        state = srv.wait(i, 300)
        if i == bad:
            assert state == q.Server.FAILED
            with pytest.raises(q.QsgError) as e:
                srv.take(i)
            assert e.value.code == 3 and "injected" in str(e.value)
        else:
            assert state == q.Server.DONE
            results[i] = srv.take(i)[0]
    st = srv.stats()
    srv.close()
    assert st["failed"] == 1 and st["completed"] == len(reqs) - 1
    ctx = q.Context(0)
    for i, r in zip(ids, reqs):
        if i != bad:
            assert np.array_equal(results[i], solo(q, ctx, r, "mixed")), i
    ctx.close()


def test_requests_admitted_while_others_run():
    """Continuous batching: a long complex128 2D request is submitted first;
    once it is RUNNING with a chunk on the device, more requests arrive.  They
    are admitted while the first one's work is in flight, their work is queued
    beside it (server statistics), they finish before it, and every result is
    bitwise the one a solo run gives."""
    import time

    import qusim_gb300 as q
    h = 51.2
    p, dx, dy = gauss_packet_2d(1024, 1024, -h, h, -h, h, 1.0, 0.3, -10.0, 0.0, 4.0)
    v = gaussian_bumps_2d(1024, 1024, -h, h, -h, h, nbumps=8, seed=7, spread=20.0)
    first = dict(psi0=p, V=v, dx=dx, dy=dy, dt=0.01, nsteps=400, order=4)
    later = make_requests(seed=11)
    srv = q.Server(0, max_running=64)
    fid = srv.submit(first["psi0"], first["V"], dx, 0.01, 400, order=4, precision="fp64", dy=dy)
    t_end = time.time() + 60
    while time.time() < t_end:
        info = srv.request_info(fid)
        if info["state"] == q.Server.RUNNING and info["chunks"] >= 1:
            break
        time.sleep(0.001)
    assert info["state"] == q.Server.RUNNING and info["chunks"] >= 1, info
    ids = [srv.submit(r["psi0"], r["V"], r["dx"], r["dt"], r["nsteps"], order=r["order"], precision="mixed",
                      dy=r.get("dy")) for r in later]
    infos = {}
    for i in ids + [fid]:
        assert srv.wait(i, 300) == q.Server.DONE
        infos[i] = srv.request_info(i)
    results = {i: srv.take(i)[0] for i in ids + [fid]}
    st = srv.stats()
    srv.close()
    f = infos[fid]
    assert f["chunks"] >= 2  # the long request advanced in several chunks
    for i in ids:
        assert f["t_first_dispatch"] < infos[i]["t_admit"] < f["t_finish"], (f, infos[i])
    assert sum(infos[i]["admitted_mid_flight"] for i in ids) >= 1
    assert st["admitted_mid_flight"] >= 1 and st["max_in_flight"] >= 2, st
    assert any(infos[i]["t_finish"] < f["t_finish"] for i in ids)
    ctx = q.Context(0)
    assert np.array_equal(results[fid], solo(q, ctx, first, "fp64"))
    for i, r in zip(ids, later):
        assert np.array_equal(results[i], solo(q, ctx, r, "mixed")), i
    ctx.close()


def test_served_length_not_power_of_two_equals_solo():
    """Requests on a 1000-site grid (Bluestein transforms in one CTA) and a
    5000-site grid (Bluestein on the four-step passes) beside power-of-two ones:
    served in chunks, bitwise their solo runs."""
    import qusim_gb300 as q
    p, v, dx = gauss_packet_1d(1000, -50, 50, 1.0, -10, 3.0, barrier=0.8)
    p5, v5, dx5 = gauss_packet_1d(5000, -100, 100, 1.0, -20, 5.0, barrier=0.8)
    reqs = make_requests()[:3] + [dict(psi0=p, V=v, dx=dx, dt=0.01, nsteps=333, order=4),
                                  dict(psi0=p5, V=v5, dx=dx5, dt=0.01, nsteps=40, order=4)]
    srv = q.Server(0)
    ids = [srv.submit(r["psi0"], r["V"], r["dx"], r["dt"], r["nsteps"], order=r["order"], precision="mixed",
                      dy=r.get("dy")) for r in reqs]
    out = []
    for i in ids:
        assert srv.wait(i, 300) == q.Server.DONE
        out.append(srv.take(i)[0])
    srv.close()
    ctx = q.Context(0)
    for r, psi in zip(reqs, out):
        assert np.array_equal(psi, solo(q, ctx, r, "mixed"))
    ctx.close()


def test_descriptor_ring_reused_many_times(monkeypatch):
    """Batched resident launches take slots of a descriptor ring, free again
    only once the launch that reads them has completed.  With an 8-slot ring
    and 60 requests of 1 to 3 chunks each, submitted while earlier ones run,
    the ring wraps dozens of times past requests that have already finished;
    every request ends DONE, bitwise equal to its solo run."""
    import qusim_gb300 as q
    monkeypatch.setenv("QSG_SERVER_RING", "8")
    rng = np.random.default_rng(11)
    reqs = []
    for k in range(60):
        n = (1024, 2048, 4096)[k % 3]
        box = 0.05 * n
        p, v, dx = gauss_packet_1d(n, -box, box, rng.uniform(0.5, 3), -0.25 * box, rng.uniform(2, 20), barrier=0.8)
        reqs.append(dict(psi0=p, V=v, dx=dx, dt=0.01, nsteps=int(rng.integers(100, 3000)), order=2 + 2 * (k % 2)))
    srv = q.Server(0, max_running=6)
    ids = []
    for k, r in enumerate(reqs):
        ids.append(srv.submit(r["psi0"], r["V"], r["dx"], r["dt"], r["nsteps"], order=r["order"],
                              precision="mixed"))
        if k % 10 == 9:
            srv.wait(ids[-8], 300)  # later submissions arrive while the ring is in use
    results = []
    for i in ids:
        assert srv.wait(i, 300) == q.Server.DONE
        results.append(srv.take(i)[0])
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    ctx = q.Context(0)
    for r, psi in zip(reqs, results):
        assert np.array_equal(psi, solo(q, ctx, r, "mixed"))
    ctx.close()
