"""1D execution plans on the GPU: every candidate plan steps to the oracle's
result, a switch between steps keeps the state, the 1D autotuner leaves the
state alone and its choice is cached for new instances of the size (in the
context and through the plan cache file), batch members keep their batch's
plan."""
import numpy as np
import pytest

from tests.workloads import gauss_packet_1d

pytestmark = pytest.mark.gpu

PLAIN_TOL = 1e-12
MIXED_TOL = 1e-5
WALL = 1


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


def packet(n):
    return gauss_packet_1d(n, -0.05 * n, 0.05 * n, 1.5, -0.01 * n, 0.005 * n + 1, barrier=0.7)


@pytest.mark.parametrize("n", [8192, 16384, 131072])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_every_1d_plan_matches_oracle(qsg, ctx, oracle, n, precision):
    """Each candidate plan (one CTA, and every four-step split with and without
    tensor-copy columns), hbar = 0.7, m = 2, O4: the oracle's result and its
    kinetic energy."""
    psi0, V, dx = packet(n)
    ref = oracle.evolve1d(psi0, V, dx, 0.01, 3, order=4, mass=2.0, hbar=0.7)
    kref = oracle.kinen1d(ref, dx, mass=2.0, hbar=0.7)
    tol, ktol = (PLAIN_TOL, 1e-10) if precision == "fp64" else (MIXED_TOL, 1e-5)
    plans = qsg.candidate_plans_1d(precision, n)
    assert len(plans) >= 2
    for p in plans:
        inst = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.01, order=4, precision=precision, mass=2.0, hbar=0.7)
        inst.set_plan(p)
        assert inst.plan().as_tuple() == p.as_tuple()
        inst.step(3)
        assert rel_l2(inst.get_psi(), ref) <= tol, p
        kin, _ = inst.energies()
        assert abs(kin - kref) <= ktol * abs(kref), p
        inst.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_plan_switch_between_steps_keeps_the_state(qsg, ctx, oracle, precision):
    """3 steps on one plan, a switch, 3 on the next, and so on through every
    candidate: the oracle's result after all the steps."""
    n = 32768
    psi0, V, dx = packet(n)
    plans = qsg.candidate_plans_1d(precision, n)
    ref = oracle.evolve1d(psi0, V, dx, 0.01, 3 * len(plans), order=2)
    inst = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.01, order=2, precision=precision)
    for p in plans:
        inst.set_plan(p)
        inst.step(3)
    tol = PLAIN_TOL if precision == "fp64" else MIXED_TOL
    assert rel_l2(inst.get_psi(), ref) <= tol
    assert inst.steps_taken() == 3 * len(plans)


def test_wall_extension_plans_match_oracle(qsg, ctx, oracle):
    """A wall above one CTA runs its 2n extension on each four-step split."""
    n = 16384
    wall = qsg.BoundaryCondition.InfiniteWall
    psi0, V, dx = gauss_packet_1d(n, -0.05 * n, 0.05 * n, 1.5, -0.01 * n, 0.01 * n + 1, barrier=0.7)
    ref = oracle.evolve1d(psi0, V, dx, 0.02, 4, order=2, wall=True)
    plans = qsg.candidate_plans_1d("mixed", n, WALL)
    assert len(plans) >= 2 and all(p.kind == 1 and p.tma == 0 for p in plans)
    for p in plans:
        inst = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.02, order=2, precision="mixed", boundary=wall)
        inst.set_plan(p)
        inst.step(4)
        assert rel_l2(inst.get_psi(), ref) <= MIXED_TOL, p
        inst.close()


def test_plan_refusals(qsg, ctx):
    psi0, V, dx = packet(16384)
    inst = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.01, precision="fp64")
    with pytest.raises(qsg.QsgError) as e:
        inst.set_plan((1, 128, 1))  # tensor-copy columns are complex64 only
    assert e.value.code == 5
    with pytest.raises(qsg.QsgError) as e:
        inst.set_plan((0, 0, 0))    # 16384 does not fit one CTA
    assert e.value.code == 5
    b = qsg.Batch(ctx, [psi0, psi0], [V, V], [dx, dx], [0.01, 0.01], precision="mixed")
    with pytest.raises(qsg.QsgError) as e:
        b.instance(0).set_plan((1, 256, 0))
    assert e.value.code == 6


def test_autotune_1d_keeps_state_and_is_cached(qsg, tmp_path, monkeypatch):
    """The tuner times every plan on a copy: psi and the step count are
    unchanged.  Its choice goes to new instances of the size in the context and,
    persisted, to a new context's instances through the plan cache file."""
    cache = tmp_path / "plans.tsv"
    monkeypatch.setenv("QSG_PLAN_CACHE", str(cache))
    ctx = qsg.Context(0)
    n = 65536
    psi0, V, dx = packet(n)
    inst = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.01, order=4, precision="mixed")
    inst.step(2)
    before = inst.get_psi().copy()
    plan, ms = inst.autotune(trial_steps=8, persist=True)
    assert ms > 0
    assert plan.as_tuple() in [p.as_tuple() for p in qsg.candidate_plans_1d("mixed", n)]
    assert inst.plan().as_tuple() == plan.as_tuple()
    assert np.array_equal(inst.get_psi(), before)
    assert inst.steps_taken() == 2
    other = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.01, order=2, precision="mixed")
    assert other.plan().as_tuple() == plan.as_tuple()
    text = cache.read_text()
    assert "\t1d\t" in text
    ctx.close()
    ctx2 = qsg.Context(0)
    fresh = qsg.Instance.create_1d(ctx2, psi0, V, dx, 0.01, order=4, precision="mixed")
    assert fresh.plan().as_tuple() == plan.as_tuple()
    # members of a batch built on the tuned plan step as the instance alone does
    b = qsg.Batch(ctx2, [psi0, psi0], [V, V], [dx, dx], [0.01, 0.01], order=4, precision="mixed")
    assert b.instance(1).plan().as_tuple() == plan.as_tuple()
    b.step(3)
    fresh.step(3)
    assert np.array_equal(b.instance(1).get_psi(), fresh.get_psi())
    ctx2.close()


def test_batch_autotune_keeps_states_and_matches_solo(qsg, ctx):
    """The batch tuner times each four-step class alone on every four-step plan
    and puts the states back; stepped on afterwards, each member equals an
    instance stepped alone that switched to the same plan at the same step, bit
    for bit.  Set by hand, a batch plan goes to every member of the length."""
    sizes = [16384, 65536, 1024, 16384, 65536, 131072]
    packs = [packet(n) for n in sizes]
    psis, Vs, dxs = [p[0] for p in packs], [p[1] for p in packs], [p[2] for p in packs]
    b = qsg.Batch(ctx, psis, Vs, dxs, [0.01] * len(sizes), order=4, precision="mixed")
    b.step(2)
    before = [b.instance(k).get_psi().copy() for k in range(len(sizes))]
    plans, ms = b.autotune(trial_steps=4)
    assert ms > 0
    for k in range(len(sizes)):
        assert np.array_equal(b.instance(k).get_psi(), before[k]), k
    for n, p in plans.items():
        assert p.as_tuple() in [c.as_tuple() for c in qsg.candidate_plans_1d("mixed", n)]
        assert n == 1024 or p.kind == 1
    b.step(3)
    for k, n in enumerate(sizes):
        solo = qsg.Instance.create_1d(ctx, psis[k], Vs[k], dxs[k], 0.01, order=4, precision="mixed")
        solo.step(2)
        solo.set_plan(plans[n])
        solo.step(3)
        assert b.instance(k).plan().as_tuple() == plans[n].as_tuple()
        assert np.array_equal(b.instance(k).get_psi(), solo.get_psi()), k
        solo.close()
    # by hand: every member of the length follows
    other = next(c for c in qsg.candidate_plans_1d("mixed", 16384) if c.as_tuple() != plans[16384].as_tuple())
    b.set_plan(16384, other)
    assert b.instance(0).plan().as_tuple() == b.instance(3).plan().as_tuple() == other.as_tuple()
    with pytest.raises(qsg.QsgError) as e:
        b.set_plan(1024, (1, 64, 0))  # a one-CTA length has no four-step plan
    assert e.value.code == 5
    with pytest.raises(qsg.QsgError) as e:
        b.plan(4096)
    assert e.value.code == 1
    b.close()


def test_failed_plan_switch_keeps_the_old_plan(qsg, ctx, monkeypatch):
    """A 1D plan switch that fails after making the new plan's tables (failure
    injected on the host, QSG_FAIL_PLAN_SWITCH) leaves the instance on its old
    plan and state: it then steps bit for bit as an instance never switched.
    In a batch, the failing class stays whole."""
    n = 65536
    psi0, V, dx = packet(n)
    a = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.01, order=4, precision="mixed")
    ref = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.01, order=4, precision="mixed")
    a.step(2)
    ref.step(2)
    keep = a.plan().as_tuple()
    other = next(p for p in qsg.candidate_plans_1d("mixed", n) if p.as_tuple() != keep)
    bytes_before = ctx.bytes_in_use()
    monkeypatch.setenv("QSG_FAIL_PLAN_SWITCH", "1")
    with pytest.raises(qsg.QsgError) as e:
        a.set_plan(other)
    assert e.value.code == 3 and "injected" in str(e.value)
    b = qsg.Batch(ctx, [psi0, psi0], [V, V], [dx, dx], [0.01, 0.01], order=4, precision="mixed")
    with pytest.raises(qsg.QsgError):
        b.set_plan(n, other)
    monkeypatch.delenv("QSG_FAIL_PLAN_SWITCH")
    assert a.plan().as_tuple() == keep and b.plan(n).as_tuple() == keep
    a.step(3)
    ref.step(3)
    assert np.array_equal(a.get_psi(), ref.get_psi())
    b.step(5)
    ref5 = qsg.Instance.create_1d(ctx, psi0, V, dx, 0.01, order=4, precision="mixed")
    ref5.step(5)  # one call of 5 steps, as the batch's
    assert np.array_equal(b.instance(0).get_psi(), ref5.get_psi())
    ref5.close()
    b.close()
    assert ctx.bytes_in_use() <= bytes_before
    a.set_plan(other)  # and the switch itself still works
    assert a.plan().as_tuple() == other.as_tuple()
