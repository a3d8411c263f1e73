"""The two forms of a complex64 2D instance (qsg_set_form).

Both run the reference's step (SplittingMethod2D, src/SplittingMethod2D.cpp:81-121)
and agree with the complex128 path to complex64 rounding.  The momentum form
keeps the state in momentum space and adds each potential factor as an
increment; its rounding error against complex128 is well below the direct
form's (the transforms' rounding scales with |V - 1|, not with |psi|).
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


def _case(n=512, seed=3):
    psi0, dx, dy = gauss_packet_2d(n, n, -50, 50, -50, 50, 1.5, 0.0, -20.0, 0.0, 5.0)
    V = gaussian_bumps_2d(n, n, -50, 50, -50, 50, nbumps=16, seed=seed, spread=25.0)
    return psi0, V, dx, dy


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("order", [2, 4])
def test_forms_against_complex128(q, order):
    ctx = q.Context(0)
    psi0, V, dx, dy = _case()
    steps, dt = 200, 0.02
    ref = q.Instance.create_2d(ctx, psi0, V, dx, dy, dt, order=order, precision="fp64")
    mom = q.Instance.create_2d(ctx, psi0, V, dx, dy, dt, order=order, precision="mixed")
    dirc = q.Instance.create_2d(ctx, psi0, V, dx, dy, dt, order=order, precision="mixed")
    assert mom.form == "momentum" and ref.form == "direct"
    dirc.form = "direct"
    assert dirc.form == "direct"
    for inst in (ref, mom, dirc):
        inst.step(steps)
    pr = ref.get_psi()
    e_mom, e_dir = _rel(mom.get_psi(), pr), _rel(dirc.get_psi(), pr)
    assert e_mom < 1e-5 and e_dir < 2e-5
    assert e_mom < e_dir / 1.8, (e_mom, e_dir)
    # norms and energies of the two forms agree to complex64 rounding
    assert abs(mom.norm2() - ref.norm2()) < 1e-6
    km, pm = mom.energies()
    kr, pr_ = ref.energies()
    assert abs(km - kr) < 1e-5 * abs(kr) and abs(pm - pr_) < 1e-5 * max(abs(pr_), 1e-3)
    for inst in (ref, mom, dirc):
        inst.close()
    ctx.close()


@pytest.mark.parametrize("form", ["momentum", "direct"])
def test_small_calls_equal_one_call(q, form):
    ctx = q.Context(0)
    psi0, V, dx, dy = _case(256, seed=7)
    a = q.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=4, precision="mixed")
    b = q.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=4, precision="mixed")
    a.form = b.form = form
    a.step(9)
    for _ in range(9):
        b.step(1)
    assert np.array_equal(a.get_psi(), b.get_psi())
    a.close()
    b.close()
    ctx.close()


def test_form_switch_mid_run(q):
    """Switching settles the deferred pass; the state carries over."""
    ctx = q.Context(0)
    psi0, V, dx, dy = _case(256, seed=8)
    ref = q.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=4, precision="fp64")
    a = q.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=4, precision="mixed")
    ref.step(20)
    a.step(10)
    a.form = "direct"
    a.step(5)
    a.form = "momentum"
    a.step(5)
    assert _rel(a.get_psi(), ref.get_psi()) < 5e-6
    a.close()
    ref.close()
    ctx.close()


def test_renormalised_steps(q):
    """renormalize = True (force normalisation each step) in the momentum form."""
    ctx = q.Context(0)
    psi0, V, dx, dy = _case(256, seed=9)
    ref = q.Instance.create_2d(ctx, psi0 * 0.7, V, dx, dy, 0.01, order=4, precision="fp64")
    a = q.Instance.create_2d(ctx, psi0 * 0.7, V, dx, dy, 0.01, order=4, precision="mixed")
    for _ in range(3):
        ref.step(4, renormalize=True)
        a.step(4, renormalize=True)
    assert abs(a.norm2() - 1.0) < 1e-6
    assert _rel(a.get_psi(), ref.get_psi()) < 5e-6
    a.close()
    ref.close()
    ctx.close()


def test_momentum_form_only_for_complex64_2d(q):
    from qusim_gb300 import QsgError
    ctx = q.Context(0)
    psi0, V, dx, dy = _case(128, seed=1)
    a = q.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=2, precision="fp64")
    with pytest.raises(QsgError):
        a.form = "momentum"
    a.form = "direct"
    a.close()
    ctx.close()


def test_read_after_every_step(q):
    """A read after every step settles the state each time; the passes that then
    transform the whole state keep hi + lo twiddles, so the momentum form stays
    at least as accurate as the direct form (no coherent growth)."""
    ctx = q.Context(0)
    psi0, V, dx, dy = _case(512, seed=5)
    steps, dt = 300, 0.02
    ref = q.Instance.create_2d(ctx, psi0, V, dx, dy, dt, order=4, precision="fp64")
    ref.step(steps)
    pr = ref.get_psi()
    errs = {}
    for form in ("momentum", "direct"):
        a = q.Instance.create_2d(ctx, psi0, V, dx, dy, dt, order=4, precision="mixed")
        a.form = form
        for _ in range(steps):
            a.step(1)
            a.norm2()
        errs[form] = _rel(a.get_psi(), pr)
        a.close()
    assert errs["momentum"] < 1e-5, errs
    assert errs["momentum"] <= 1.2 * errs["direct"], errs
    ref.close()
    ctx.close()


@pytest.mark.parametrize("form", ["momentum", "direct"])
def test_imaginary_time_non_square(q, form):
    """Imaginary time (dt = -i tau: real decaying factors, |V - 1| up to ~tau V)
    on a non-square grid, renormalised every call, against complex128."""
    ctx = q.Context(0)
    nx, ny = 512, 256
    psi0, dx, dy = gauss_packet_2d(nx, ny, -40, 40, -20, 20, 0.5, 0.0, -5.0, 0.0, 4.0)
    V = gaussian_bumps_2d(nx, ny, -40, 40, -20, 20, nbumps=8, seed=12, spread=15.0, hmin=0.0, hmax=1.0)
    dt = -0.01j
    ref = q.Instance.create_2d(ctx, psi0, V, dx, dy, dt, order=4, precision="fp64")
    a = q.Instance.create_2d(ctx, psi0, V, dx, dy, dt, order=4, precision="mixed")
    a.form = form
    for _ in range(10):
        ref.step(5, renormalize=True)
        a.step(5, renormalize=True)
    assert _rel(a.get_psi(), ref.get_psi()) < 5e-6
    assert abs(a.norm2() - 1.0) < 1e-6
    ka, pa = a.energies()
    kr, pr = ref.energies()
    assert abs((ka + pa) - (kr + pr)) < 1e-5 * abs(kr + pr)
    a.close()
    ref.close()
    ctx.close()


@pytest.mark.parametrize("n", [2048, 4096])
def test_tensor_copy_column_pass_is_bitwise_the_plain_one(q, monkeypatch, n):
    """The momentum-form column pass fed by tensor copies (QSG_COL_TMA, on by
    default where the tile shape is compiled) computes exactly what the
    load-instruction pass computes: same states, same step norms."""
    psi0, dx, dy = gauss_packet_2d(n, n, -0.05 * n, 0.05 * n, -0.05 * n, 0.05 * n, 1.5, 0.0, -0.01 * n, 0.0,
                                   0.004 * n)
    V = gaussian_bumps_2d(n, n, -0.05 * n, 0.05 * n, -0.05 * n, 0.05 * n, nbumps=8, seed=13, spread=0.02 * n)
    out = []
    for tma in ("1", "0"):
        monkeypatch.setenv("QSG_COL_TMA", tma)
        c = q.Context(0)
        a = q.Instance.create_2d(c, psi0, V, dx, dy, 0.01, order=4, precision="mixed")
        a.step(3)
        a.step(2, renormalize=True)  # its last column pass keeps hi + lo twiddles
        a.step(2)
        sn = a.step_norm2()
        a.sync()
        out.append((a.get_psi(), sn, a.plan().as_tuple()))
        a.close()
        c.close()
    assert out[0][2] == out[1][2]
    assert out[0][1] == out[1][1]
    assert np.array_equal(out[0][0], out[1][0])


def test_bounded_wait_runs_out_cleanly(q):
    """A tensor-copy column pass whose copies are withheld: every CTA's first
    wait runs out after 1 s and the pass returns.  A pass that ran out of time
    may leave some tiles of the state updated and others not, so the instance's
    state counts as lost: the check reports QSG_ERR_TIMEOUT, and every later
    call on that instance (sync, reads, steps) does too until qsg_set_psi gives
    it a new state.  The context and its other instances keep working."""
    n = 2048
    psi0, dx, dy = gauss_packet_2d(n, n, -100, 100, -100, 100, 1.5, 0.0, -20.0, 0.0, 8.0)
    V = gaussian_bumps_2d(n, n, -100, 100, -100, 100, nbumps=8, seed=14, spread=40.0)
    ctx = q.Context(0)
    a = q.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=4, precision="mixed")
    b = q.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=4, precision="mixed")
    a.step(2)
    b.step(2)
    assert a.check_wait_timeout() == 4
    for call in (a.sync, a.get_psi, a.norm2, a.energies, lambda: a.step(1)):
        with pytest.raises(q.QsgError) as e:
            call()
        assert e.value.code == 4 and "qsg_set_psi" in str(e.value)
    b.step(1)  # the other instance is unaffected
    b_state = b.get_psi()
    a.set_psi(b_state)  # a new state makes the instance usable again
    a.step(2)
    b.step(2)
    assert np.array_equal(a.get_psi(), b.get_psi())
    ref = q.Instance.create_2d(ctx, psi0[:256, :256], V[:256, :256], dx, dy, 0.01, order=4, precision="fp64")
    assert ref.check_wait_timeout() == 5  # complex128: no such pass
    for inst in (a, b, ref):
        inst.close()
    ctx.close()
