"""GPU parity on the two benchmark grids themselves, at their full size.

The 2D bumps workload (1024^2 on [-100,100)^2, 16 seeded Gaussian bumps, O4,
dt = 0.02) and the large double-slit workload (4096^2 on [-200,200)^2, O4,
dt = 0.01) are built with the generators the benchmark uses
(tests/workloads.py), stepped a few O4 steps on the GPU, and compared with the
oracle (the C restatement, bit-exact with the reference's own SplittingMethod2D
on every golden fixture) on the same inputs:

  complex128: relative L2 <= 1e-12, Norm2 / KinEn / PotEn to 1e-11;
  complex64:  relative L2 <= 1e-5 (both forms), Norm2 to 1e-6, energies to 1e-4.

Every candidate plan of each grid is run, so whichever plan the autotuner
picks for the benchmark is covered (on 4096^2 complex64 it picks the x split
g = 4 with radix-16 rows and the 1024 x 8 column tile, whose momentum-form
column passes are staged by tensor copies).  A full-size O4 step of the
oracle takes a few seconds on one CPU core, so the step counts are small.
"""
import numpy as np
import pytest

from tests.workloads import config_2d_1024, config_2d_4096

pytestmark = pytest.mark.gpu

PLAIN_TOL = 1e-12
MIXED_TOL = 1e-5


def rel_l2(a, b):
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def close(a, b, tol):
    return abs(a - b) <= tol * max(1.0, abs(b))


@pytest.fixture(scope="module")
def qsg():
    import qusim_gb300 as q
    q.load()
    return q


@pytest.fixture(scope="module")
def ctx(qsg):
    c = qsg.Context(0)
    yield c
    c.close()


def oracle_run(oracle, cfg, steps):
    ref = oracle.evolve2d(cfg["psi"], cfg["V"], cfg["dx"], cfg["dy"], cfg["dt"], steps, order=cfg["order"])
    dv = cfg["dx"] * cfg["dy"]
    obs = dict(norm2=oracle.norm2(ref, dv), kin=oracle.kinen2d(ref, cfg["dx"], cfg["dy"]),
               pot=oracle.poten(ref, cfg["V"], dv))
    return ref, obs


@pytest.fixture(scope="module")
def bumps_1024(oracle):
    cfg = config_2d_1024()
    steps = 10
    ref, obs = oracle_run(oracle, cfg, steps)
    return cfg, steps, ref, obs


@pytest.fixture(scope="module")
def slit_4096(oracle):
    cfg = config_2d_4096()
    steps = 3
    ref, obs = oracle_run(oracle, cfg, steps)
    return cfg, steps, ref, obs


def check_run(qsg, ctx, case, precision, plan=None, form=None):
    cfg, steps, ref, obs = case
    inst = qsg.Instance.create_2d(ctx, cfg["psi"], cfg["V"], cfg["dx"], cfg["dy"], cfg["dt"],
                                  order=cfg["order"], precision=precision)
    try:
        if plan is not None:
            inst.set_plan(plan)
        if form is not None:
            inst.form = form
        inst.step(steps)
        psi = inst.get_psi()
        err = rel_l2(psi, ref)
        kin, pot = inst.energies()
        nrm = inst.norm2()
    finally:
        inst.close()
    if precision == "fp64":
        assert err <= PLAIN_TOL, (plan, form, err)
        assert close(nrm, obs["norm2"], 1e-11), (nrm, obs["norm2"])
        assert close(kin, obs["kin"], 1e-11), (kin, obs["kin"])
        assert close(pot, obs["pot"], 1e-11), (pot, obs["pot"])
    else:
        assert err <= MIXED_TOL, (plan, form, err)
        assert close(nrm, obs["norm2"], 1e-6), (nrm, obs["norm2"])
        assert close(kin, obs["kin"], 1e-4), (kin, obs["kin"])
        assert close(pot, obs["pot"], 1e-4), (pot, obs["pot"])
    return err


def candidates(qsg, ctx, cfg, precision):
    """Every plan compiled for the grid (qsg_candidate_plans), as tuples."""
    from qusim_gb300 import _lib
    nx, ny = cfg["psi"].shape
    prec = _lib.QSG_MIXED if precision == "mixed" else _lib.QSG_FP64
    n = ctx.lib.qsg_candidate_plans(prec, nx, ny, None, 0)
    arr = (_lib.Plan2D * max(n, 1))()
    n = ctx.lib.qsg_candidate_plans(prec, nx, ny, arr, n)
    return [arr[i].as_tuple() for i in range(n)]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_bumps_1024_default_plan_vs_oracle(qsg, ctx, bumps_1024, precision):
    check_run(qsg, ctx, bumps_1024, precision)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_bumps_1024_every_plan_vs_oracle(qsg, ctx, bumps_1024, precision):
    cfg = bumps_1024[0]
    plans = candidates(qsg, ctx, cfg, precision)
    assert plans
    for p in plans:
        check_run(qsg, ctx, bumps_1024, precision, plan=p)


def test_bumps_1024_direct_form_vs_oracle(qsg, ctx, bumps_1024):
    check_run(qsg, ctx, bumps_1024, "mixed", form="direct")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_slit_4096_default_plan_vs_oracle(qsg, ctx, slit_4096, precision):
    check_run(qsg, ctx, slit_4096, precision)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_slit_4096_every_plan_vs_oracle(qsg, ctx, slit_4096, precision):
    """Includes the benchmark's plans: (4, 16, 512, 32, 8, 0) for complex64 (the
    tensor-copy column pass) and (2, 8, 512, 8, 2, 0) for complex128."""
    cfg = slit_4096[0]
    plans = candidates(qsg, ctx, cfg, precision)
    want = (4, 16, 512, 32, 8, 0) if precision == "mixed" else (2, 8, 512, 8, 2, 0)
    assert want in plans, plans
    for p in plans:
        check_run(qsg, ctx, slit_4096, precision, plan=p)


def test_slit_4096_direct_form_vs_oracle(qsg, ctx, slit_4096):
    check_run(qsg, ctx, slit_4096, "mixed", plan=(4, 16, 512, 32, 8, 0), form="direct")
