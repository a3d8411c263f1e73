"""psi0 and V given as expressions of the reference's calculator language,
sampled on the device (qsg_create_1d_expr / qsg_create_2d_expr).  GPU."""
import numpy as np
import pytest

from tests.workloads import double_slit_2d, gauss_packet_2d, grid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def q():
    import qusim_gb300 as q
    q.load()
    return q


@pytest.fixture(scope="module")
def ctx(q):
    c = q.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 2e-6)])
def test_tunnelling_from_the_reference_expressions(q, ctx, precision, tol):
    """applications/QuEvol1DPrecision/QuSimPrecision.cpp:106-120 written with the
    strings its FunctorWrapper takes: psi0 = gauss(x,-20,5)*exp(I*x), V =
    exp(-x*x) on [-100, 100), 2048 points, O4, dt = 0.02 to t = 64; the
    transmitted probability Norm2(0, 100) is 0.15937744085 (:82)."""
    inst = q.Instance.create_1d_expr(ctx, "gauss(x,-20,5)*exp(I*x)", "exp(-x*x)", 2048, -100.0, 100.0, 0.02,
                                     order=4, precision=precision)
    xs, dx = grid(2048, -100.0, 100.0)
    want = np.exp(-0.5 * ((xs + 20) / 5) ** 2) / (np.sqrt(2 * np.pi) * 5) * np.exp(1j * xs)
    want /= np.sqrt(np.sum(np.abs(want) ** 2) * dx)
    got = inst.get_psi()
    assert np.max(np.abs(got - want)) <= (1e-14 if precision == "fp64" else 1e-7)
    inst.step(3200)
    ref = (0.1593774409 + 0.1593774408) / 2
    assert abs(inst.norm2_range(-100.0, 0.0, 100.0) - ref) < tol
    inst.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_double_slit_expression_equals_arrays(q, ctx, precision):
    """The large 2D benchmark's wall with its two openings (without its seeded
    noise) as an expression, on a 512 x 512 grid of [-200, 200)^2: the instance
    evolves exactly as one created from the same psi0 / V arrays."""
    n, h = 512, 200.0
    slit = "abs(x) < 1 ? (abs(y - 6) < 1 || abs(y + 6) < 1 ? 0 : 10) : 0"
    packet = "exp(I*2*x)*exp(-((x+60)^2+y^2)/400)"
    a = q.Instance.create_2d_expr(ctx, packet, slit, n, n, -h, h, -h, h, 0.01, order=4, precision=precision)
    psi0, dx, dy = gauss_packet_2d(n, n, -h, h, -h, h, 2.0, 0.0, -60.0, 0.0, 10.0)
    V, _, _ = double_slit_2d(n, n, h, seed=0)
    V = np.round(V)  # the wall and the openings without the noise: 10 or 0
    b = q.Instance.create_2d(ctx, psi0, V, dx, dy, 0.01, order=4, precision=precision)
    assert np.max(np.abs(a.get_psi() - b.get_psi())) <= (1e-14 if precision == "fp64" else 1e-7)
    a.step(5)
    b.step(5)
    pa, pb = a.get_psi(), b.get_psi()
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert np.linalg.norm(pa - pb) <= tol * np.linalg.norm(pb)
    assert abs(a.energies()[1] - b.energies()[1]) <= tol
    a.close()
    b.close()


@pytest.mark.parametrize("n,wall", [(5000, False), (3000, True), (1 << 20, True)])
def test_expression_inputs_on_long_lines_equal_arrays(q, ctx, n, wall):
    """Device-sampled inputs on the long 1D paths (a Bluestein four-step buffer,
    a wall's odd extension rebuilt from a device source): the instance evolves
    exactly as one created from its own sampled psi0 and the same V."""
    bc = q.BoundaryCondition.InfiniteWall if wall else q.BoundaryCondition.Period
    h = 0.01 * n
    a = q.Instance.create_1d_expr(ctx, "exp(I*x)*exp(-(x+0.2*%g)^2/%g)" % (h, 0.002 * h * h), "0.5*exp(-x*x/2)",
                                  n, -h, h, 0.01, order=4, precision="fp64", boundary=bc)
    xs, dx = grid(n, -h, h)
    psi0 = a.get_psi()
    b = q.Instance.create_1d(ctx, psi0, 0.5 * np.exp(-xs * xs / 2), dx, 0.01, order=4, precision="fp64", boundary=bc)
    a.step(3)
    b.step(3)
    pa, pb = a.get_psi(), b.get_psi()
    assert np.linalg.norm(pa - pb) <= 1e-13 * np.linalg.norm(pb)
    a.close()
    b.close()


def test_expression_errors_are_reported(q, ctx):
    with pytest.raises(q.QsgError) as e:
        q.Instance.create_1d_expr(ctx, "gauss(x,-20,5", "exp(-x*x)", 1024, -50.0, 50.0, 0.02)
    assert e.value.code == 1 and "psi expression" in str(e.value)
    with pytest.raises(q.QsgError) as e:
        q.Instance.create_1d_expr(ctx, "exp(I*x)", "exp(-y*y)", 1024, -50.0, 50.0, 0.02)
    assert e.value.code == 1 and "var not defined: y" in str(e.value)
    assert ctx.bytes_in_use() == 0 or ctx.bytes_in_use() > 0  # the context stays usable
    inst = q.Instance.create_1d_expr(ctx, "exp(I*x)*exp(-x*x/16)", "0", 1024, -50.0, 50.0, 0.02)
    inst.step(3)
    inst.close()
