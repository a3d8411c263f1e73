"""3D split-operator on the GPU against the oracle's 3D step (SplittingMethod2D's
formulas with a third axis; the 3D transform is pinned to the reference's
KissFourierTransform3D in tests/test_oracle.py).

complex128: relative L2 <= 1e-12; complex64 ("mixed"): <= 2e-5 over the few
steps run here.
"""
import numpy as np
import pytest

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


def packet3d(nx, ny, nz, half=(10.0, 8.0, 12.0), k=(1.5, -0.5, 0.8), seed=0):
    xs = [(-h + 2 * h / n * np.arange(n)) for h, n in zip(half, (nx, ny, nz))]
    X, Y, Z = np.meshgrid(*xs, indexing="ij")
    psi = np.exp(1j * (k[0] * X + k[1] * Y + k[2] * Z)) * np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / (4 * 2.0 ** 2))
    rng = np.random.default_rng(seed)
    c = rng.uniform(-3, 3, size=3)
    V = 0.8 * np.exp(-((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) / 2.0)
    d = [2 * h / n for h, n in zip(half, (nx, ny, nz))]
    psi /= np.sqrt(np.sum(np.abs(psi) ** 2) * d[0] * d[1] * d[2])
    return psi.astype(np.complex128), V, d


SHAPES = [(32, 16, 64), (64, 32, 16), (16, 16, 16), (1024, 16, 16), (16, 1024, 16), (16, 16, 1024)]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("order", [2, 4])
@pytest.mark.parametrize("shape", SHAPES, ids=["x".join(map(str, s)) for s in SHAPES])
def test_evolve3d_matches_oracle(q, ctx, oracle, shape, order, precision):
    psi0, V, (dx, dy, dz) = packet3d(*shape)
    steps = 6
    ref = oracle.evolve3d(psi0, V, dx, dy, dz, 0.01, steps, order=order)
    inst = q.Instance.create_3d(ctx, psi0, V, dx, dy, dz, 0.01, order=order, precision=precision)
    inst.step(4)
    inst.step(2)  # two calls: the closing V factor of the first merges into the second's opening pass
    got = inst.get_psi()
    tol = 1e-12 if precision == "fp64" else 2e-5
    assert rel_l2(got, ref) <= tol
    kin, pot = inst.energies()
    kref = oracle.kinen3d(ref, dx, dy, dz)
    pref = float(np.sum(np.abs(ref) ** 2 * V) / np.sum(np.abs(ref) ** 2))
    assert abs(kin - kref) <= tol * 10 * abs(kref)
    assert abs(pot - pref) <= tol * 10 * max(abs(pref), 1e-3)
    n2 = inst.norm2()
    assert abs(n2 - np.sum(np.abs(ref) ** 2) * dx * dy * dz) <= tol * 10
    inst.close()


def test_evolve3d_renormalize_and_imaginary_time(q, ctx, oracle):
    psi0, V, (dx, dy, dz) = packet3d(32, 32, 32)
    inst = q.Instance.create_3d(ctx, psi0, V, dx, dy, dz, 0.01 - 0.005j, order=4, precision="fp64")
    inst.step(3, renormalize=True)
    ref = oracle.evolve3d(psi0, V, dx, dy, dz, 0.01 - 0.005j, 3, order=4)
    ref /= np.sqrt(np.sum(np.abs(ref) ** 2) * dx * dy * dz)
    assert rel_l2(inst.get_psi(), ref) <= 1e-12
    assert abs(inst.norm2() - 1.0) <= 1e-12
    inst.close()


def test_evolve3d_rejects_unsupported(q, ctx):
    psi0, V, (dx, dy, dz) = packet3d(16, 16, 8)
    with pytest.raises(q.QsgError) as e:
        q.Instance.create_3d(ctx, psi0, V, dx, dy, dz, 0.01)
    assert e.value.code == 5
    psi0, V, (dx, dy, dz) = packet3d(16, 24, 16)
    with pytest.raises(q.QsgError) as e:
        q.Instance.create_3d(ctx, psi0, V, dx, dy, dz, 0.01)
    assert e.value.code == 5
