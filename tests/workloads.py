"""Seeded synthetic inputs with the shapes of the benchmark configurations.

Gaussian packets use psi ~ exp(i k.r) exp(-|r - r0|^2 / (4 s^2)), normalised to
sum |psi|^2 dv = 1; potentials are real.  Grids are x_i = x0 + i dx with
dx = (x1 - x0) / n and index iy + ix*ny (y contiguous), as QuSim samples them
(src/EvolverImpl1D.cpp:33-81, src/EvolverImpl2D.cpp:39-98).
"""
from __future__ import annotations

import numpy as np


def grid(n, x0, x1):
    dx = (x1 - x0) / n
    return x0 + dx * np.arange(n), dx


def gauss_packet_1d(n, x0, x1, k0, xc, s, barrier=0.5):
    """Packet plus the barrier V = barrier * exp(-x^2/2)."""
    xs, dx = grid(n, x0, x1)
    psi = np.exp(1j * k0 * xs) * np.exp(-((xs - xc) ** 2) / (4 * s * s))
    psi /= np.sqrt(np.sum(np.abs(psi) ** 2) * dx)
    V = barrier * np.exp(-xs * xs / 2)
    return psi.astype(np.complex128), V.astype(np.float64), dx


def gauss_packet_2d(nx, ny, x0, x1, y0, y1, kx, ky, xc, yc, s):
    xs, dx = grid(nx, x0, x1)
    ys, dy = grid(ny, y0, y1)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    psi = np.exp(1j * (kx * X + ky * Y)) * np.exp(-((X - xc) ** 2 + (Y - yc) ** 2) / (4 * s * s))
    psi /= np.sqrt(np.sum(np.abs(psi) ** 2) * dx * dy)
    return psi.astype(np.complex128), dx, dy


def gaussian_bumps_2d(nx, ny, x0, x1, y0, y1, nbumps=16, seed=0, spread=30.0,
                      hmin=-1.0, hmax=1.0, wmin=1.0, wmax=5.0):
    """Sum of seeded Gaussian bumps h exp(-|r-c|^2/(2w^2)), c ~ U[-spread, spread]^2."""
    rng = np.random.default_rng(seed)
    xs, _ = grid(nx, x0, x1)
    ys, _ = grid(ny, y0, y1)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    V = np.zeros((nx, ny))
    c = rng.uniform(-spread, spread, size=(nbumps, 2))
    h = rng.uniform(hmin, hmax, size=nbumps)
    w = rng.uniform(wmin, wmax, size=nbumps)
    for i in range(nbumps):
        V += h[i] * np.exp(-((X - c[i, 0]) ** 2 + (Y - c[i, 1]) ** 2) / (2 * w[i] ** 2))
    return V


def config_1d_plain():
    """N=4096 on [-200,200), k0=1, x0=-50, s=10, V=0.5 exp(-x^2/2), dt=0.05, O2 x 2000."""
    psi, V, dx = gauss_packet_1d(4096, -200.0, 200.0, 1.0, -50.0, 10.0, barrier=0.5)
    return dict(psi=psi, V=V, dx=dx, x0=-200.0, x1=200.0, dt=0.05, steps=2000, order=2)


def config_2d_1024():
    """1024^2 on [-100,100)^2, k=(1.5,0), s=8 at (-40,0); 16 bumps (seed 0); dt=0.02, O4 x 1000."""
    psi, dx, dy = gauss_packet_2d(1024, 1024, -100, 100, -100, 100, 1.5, 0.0, -40.0, 0.0, 8.0)
    V = gaussian_bumps_2d(1024, 1024, -100, 100, -100, 100, nbumps=16, seed=0, spread=30.0)
    return dict(psi=psi, V=V, dx=dx, dy=dy, dt=0.02, steps=1000, order=4)


def double_slit_2d(nx=4096, ny=4096, half=200.0, seed=0):
    """Wall V=10 on |x|<1 with openings of width 2 at y=+-6, plus U[-0.01,0.01] noise."""
    xs, dx = grid(nx, -half, half)
    ys, dy = grid(ny, -half, half)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    V = np.where(np.abs(X) < 1.0, 10.0, 0.0)
    V = np.where((np.abs(X) < 1.0) & ((np.abs(Y - 6.0) < 1.0) | (np.abs(Y + 6.0) < 1.0)), 0.0, V)
    V = V + np.random.default_rng(seed).uniform(-0.01, 0.01, size=(nx, ny))
    return V, dx, dy


def config_2d_4096():
    """4096^2 on [-200,200)^2, double slit, k=(2,0), s=10 at (-60,0); dt=0.01, O4 x 2000."""
    psi, dx, dy = gauss_packet_2d(4096, 4096, -200, 200, -200, 200, 2.0, 0.0, -60.0, 0.0, 10.0)
    V, _, _ = double_slit_2d()
    return dict(psi=psi, V=V, dx=dx, dy=dy, dt=0.01, steps=2000, order=4)


def gaussian_bumps_1d(xs, nbumps, rng, lo, hi, hmin=-1.0, hmax=1.0, wmin=1.0, wmax=5.0):
    """Sum of nbumps Gaussian bumps h exp(-(x-c)^2/(2w^2)), c ~ U[lo, hi]."""
    c = rng.uniform(lo, hi, size=nbumps)
    h = rng.uniform(hmin, hmax, size=nbumps)
    w = rng.uniform(wmin, wmax, size=nbumps)
    V = np.zeros_like(xs)
    for i in range(nbumps):
        V += h[i] * np.exp(-((xs - c[i]) ** 2) / (2 * w[i] ** 2))
    return V


def batch_1d(count=2048, emin=10, emax=17, seed=0):
    """The batched 1D configuration: N = 2^e, e ~ U{emin..emax}; box [-0.05N, 0.05N)
    (dx = 0.1); packet k0 ~ U[0.5,3], s ~ U[2,20] at -0.25 of the box; 8 bumps
    (heights U[-1,1], widths U[1,5]) with centres inside the box; dt = 0.01, O2."""
    rng = np.random.default_rng(seed)
    es = rng.integers(emin, emax + 1, size=count)
    psis, Vs, dxs = [], [], []
    for e in es:
        n = 1 << int(e)
        half = 0.05 * n
        xs, dx = grid(n, -half, half)
        k0 = rng.uniform(0.5, 3.0)
        s = rng.uniform(2.0, 20.0)
        xc = -0.25 * 2 * half * 0.5
        psi = np.exp(1j * k0 * xs) * np.exp(-((xs - xc) ** 2) / (4 * s * s))
        psi /= np.sqrt(np.sum(np.abs(psi) ** 2) * dx)
        psis.append(psi.astype(np.complex128))
        Vs.append(gaussian_bumps_1d(xs, 8, rng, -half, half))
        dxs.append(dx)
    return psis, Vs, dxs


# --- Born-series scattering ---------------------------------------------------

# (name, n, x0, x1, v0, en, epsilon, direction, order, preconditional,
#  preconditioner (0 identity, 1 Vellekoop, 2 Hao1, 3 Hao2), slow, computes);
# potential v0 exp(-x^2), the one of applications/QuScattering1DPrecision
# (QuScattering1DPrecision.cpp:180-221), on power-of-two grids
BORN_1D_CASES = [
    ("born1d_n2048_naive_o3_c2", 2048, -100.0, 100.0, 0.5, 0.5, 0.01, 1.0, 3, False, 1, 1.0, 2),
    ("born1d_n2048_vellekoop_o5", 2048, -100.0, 100.0, 0.5, 0.5, 0.51, 1.0, 5, True, 1, 1.0, 1),
    ("born1d_n2048_hao1_o10_s05", 2048, -100.0, 100.0, 0.5, 0.5, 0.0, 1.0, 10, True, 2, 0.5, 1),
    ("born1d_n2048_hao2_o10_s07_left", 2048, -100.0, 100.0, 0.5, 0.5, 0.0, -1.0, 10, True, 3, 0.7, 1),
    ("born1d_n2048_identity_o10_s05", 2048, -100.0, 100.0, 0.5, 0.5, 0.0, 1.0, 10, True, 0, 0.5, 1),
    ("born1d_n2048_identity_o10_s1", 2048, -100.0, 100.0, 0.5, 0.5, 0.0, 1.0, 10, True, 0, 1.0, 1),
    ("born1d_n1000_vellekoop_o5", 1000, -100.0, 100.0, 1.0, 0.5, 0.0, 1.0, 5, True, 1, 1.0, 1),
]

# (name, nx, ny, hx, hy, en, epsilon, dirx, diry, order, preconditional,
#  preconditioner, slow, computes)
BORN_2D_CASES = [
    ("born2d_128x64_naive_o2", 128, 64, 60.0, 45.0, 0.5, 0.1, 1.0, 0.0, 2, False, 1, 1.0, 1),
    ("born2d_128x128_vellekoop_o4_c2", 128, 128, 60.0, 45.0, 2.0, 0.0, 1.0, 0.5, 4, True, 1, 1.0, 2),
    ("born2d_64x128_hao2_o3_s05", 64, 128, 45.0, 60.0, 2.0, 0.0, 0.0, 1.0, 3, True, 3, 0.5, 1),
    ("born2d_128x128_identity_o3", 128, 128, 40.0, 40.0, 2.0, 0.0, 1.0, 1.0, 3, True, 0, 1.0, 1),
]

BORN_XSEC_ANGLES = 8      # ComputeXSection at theta = 2 pi i / 8
BORN_XSEC_TOTAL = 16      # ComputeTotalXSection(16)


def born_potential_1d(n, x0, x1, v0):
    """v0 exp(-x^2) sampled at x_i = x0 + i dx (complex, as the functor returns)."""
    xs, dx = grid(n, x0, x1)
    return (v0 * np.exp(-xs * xs)).astype(np.complex128), dx


def born_potential_2d(nx, ny, x0, x1, y0, y1, v0=0.3, seed=0):
    """A Gaussian well v0 exp(-(x^2+y^2)/4) plus a weak seeded absorbing
    imaginary part (complex, as the functor returns)."""
    xs, dx = grid(nx, x0, x1)
    ys, dy = grid(ny, y0, y1)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    rng = np.random.default_rng(seed)
    c = rng.uniform(-5, 5, size=2)
    V = v0 * np.exp(-(X * X + Y * Y) / 4) - 0.02j * np.exp(-((X - c[0]) ** 2 + (Y - c[1]) ** 2) / 8)
    return V.astype(np.complex128), dx, dy


def xsec_cosines(count=BORN_XSEC_ANGLES):
    th = 2 * np.pi * np.arange(count) / count
    return np.stack([np.cos(th), np.sin(th)], axis=1)


# --- expressions of the reference's calculator (src/Cal.cpp) -------------------

# every operator and function of the language, at the points CAL_POINTS (x, y)
CAL_EXPRESSIONS = [
    "gauss(x,-20,5)*exp(I*x)",
    "exp(-x*x)",
    "0.5*exp(-x^2/2)",
    "exp(I*1.5*x)*exp(-((x+40)^2+y^2)/256)",
    "abs(x) < 1 ? (abs(y - 6) < 1 || abs(y + 6) < 1 ? 0 : 10) : 0",
    "2^-x^2 + 3*x - y/2",
    "sin(x)*cos(y) + tan(x/3) - asin(x/10) + acos(y/10) + atan(x*y)",
    "sinh(x/5) + tanh(y) + atanh(x/20) + log(1 + x*x) + sqrt(2 + y)",
    "abs(x + I*y) * (x - 0.5)",
    "x > 0 && y < 1 ? exp(I*(x+y)) : -1",
    "x >= 1 || y <= -1",
    "(x + I*y)^2.5",
    "-x^2",
    "+x*2 - -y",
    "1.5e-1*x + 2E2",
    "gauss(x, 0, 1 + I)",
    "Pi*x/ (1 + y*y)",
    "x < 0 ? x < -5 ? 1 : 2 : 3",
    "sqrt(-1 - x*x) + log(-2 + I*y)",
]
CAL_POINTS = [(-18.0, -6.5), (-0.3, 0.0), (0.5, 6.4), (1.7, 0.25), (6.2, -1.0)]
# expressions both calculators refuse
CAL_BAD = ["sin(x", "foo(x)", "x +", "unknownvar + 1", "(x", "x ? 1"]
