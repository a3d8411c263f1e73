"""Generate the golden fixtures in this folder from the reference itself.

Runs the reference's own SplittingMethod1D/2D, KISS FourierTransform and
Born-series solvers (QuPerturbation1DImpl/2DImpl),
compiled from its sources by ``make -C oracle ref`` (oracle/_ref), on seeded
inputs and stores inputs + outputs as .npz.  The reference tree is needed
only here; the committed fixtures travel without it.

    python tests/golden/make_golden.py [name-prefix ...]

With name prefixes, only the fixtures whose names start with one of them are
written (the others are left as they are).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402
from tests.workloads import (BORN_1D_CASES, BORN_2D_CASES, BORN_XSEC_TOTAL, CAL_BAD,  # noqa: E402
                             CAL_EXPRESSIONS, CAL_POINTS, born_potential_1d, born_potential_2d, gauss_packet_1d,
                             gauss_packet_2d, gaussian_bumps_2d, xsec_cosines)


ONLY = tuple(sys.argv[1:])


def wanted(name):
    return not ONLY or name.startswith(ONLY)


def save(name, **arrays):
    if not wanted(name):
        return
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    print("wrote", os.path.relpath(path, ROOT), os.path.getsize(path), "bytes")


def main():
    orc.build(ref=True)
    ref = orc.Reference()

    # FFT ramp input x[i] = i (not stored: np.arange), the shapes of applications/QuSimTest/TestFFT.cpp:89-99
    for n in (1234, 4096):
        x = np.arange(n, dtype=np.complex128)
        save(f"fft1d_ramp_{n}", fwd=ref.fft1d(x), inv=ref.fft1d(x, inverse=True))
    for nx, ny in ((123, 234), (64, 128)):
        x = np.arange(nx * ny, dtype=np.complex128).reshape(nx, ny)
        save(f"fft2d_ramp_{nx}x{ny}", fwd=ref.fft2d(x), inv=ref.fft2d(x, inverse=True))

    # 3D FFT (KissFourierTransform3D) on ramps: the component the 3D split-operator
    # step shares with the reference (which has no 3D evolver)
    for shape in ((6, 10, 14), (16, 8, 32)):
        x = np.arange(int(np.prod(shape)), dtype=np.complex128).reshape(shape) * (1 + 0.5j)
        save("fft3d_ramp_%dx%dx%d" % shape, fwd=ref.fft3d(x), inv=ref.fft3d(x, inverse=True))

    # 1D evolutions.  (name, n, x0, x1, k0, xc, s, order, wall, dt, batch, calls, fnes[, mass, hbar])
    cases_1d = [
        # the 1D plain configuration: N=4096 on [-200,200), k0=1, x0=-50, s=10,
        # V=0.5 exp(-x^2/2), dt=0.05, 2000 O2 steps
        ("evolve1d_n4096_o2_2000", 4096, -200.0, 200.0, 1.0, -50.0, 10.0, 2, False, 0.05, 2000, 1, False),
        ("evolve1d_n4096_o4_200", 4096, -200.0, 200.0, 1.0, -50.0, 10.0, 4, False, 0.05, 200, 1, False),
        ("evolve1d_n256_o2_b7x3_fnes", 256, -30.0, 30.0, 2.0, -5.0, 2.0, 2, False, 0.01, 7, 3, True),
        ("evolve1d_n1024_o4_imag", 1024, -50.0, 50.0, 1.5, -10.0, 3.0, 4, False, 0.02 - 0.005j, 40, 1, False),
        ("evolve1d_n512_o2_wall", 512, -40.0, 40.0, 1.0, -10.0, 3.0, 2, True, 0.02, 100, 1, False),
        ("evolve1d_n1000_o2", 1000, -50.0, 50.0, 1.0, -10.0, 3.0, 2, False, 0.02, 100, 1, False),
        # hbar and mass away from 1: the periodic KinEn omits hbar^2
        # (src/SplittingMethod1D.cpp:101-102), the wall KinEn keeps it (:118)
        ("evolve1d_n1024_o2_hbar07_m2", 1024, -50.0, 50.0, 1.5, -10.0, 3.0, 2, False, 0.02, 150, 1, False,
         2.0, 0.7),
        ("evolve1d_n512_o4_wall_hbar07_m2", 512, -40.0, 40.0, 1.0, -10.0, 3.0, 4, True, 0.02, 60, 1, False,
         2.0, 0.7),
        # a wall of a length that is not a power of two: KISS transforms of 2n = 1200
        ("evolve1d_n600_o4_wall", 600, -40.0, 40.0, 1.0, -10.0, 3.0, 4, True, 0.02, 40, 1, False),
        # periodic lengths above 4096 that are not powers of two: 5000 = 2^3 5^4 and the
        # prime 4099 (a generic-radix KISS transform), renormalising calls
        ("evolve1d_n5000_o4", 5000, -100.0, 100.0, 1.0, -20.0, 5.0, 4, False, 0.02, 20, 1, False),
        ("evolve1d_n4099_o2_b5x2_fnes", 4099, -80.0, 80.0, 1.0, -15.0, 4.0, 2, False, 0.02, 5, 2, True),
        # a wall whose 2n = 6000 extension is too long for one CTA's Bluestein transform
        ("evolve1d_n3000_o4_wall", 3000, -60.0, 60.0, 1.0, -15.0, 4.0, 4, True, 0.02, 20, 1, False),
    ]
    for case in cases_1d:
        name, n, x0, x1, k0, xc, s, order, wall, dt, batch, calls, fnes = case[:13]
        mass, hbar = case[13:] if len(case) > 13 else (1.0, 1.0)
        if not wanted(name):
            continue
        psi0, V, dx = gauss_packet_1d(n, x0, x1, k0, xc, s, barrier=0.5)
        psi, nrm, kin, pot = ref.evolve1d(psi0, V, x0, x1, dt, batch, calls=calls, order=order,
                                          mass=mass, hbar=hbar, wall=wall, fnes=fnes)
        extra = {} if (mass, hbar) == (1.0, 1.0) else dict(mass=np.float64(mass), hbar=np.float64(hbar))
        save(name, psi0=psi0, V=V, psi=psi, norm2=nrm, kin=kin, pot=pot,
             params=np.array([n, x0, x1, order, int(wall), batch, calls, int(fnes)], dtype=np.float64),
             dt=np.complex128(dt), **extra)

    # 2D evolutions.  (name, nx, ny, half_x, half_y, order, dt, batch, calls, fnes[, mass, hbar])
    cases_2d = [
        ("evolve2d_128x256_o2_50", 128, 256, 20.0, 40.0, 2, 0.02, 50, 1, False),
        ("evolve2d_256x128_o4_20", 256, 128, 30.0, 30.0, 4, 0.02, 20, 1, False),
        ("evolve2d_128x128_o4_b5x2_fnes", 128, 128, 10.0, 20.0, 4, 0.01 - 0.002j, 5, 2, True),
        ("evolve2d_128x256_o4_hbar07_m2", 128, 256, 20.0, 40.0, 4, 0.02, 20, 1, False, 2.0, 0.7),
        # sides that are not powers of two: KISS radices 3, 5 (45) and 2, 5, 7 (70, a generic
        # radix-7 butterfly); 96 x 50 mixes a power-of-two-free side with radix 3 and 2
        ("evolve2d_45x70_o2_30", 45, 70, 9.0, 14.0, 2, 0.02, 30, 1, False),
        ("evolve2d_96x50_o4_10", 96, 50, 12.0, 10.0, 4, 0.02, 10, 1, False),
    ]
    for case in cases_2d:
        name, nx, ny, hx, hy, order, dt, batch, calls, fnes = case[:10]
        mass, hbar = case[10:] if len(case) > 10 else (1.0, 1.0)
        if not wanted(name):
            continue
        x0, x1, y0, y1 = -hx, hx, -hy, hy
        psi0, dx, dy = gauss_packet_2d(nx, ny, x0, x1, y0, y1, kx=1.5, ky=0.0, xc=-0.3 * hx, yc=0.0, s=0.1 * hx)
        V = gaussian_bumps_2d(nx, ny, x0, x1, y0, y1, nbumps=16, seed=0, spread=0.5 * hx)
        psi, nrm, kin, pot = ref.evolve2d(psi0, V, x0, x1, y0, y1, dt, batch, calls=calls,
                                          order=order, mass=mass, hbar=hbar, fnes=fnes)
        extra = {} if (mass, hbar) == (1.0, 1.0) else dict(mass=np.float64(mass), hbar=np.float64(hbar))
        save(name, psi0=psi0, V=V, psi=psi, norm2=nrm, kin=kin, pot=pot,
             params=np.array([nx, ny, x0, x1, y0, y1, order, batch, calls, int(fnes)], dtype=np.float64),
             dt=np.complex128(dt), **extra)

    # expressions of the reference's calculator (src/Cal.cpp) at a few points
    # (tests/workloads.py CAL_EXPRESSIONS / CAL_POINTS)
    if wanted("cal_exprs"):
        vals = np.zeros((len(CAL_EXPRESSIONS), len(CAL_POINTS)), np.complex128)
        for i, e in enumerate(CAL_EXPRESSIONS):
            for j, (x, y) in enumerate(CAL_POINTS):
                v = ref.cal_eval(e, {"x": x, "y": y})
                assert v is not None, e
                vals[i, j] = v
        bad = np.array([ref.cal_eval(e, {"x": 1.0, "y": 2.0}) is None for e in CAL_BAD])
        save("cal_exprs", values=vals, bad_fail=bad)

    # Born-series scattering, 1D and 2D (tests/workloads.py BORN_*_CASES)
    for (name, n, x0, x1, v0, en, eps, direction, order, pre, precer, slow,
         computes) in BORN_1D_CASES:
        if not wanted(name):
            continue
        V, _ = born_potential_1d(n, x0, x1, v0)
        r = ref.born1d(V, x0, x1, en, eps, direction=direction, order=order, preconditional=pre,
                       preconditioner=precer, slow=slow, computes=computes)
        # V (the input) is stored: numpy's exp differs in the last bit between platforms
        save(name, V=V, dpsi=r["dpsi"], psi0=r["psi0"], v=r["v"], epsilon=r["epsilon"],
             R=r["R"], T=r["T"])
    cs = xsec_cosines()
    for (name, nx, ny, hx, hy, en, eps, dirx, diry, order, pre, precer, slow,
         computes) in BORN_2D_CASES:
        if not wanted(name):
            continue
        V, _, _ = born_potential_2d(nx, ny, -hx, hx, -hy, hy)
        r = ref.born2d(V, -hx, hx, -hy, hy, en, eps, dirx=dirx, diry=diry, order=order,
                       preconditional=pre, preconditioner=precer, slow=slow, computes=computes,
                       cosxy=cs, ntot=BORN_XSEC_TOTAL)
        # psi0 and v by their sums (V is regenerated from the workload)
        save(name, dpsi=r["dpsi"], psi0_sum=r["psi0"].sum(), v_sum=r["v"].sum(),
             epsilon=r["epsilon"], delta_norm=r["delta_norm"], xsec=np.array(r["xsec"]),
             total=r["total"])


if __name__ == "__main__":
    main()
