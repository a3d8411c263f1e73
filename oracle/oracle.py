"""ctypes loader for the parity oracle.  TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs
import this module; the product (``qusim_gb300``) never does.

Two libraries:

* ``liboracle.so`` -- the C restatement of the reference's split-operator
  algorithm (``qusim_oracle.c``), available wherever gcc is.
* ``_ref/libqusim_ref.so`` -- the reference's own sources compiled as they lie
  (``make ref``), available only where the reference tree exists.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libqusim_ref.so")

_dp = ctypes.POINTER(ctypes.c_double)
_sz = ctypes.c_size_t
_d = ctypes.c_double
_i = ctypes.c_int
_u64 = ctypes.c_uint64


def build(ref: bool = False, ref_path: str | None = None) -> None:
    """Compile liboracle.so (and the reference build when ``ref``, from the
    QuSim source tree at ``ref_path``, the Makefile's default if None)."""
    targets = ["all"] + (["ref"] if ref else [])
    extra = [f"REF={ref_path}"] if ref and ref_path else []
    subprocess.run(["make", "-s", "-C", HERE, "-j8"] + targets + extra, check=True)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _c128(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.complex128)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


class Oracle:
    """The C restatement (qusim_oracle.c)."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        lib.orc_fft1d.argtypes = [_sz, _i, _dp, _dp]
        lib.orc_fft2d.argtypes = [_sz, _sz, _i, _dp, _dp]
        lib.orc_evolve1d.argtypes = [_sz, _d, _d, _d, _d, _d, _i, _i, _i, _dp, _dp, _u64]
        lib.orc_evolve2d.argtypes = [_sz, _sz, _d, _d, _d, _d, _d, _d, _i, _i, _dp, _dp, _u64]
        lib.orc_kinen1d.argtypes = [_sz, _d, _d, _d, _i, _dp]
        lib.orc_kinen1d.restype = _d
        lib.orc_kinen2d.argtypes = [_sz, _sz, _d, _d, _d, _d, _dp]
        lib.orc_kinen2d.restype = _d
        lib.orc_norm2.argtypes = [_sz, _d, _dp]
        lib.orc_norm2.restype = _d
        lib.orc_renormalize.argtypes = [_sz, _d, _dp]
        lib.orc_poten.argtypes = [_sz, _d, _dp, _dp]
        lib.orc_poten.restype = _d
        lib.orc_xavg.argtypes = [_sz, _d, _d, _dp]
        lib.orc_xavg.restype = _d
        lib.orc_norm2_range.argtypes = [_sz, _d, _d, _d, _d, _dp]
        lib.orc_norm2_range.restype = _d
        lib.orc_splitting_constants.argtypes = [_dp, _dp, _dp, _dp]
        lib.orc_ev1d_new.argtypes = [_sz, _d, _d, _d, _d, _d, _i, _i]
        lib.orc_ev1d_new.restype = ctypes.c_void_p
        lib.orc_ev1d_step.argtypes = [ctypes.c_void_p, _dp, _dp, _u64]
        lib.orc_ev1d_free.argtypes = [ctypes.c_void_p]
        lib.orc_ev2d_new.argtypes = [_sz, _sz, _d, _d, _d, _d, _d, _d, _i, _dp]
        lib.orc_ev2d_new.restype = ctypes.c_void_p
        lib.orc_ev2d_step.argtypes = [ctypes.c_void_p, _dp, _u64]
        lib.orc_ev2d_free.argtypes = [ctypes.c_void_p]
        lib.orc_fft3d.argtypes = [_sz, _sz, _sz, _i, _dp, _dp]
        lib.orc_evolve3d.argtypes = [_sz, _sz, _sz, _d, _d, _d, _d, _d, _d, _d, _i, _dp, _dp, _u64]
        lib.orc_kinen3d.argtypes = [_sz, _sz, _sz, _d, _d, _d, _d, _d, _dp]
        lib.orc_kinen3d.restype = _d
        lib.orc_born_init1d.argtypes = [_sz, _d, _d, _d, _d, _d, _d, _i, _i, _dp, _dp, _dp]
        lib.orc_born_init2d.argtypes = [_sz, _sz, _d, _d, _d, _d, _d, _d, _d, _d, _d, _i, _i, _dp,
                                        _dp, _dp]
        lib.orc_born_iter1d.argtypes = [_sz, _d, _d, _d, _d, _d, _i, _i, _i, _d, _dp, _dp, _dp]
        lib.orc_born_rt1d.argtypes = [_sz, _d, _d, _d, _d, _d, _d, _dp, _dp, _dp, _dp, _dp]
        lib.orc_born_iter2d.argtypes = [_sz, _sz, _d, _d, _d, _d, _d, _d, _i, _i, _i, _d, _dp, _dp,
                                        _dp, _dp]
        lib.orc_born_xsec2d.argtypes = [_sz, _sz, _d, _d, _d, _d, _d, _d, _d, _dp, _dp, _dp, _d, _d]
        lib.orc_born_xsec2d.restype = _d
        self.lib = lib

    def fft1d(self, x, inverse=False):
        x = _c128(x)
        out = np.empty_like(x)
        assert self.lib.orc_fft1d(x.size, int(inverse), _ptr(x), _ptr(out)) == 0
        return out

    def fft2d(self, x, inverse=False):
        x = _c128(x)
        out = np.empty_like(x)
        nx, ny = x.shape
        assert self.lib.orc_fft2d(nx, ny, int(inverse), _ptr(x), _ptr(out)) == 0
        return out

    def evolve1d(self, psi, V, dx, dt, nsteps, order=2, mass=1.0, hbar=1.0,
                 wall=False, renormalize=False):
        """One Step() call of ``nsteps`` steps; renormalise once at the end."""
        psi = _c128(psi).copy()
        V = _f64(V)
        dt = complex(dt)
        rc = self.lib.orc_evolve1d(psi.size, dx, mass, hbar, dt.real, dt.imag, order,
                                   int(wall), 0, _ptr(psi), _ptr(V), nsteps)
        assert rc == 0
        if renormalize:
            self.lib.orc_renormalize(psi.size, dx, _ptr(psi))
        return psi

    def evolve2d(self, psi, V, dx, dy, dt, nsteps, order=2, mass=1.0, hbar=1.0,
                 renormalize=False):
        psi = _c128(psi).copy()
        V = _f64(V)
        dt = complex(dt)
        nx, ny = psi.shape
        rc = self.lib.orc_evolve2d(nx, ny, dx, dy, mass, hbar, dt.real, dt.imag, order, 0,
                                   _ptr(psi), _ptr(V), nsteps)
        assert rc == 0
        if renormalize:
            self.lib.orc_renormalize(psi.size, dx * dy, _ptr(psi))
        return psi

    def norm2(self, psi, dv):
        psi = _c128(psi)
        return self.lib.orc_norm2(psi.size, dv, _ptr(psi))

    def poten(self, psi, V, dv):
        psi, V = _c128(psi), _f64(V)
        return self.lib.orc_poten(psi.size, dv, _ptr(psi), _ptr(V))

    def kinen1d(self, psi, dx, mass=1.0, hbar=1.0, wall=False):
        psi = _c128(psi)
        return self.lib.orc_kinen1d(psi.size, dx, mass, hbar, int(wall), _ptr(psi))

    def kinen2d(self, psi, dx, dy, mass=1.0, hbar=1.0):
        psi = _c128(psi)
        nx, ny = psi.shape
        return self.lib.orc_kinen2d(nx, ny, dx, dy, mass, hbar, _ptr(psi))

    def xavg(self, psi, x0, dx):
        psi = _c128(psi)
        return self.lib.orc_xavg(psi.size, x0, dx, _ptr(psi))

    def norm2_range(self, psi, x0, dx, xa, xb):
        psi = _c128(psi)
        return self.lib.orc_norm2_range(psi.size, x0, dx, xa, xb, _ptr(psi))

    def fft3d(self, x, inverse=False):
        x = _c128(x)
        out = np.empty_like(x)
        nx, ny, nz = x.shape
        assert self.lib.orc_fft3d(nx, ny, nz, int(inverse), _ptr(x), _ptr(out)) == 0
        return out

    def evolve3d(self, psi, V, dx, dy, dz, dt, nsteps, order=2, mass=1.0, hbar=1.0):
        """The 3D split-operator step (SplittingMethod2D's formulas with a third axis)."""
        psi = _c128(psi).copy()
        V = _f64(V)
        dt = complex(dt)
        nx, ny, nz = psi.shape
        assert self.lib.orc_evolve3d(nx, ny, nz, dx, dy, dz, mass, hbar, dt.real, dt.imag, order, _ptr(psi),
                                     _ptr(V), nsteps) == 0
        return psi

    def kinen3d(self, psi, dx, dy, dz, mass=1.0, hbar=1.0):
        psi = _c128(psi)
        nx, ny, nz = psi.shape
        return self.lib.orc_kinen3d(nx, ny, nz, dx, dy, dz, mass, hbar, _ptr(psi))

    def born1d(self, V, x0, x1, en, epsilon, direction=1.0, mass=1.0, hbar=1.0, order=1,
               preconditional=False, preconditioner=1, slow=1.0, computes=1):
        """QuPerturbation1D: init + ``computes`` Compute() calls.  Returns a dict
        with dpsi, psi0, v, epsilon, R, T.  preconditioner: 0 identity,
        1 Vellekoop, 2 Hao1, 3 Hao2."""
        v = _c128(V).copy()
        n = v.size
        dx = (x1 - x0) / n
        psi0 = np.empty(n, np.complex128)
        eps = ctypes.c_double(epsilon)
        rc = self.lib.orc_born_init1d(n, x0, dx, en, direction, mass, hbar, int(preconditional),
                                      preconditioner, ctypes.byref(eps), _ptr(v), _ptr(psi0))
        if rc != 0:
            raise ValueError("world too small for the absorbing layer")
        dpsi = np.zeros(n, np.complex128)
        R, T = ctypes.c_double(), ctypes.c_double()
        for _ in range(computes):
            assert self.lib.orc_born_iter1d(n, dx, en, eps.value, mass, hbar, order,
                                            int(preconditional), preconditioner, slow, _ptr(psi0),
                                            _ptr(v), _ptr(dpsi)) == 0
            self.lib.orc_born_rt1d(n, x0, dx, en, direction, mass, hbar, _ptr(psi0), _ptr(dpsi),
                                   _ptr(v), ctypes.byref(R), ctypes.byref(T))
        return dict(dpsi=dpsi, psi0=psi0, v=v, epsilon=eps.value, R=R.value, T=T.value)

    def born2d(self, V, x0, x1, y0, y1, en, epsilon, dirx=1.0, diry=0.0, mass=1.0, hbar=1.0,
               order=1, preconditional=False, preconditioner=1, slow=1.0, computes=1,
               cosxy=(), ntot=0):
        """QuPerturbation2D: init + ``computes`` Compute() calls; then
        ComputeXSection for each (cosx, cosy) and ComputeTotalXSection(ntot)."""
        v = _c128(V).copy()
        nx, ny = v.shape
        dx, dy = (x1 - x0) / nx, (y1 - y0) / ny
        psi0 = np.empty((nx, ny), np.complex128)
        eps = ctypes.c_double(epsilon)
        rc = self.lib.orc_born_init2d(nx, ny, x0, dx, y0, dy, en, dirx, diry, mass, hbar,
                                      int(preconditional), preconditioner, ctypes.byref(eps),
                                      _ptr(v), _ptr(psi0))
        if rc != 0:
            raise ValueError("world too small for the absorbing layer")
        dpsi = np.zeros((nx, ny), np.complex128)
        dn = ctypes.c_double(0.0)
        for _ in range(computes):
            assert self.lib.orc_born_iter2d(nx, ny, dx, dy, en, eps.value, mass, hbar, order,
                                            int(preconditional), preconditioner, slow, _ptr(psi0),
                                            _ptr(v), _ptr(dpsi), ctypes.byref(dn)) == 0

        def xs(cx, cy):
            return self.lib.orc_born_xsec2d(nx, ny, x0, dx, y0, dy, en, mass, hbar, _ptr(psi0),
                                            _ptr(dpsi), _ptr(v), cx, cy)
        xsec = [xs(cx, cy) for cx, cy in cosxy]
        tot = None
        if ntot > 0:
            tot = sum(xs(np.cos(i * 2 * np.pi / ntot), np.sin(i * 2 * np.pi / ntot))
                      for i in range(ntot)) * (2 * np.pi / ntot)
        return dict(dpsi=dpsi, psi0=psi0, v=v, epsilon=eps.value, delta_norm=dn.value,
                    xsec=xsec, total=tot)

    def splitting_constants(self):
        v = [ctypes.c_double() for _ in range(4)]
        self.lib.orc_splitting_constants(*[ctypes.byref(c) for c in v])
        return tuple(c.value for c in v)


class Stepper2D:
    """A persistent oracle 2D evolver (tables built once), for timing."""

    def __init__(self, orc: "Oracle", psi, V, dx, dy, dt, order=4, mass=1.0, hbar=1.0):
        self.lib = orc.lib
        self.V = _f64(V)
        self.psi = _c128(psi).copy()
        dt = complex(dt)
        nx, ny = self.psi.shape
        self.h = self.lib.orc_ev2d_new(nx, ny, dx, dy, mass, hbar, dt.real, dt.imag, order, _ptr(self.V))
        assert self.h

    def step(self, n):
        self.lib.orc_ev2d_step(self.h, _ptr(self.psi), n)

    def close(self):
        if self.h:
            self.lib.orc_ev2d_free(self.h)
            self.h = None


class Stepper1D:
    def __init__(self, orc: "Oracle", psi, V, dx, dt, order=2, mass=1.0, hbar=1.0):
        self.lib = orc.lib
        self.V = _f64(V)
        self.psi = _c128(psi).copy()
        dt = complex(dt)
        self.h = self.lib.orc_ev1d_new(self.psi.size, dx, mass, hbar, dt.real, dt.imag, order, 0)
        assert self.h

    def step(self, n):
        self.lib.orc_ev1d_step(self.h, _ptr(self.psi), _ptr(self.V), n)

    def close(self):
        if self.h:
            self.lib.orc_ev1d_free(self.h)
            self.h = None


class Reference:
    """The reference's own SplittingMethod1D/2D (compiled from its sources)."""

    def __init__(self, path: str = REF_SO):
        lib = ctypes.CDLL(path)
        lib.ref_evolve1d.argtypes = [_sz, _d, _d, _d, _d, _d, _d, _i, _i, _i, _dp, _dp,
                                     _u64, _u64, _dp, _dp, _dp]
        lib.ref_evolve2d.argtypes = [_sz, _sz, _d, _d, _d, _d, _d, _d, _d, _d, _i, _i, _dp,
                                     _dp, _u64, _u64, _dp, _dp, _dp]
        lib.ref_fft1d.argtypes = [_sz, _i, _dp, _dp]
        lib.ref_fft2d.argtypes = [_sz, _sz, _i, _dp, _dp]
        lib.ref_fft3d.argtypes = [_sz, _sz, _sz, _i, _dp, _dp]
        lib.ref_born1d.argtypes = [_sz, _d, _d, _dp, _d, _d, _d, _d, _d, _i, _i, ctypes.c_char_p,
                                   _d, _i, _dp, _dp, _dp, _dp]
        lib.ref_cal_eval.argtypes = [ctypes.c_char_p, _i, ctypes.POINTER(ctypes.c_char_p), _dp, _dp]
        lib.ref_born2d.argtypes = [_sz, _sz, _d, _d, _d, _d, _dp, _d, _d, _d, _d, _d, _d, _i, _i,
                                   ctypes.c_char_p, _d, _i, _dp, _dp, _dp, _dp, _dp, _i, _dp, _i,
                                   _dp]
        self.lib = lib

    @staticmethod
    def available(path: str = REF_SO) -> bool:
        return os.path.exists(path)

    def fft1d(self, x, inverse=False):
        x = _c128(x)
        out = np.empty_like(x)
        assert self.lib.ref_fft1d(x.size, int(inverse), _ptr(x), _ptr(out)) == 0
        return out

    def fft2d(self, x, inverse=False):
        x = _c128(x)
        out = np.empty_like(x)
        nx, ny = x.shape
        assert self.lib.ref_fft2d(nx, ny, int(inverse), _ptr(x), _ptr(out)) == 0
        return out

    def evolve1d(self, psi, V, x0, x1, dt, batch, calls=1, order=2, mass=1.0, hbar=1.0,
                 wall=False, fnes=False):
        """Returns (psi, norm2, kin, pot) after ``calls`` Step() calls."""
        psi = _c128(psi).copy()
        V = _f64(V)
        dt = complex(dt)
        outs = [ctypes.c_double() for _ in range(3)]
        rc = self.lib.ref_evolve1d(psi.size, x0, x1, mass, hbar, dt.real, dt.imag, order,
                                   int(wall), int(fnes), _ptr(psi), _ptr(V), batch, calls,
                                   *[ctypes.pointer(o) for o in outs])
        assert rc == 0
        return (psi,) + tuple(o.value for o in outs)

    def evolve2d(self, psi, V, x0, x1, y0, y1, dt, batch, calls=1, order=2, mass=1.0,
                 hbar=1.0, fnes=False):
        psi = _c128(psi).copy()
        V = _f64(V)
        dt = complex(dt)
        nx, ny = psi.shape
        outs = [ctypes.c_double() for _ in range(3)]
        rc = self.lib.ref_evolve2d(nx, ny, x0, x1, y0, y1, mass, hbar, dt.real, dt.imag,
                                   order, int(fnes), _ptr(psi), _ptr(V), batch, calls,
                                   *[ctypes.pointer(o) for o in outs])
        assert rc == 0
        return (psi,) + tuple(o.value for o in outs)

    def fft3d(self, x, inverse=False):
        x = _c128(x)
        out = np.empty_like(x)
        nx, ny, nz = x.shape
        assert self.lib.ref_fft3d(nx, ny, nz, int(inverse), _ptr(x), _ptr(out)) == 0
        return out

    def cal_eval(self, expr, variables):
        """The reference's Cal(expr) with the variables set, then Val(); None if it does not parse."""
        names = (ctypes.c_char_p * max(1, len(variables)))(*[k.encode() for k in variables])
        vals = np.array([[complex(v).real, complex(v).imag] for v in variables.values()] or [[0.0, 0.0]])
        out = np.zeros(2)
        rc = self.lib.ref_cal_eval(expr.encode(), len(variables), names, _ptr(vals), _ptr(out))
        return None if rc != 0 else complex(out[0], out[1])

    PRECONDITIONERS = (b"BornIndentity", b"Vellekoop", b"Hao1", b"Hao2")

    def born1d(self, V, x0, x1, en, epsilon, direction=1.0, mass=1.0, hbar=1.0, order=1,
               preconditional=False, preconditioner=1, slow=1.0, computes=1):
        """The reference's QuPerturbation1DImpl (same arguments and result as
        Oracle.born1d)."""
        V = _c128(V)
        n = V.size
        dpsi, psi0, v = (np.zeros(n, np.complex128) for _ in range(3))
        sc = np.zeros(3)
        prec = self.PRECONDITIONERS[preconditioner] if preconditional else None
        rc = self.lib.ref_born1d(n, x0, x1, _ptr(V), en, epsilon, direction, mass, hbar, order,
                                 int(preconditional), prec, slow, computes, _ptr(dpsi), _ptr(psi0),
                                 _ptr(v), _ptr(sc))
        if rc != 0:
            raise ValueError("reference init failed")
        return dict(dpsi=dpsi, psi0=psi0, v=v, epsilon=sc[2], R=sc[0], T=sc[1])

    def born2d(self, V, x0, x1, y0, y1, en, epsilon, dirx=1.0, diry=0.0, mass=1.0, hbar=1.0,
               order=1, preconditional=False, preconditioner=1, slow=1.0, computes=1,
               cosxy=(), ntot=0):
        V = _c128(V)
        nx, ny = V.shape
        dpsi, psi0, v = (np.zeros((nx, ny), np.complex128) for _ in range(3))
        sc = np.zeros(2)
        cs = np.ascontiguousarray(np.asarray(cosxy, dtype=np.float64).reshape(-1, 2))
        xsec = np.zeros(max(len(cs), 1))
        tot = ctypes.c_double(0.0)
        prec = self.PRECONDITIONERS[preconditioner] if preconditional else None
        rc = self.lib.ref_born2d(nx, ny, x0, x1, y0, y1, _ptr(V), en, epsilon, dirx, diry, mass,
                                 hbar, order, int(preconditional), prec, slow, computes,
                                 _ptr(dpsi), _ptr(psi0), _ptr(v), _ptr(sc), _ptr(cs), len(cs),
                                 _ptr(xsec), ntot, ctypes.byref(tot))
        if rc != 0:
            raise ValueError("reference init failed")
        return dict(dpsi=dpsi, psi0=psi0, v=v, epsilon=sc[1], delta_norm=sc[0],
                    xsec=list(xsec[:len(cs)]), total=tot.value if ntot > 0 else None)


def rel_l2(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))
