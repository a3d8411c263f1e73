"""Born-series scattering solvers on the GB300 engine: a mirror of the
reference's QuPerturbation1D / QuPerturbation2D (include/QuSim.h:643-806,
src/QuSim.cpp:405-630) over the qsg_born_* C ABI.

    from qusim_gb300 import QuPerturbation1D, Options, SolverMethod
    per = QuPerturbation1D()
    per.init(lambda x: 0.5 * np.exp(-x * x), -100, 100, 2048, 0.5, 0.51, 1,
             SolverMethod.BornSerise, 1, 1, Options().Order(5).Preconditional(True))
    per.Compute()
    per.GetR(), per.GetT()

Options keys read: "order", "preconditional", "preconditioner", "slow"
(src/PerturbationOptions.cpp:8-43), plus "precision" ("fp64" or "mixed") and
"device_ordinal".  One difference from the reference: its
OptionsImpl::GetBool(key, default) (src/OptionsImpl.cpp:88-91) returns
whether the key is present, so Options().Preconditional(False) selects the
preconditioned series there; here the value is used.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import check
from .evolver import Options, SolverMethod, _check_device, default_context

_PRECONDITIONERS = {"Vellekoop": _lib.QSG_BORN_VELLEKOOP, "Hao1": _lib.QSG_BORN_HAO1,
                    "Hao2": _lib.QSG_BORN_HAO2, "BornIndentity": _lib.QSG_BORN_IDENTITY}


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def born_opts(opts: Options) -> _lib.BornOpts:
    """qsg_born_opts from the reference's option keys."""
    o = _lib.BornOpts()
    _lib.load().qsg_born_default_opts(ctypes.byref(o))
    o.order = int(opts.get("order", 1))
    o.preconditional = int(bool(opts.get("preconditional", False)))
    o.slow = float(opts.get("slow", 1.0))
    pre = opts.get("preconditioner")
    if pre is not None:
        if pre not in _PRECONDITIONERS:
            raise RuntimeError("Unknown preconditioner")
        o.preconditioner = _PRECONDITIONERS[pre]
    return o


def _precision(opts: Options) -> int:
    p = opts.get("precision", "fp64")
    return _lib.QSG_MIXED if p == "mixed" else _lib.QSG_FP64


class _ScatteringSolver:
    def __init__(self):
        self.h = None

    def _check_met(self, met):
        if met != SolverMethod.BornSerise:
            raise RuntimeError("not support method!")
        self._met = met

    def close(self):
        if self.h:
            _lib.load().qsg_born_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def Compute(self):
        check(self.lib.qsg_born_compute(self.h))

    def GetEnergy(self):
        return self._en

    def GetMomentum(self):
        return np.sqrt(2 * self._mass * self._en)

    def GetMethod(self):
        return self._met

    def GetEpsilon(self):
        e = ctypes.c_double()
        check(self.lib.qsg_born_epsilon(self.h, ctypes.byref(e)))
        return e.value

    def _get(self, what):
        out = np.empty(self._shape, np.complex128)
        check(self.lib.qsg_born_get(self.h, what, _dptr(out.view(np.float64))))
        return out

    def GetPsi(self):
        """The scattered part of the wave function."""
        return self._get(_lib.QSG_BORN_PSI)

    def GetPsi0(self):
        return self._get(_lib.QSG_BORN_PSI0)

    def GetV(self):
        return self._get(_lib.QSG_BORN_V)


class QuPerturbation1D(_ScatteringSolver):
    def init(self, v, x0, x1, n, en, epsilon, direction, met, mass, hbar, opts: Options):
        """v: a callable V(x) (complex) or an array of n samples at x0 + i dx."""
        _check_device(opts)
        self._check_met(met)
        n = int(n)
        dx = (x1 - x0) / n
        xs = x0 + dx * np.arange(n)
        V = np.ascontiguousarray(np.asarray([v(x) for x in xs] if callable(v) else v, dtype=np.complex128))
        ctx = default_context(opts.get("device_ordinal", 0))
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        o = born_opts(opts)
        check(self.lib.qsg_born_create_1d(ctx.h, n, x0, x1, _dptr(V.view(np.float64)), en, epsilon, direction,
                                          mass, hbar, ctypes.byref(o), _precision(opts), ctypes.byref(h)))
        self.h = h
        self._ctx = ctx
        ctx._adopt(self)
        self._shape = (n,)
        self._n, self._dx, self._en, self._mass, self._hbar = n, dx, float(en), float(mass), float(hbar)

    def GetNPoints(self):
        return self._n

    def GetR(self):
        r, t = ctypes.c_double(), ctypes.c_double()
        check(self.lib.qsg_born_rt(self.h, ctypes.byref(r), ctypes.byref(t)))
        return r.value

    def GetT(self):
        r, t = ctypes.c_double(), ctypes.c_double()
        check(self.lib.qsg_born_rt(self.h, ctypes.byref(r), ctypes.byref(t)))
        return t.value

    # src/Perturbation1DImpl.h:22-61
    def GetMaxMomentum(self):
        return 2 * np.pi / self._dx * self._hbar

    def GetMaxEnergy(self):
        return 0.5 * self.GetMaxMomentum() ** 2 / self._mass

    def GetMomentumGap(self):
        return 2 * np.pi / (self._dx * self._n) * self._hbar

    def GetEpsilonMomentumWidth(self):
        return self._mass * abs(self.GetEpsilon()) / np.sqrt(2 * self._mass * self._en)

    def GetEnergyGap(self):
        return np.sqrt(2 * self._mass * self._en) / self._mass * self.GetMomentumGap()

    def GetEpsilonDecayLength(self):
        return 2 * np.pi / (self.GetMomentum() / self._hbar * self.GetEpsilon() / (2 * self._en))

    def GetEpsilonBoundaryError(self):
        return np.exp(-(self._n * self._dx / 2) * (self.GetMomentum() / self._hbar) * self.GetEpsilon()
                      / (2 * self._en))


class QuPerturbation2D(_ScatteringSolver):
    def init(self, v, x0, x1, nx, y0, y1, ny, en, epsilon, directionx, directiony, met, mass, hbar,
             opts: Options):
        """v: a callable V(x, y) (complex) or an (nx, ny) array (index iy + ix*ny)."""
        _check_device(opts)
        self._check_met(met)
        nx, ny = int(nx), int(ny)
        dx, dy = (x1 - x0) / nx, (y1 - y0) / ny
        if callable(v):
            xs = x0 + dx * np.arange(nx)
            ys = y0 + dy * np.arange(ny)
            V = np.array([[v(x, y) for y in ys] for x in xs], dtype=np.complex128)
        else:
            V = np.asarray(v, dtype=np.complex128).reshape(nx, ny)
        V = np.ascontiguousarray(V)
        ctx = default_context(opts.get("device_ordinal", 0))
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        o = born_opts(opts)
        check(self.lib.qsg_born_create_2d(ctx.h, nx, ny, x0, x1, y0, y1, _dptr(V.view(np.float64)), en, epsilon,
                                          directionx, directiony, mass, hbar, ctypes.byref(o), _precision(opts),
                                          ctypes.byref(h)))
        self.h = h
        self._ctx = ctx
        ctx._adopt(self)
        self._shape = (nx, ny)
        self._en, self._mass, self._hbar = float(en), float(mass), float(hbar)

    def ComputeXSection(self, cosx, cosy):
        return float(self.ComputeXSections([(cosx, cosy)])[0])

    def ComputeXSections(self, cosxy):
        """ComputeXSection for many directions in one pass over the grid."""
        cs = np.ascontiguousarray(np.asarray(cosxy, dtype=np.float64).reshape(-1, 2))
        out = np.empty(len(cs))
        check(self.lib.qsg_born_xsection(self.h, len(cs), _dptr(cs), _dptr(out)))
        return out

    def ComputeTotalXSection(self, n):
        out = ctypes.c_double()
        check(self.lib.qsg_born_total_xsection(self.h, int(n), ctypes.byref(out)))
        return out.value

    def GetDeltaPsiNorm(self):
        out = ctypes.c_double()
        check(self.lib.qsg_born_delta_norm(self.h, ctypes.byref(out)))
        return out.value
