"""Python mirror of QuSim's Evolver / Options API for the GPU_GB300 device.

Same names, argument meaning and error behaviour as include/QuSim.h:
``Evolver1D.init(psi, force_normalization, dt, force_normalization_each_step,
v, x0, x1, n, b, solver, mass, hbar, opts)`` (QuSim.h:558-563),
``Evolver2D.init(..., x0, x1, nx, y0, y1, ny, ...)`` (QuSim.h:583-589), then
``step() / Norm2() / Time() / PotEn() / KinEn() / GetPsi() / GetV()``.
psi and v may be callables of x (or x, y), sampled on the host at
x_i = x0 + i*dx exactly as QuEvolver1DImpl::InitPsi / InitPotential do
(src/EvolverImpl1D.cpp:33-81, src/EvolverImpl2D.cpp:39-98), or arrays of the
grid values.

Only the split-operator methods on the "GPU_GB300" device are served here;
anything else raises, as the reference raises for unsupported solvers
(src/QuSim.cpp:99).
"""
from __future__ import annotations

import atexit
import ctypes
import weakref
import enum

import numpy as np

from . import _lib
from ._lib import QsgError, check


class BoundaryCondition(enum.Enum):
    Period = 0
    InfiniteWall = 1


class SolverMethod(enum.Enum):
    Unknown = 0
    SplittingMethodO2 = 1
    SplittingMethodO4 = 2
    BornSerise = 3  # the reference's spelling (include/QuSim.h:492)


class Options:
    """Key/value options (include/QuSim.h:286-458).  Gb300() selects this engine."""

    def __init__(self):
        self._kv = {}

    def Gb300(self):
        self._kv["device"] = "GPU_GB300"
        return self

    def Batch(self, n: int):
        self._kv["batch"] = int(n)
        return self

    def Precision(self, p: str):
        if p not in ("fp64", "mixed"):
            raise ValueError(f"invalid precision: {p}")
        self._kv["precision"] = p
        return self

    def Form(self, f: str):
        """complex64 2D state form: "momentum" (default) or "direct" (qsg_set_form)."""
        if f not in ("momentum", "direct"):
            raise ValueError(f"invalid form: {f}")
        self._kv["form"] = f
        return self

    def HbmBudget(self, nbytes: int):
        self._kv["hbm_budget"] = int(nbytes)
        return self

    def DeviceOrdinal(self, i: int):
        self._kv["device_ordinal"] = int(i)
        return self

    # Born-series options (include/QuSim.h:288-333)
    def Order(self, n: int):
        self._kv["order"] = int(n)
        return self

    def Preconditional(self, v: bool):
        self._kv["preconditional"] = bool(v)
        return self

    def Slow(self, v: float):
        self._kv["slow"] = float(v)
        return self

    def VellekoopPreconditioner(self):
        self._kv["preconditioner"] = "Vellekoop"
        return self

    def Hao1Preconditioner(self):
        self._kv["preconditioner"] = "Hao1"
        return self

    def Hao2Preconditioner(self):
        self._kv["preconditioner"] = "Hao2"
        return self

    def BornIdentityPreconditioner(self):
        self._kv["preconditioner"] = "BornIndentity"
        return self

    def SetInt(self, k, v):
        self._kv[k] = int(v)

    def SetString(self, k, v):
        self._kv[k] = str(v)

    def SetReal(self, k, v):
        self._kv[k] = float(v)

    def SetBool(self, k, v):
        self._kv[k] = bool(v)

    def get(self, k, default=None):
        return self._kv.get(k, default)


_live_contexts = weakref.WeakSet()


@atexit.register
def _close_contexts():
    # at interpreter exit, while the CUDA runtime is still up: every context
    # closes its instances, batches and solvers, then itself
    for c in list(_live_contexts):
        try:
            c.close()
        except Exception:
            pass


class Context:
    """One qsg_ctx (a device, a stream, an HBM budget)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        lib = _lib.load()
        h = ctypes.c_void_p()
        check(lib.qsg_init(device, hbm_budget, ctypes.byref(h)))
        self.h = h
        self.lib = lib
        self._children = weakref.WeakSet()
        _live_contexts.add(self)

    def _adopt(self, obj):
        """obj (an instance, batch or solver of this context) is closed before the context."""
        self._children.add(obj)

    def close(self):
        if self.h:
            for c in list(self._children):
                c.close()
            self.lib.qsg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return self.lib.qsg_ctx_stream(self.h) or 0

    def bytes_in_use(self) -> int:
        return self.lib.qsg_ctx_bytes_in_use(self.h)

    def profile(self, on):
        """on: True / 1 times every launch with CUDA events; 2 counts launches only; False / 0 off."""
        check(self.lib.qsg_profile_enable(self.h, int(on)))

    def profile_read(self):
        n = self.lib.qsg_profile_read(self.h, 0, None, None, None)
        names = (ctypes.c_char_p * max(n, 1))()
        launches = (ctypes.c_uint64 * max(n, 1))()
        ms = (ctypes.c_double * max(n, 1))()
        n = self.lib.qsg_profile_read(self.h, n, names, launches, ms)
        return {names[i].decode(): (int(launches[i]), float(ms[i])) for i in range(n)}


_default_ctx = {}


def default_context(device: int = 0) -> Context:
    if device not in _default_ctx:
        _default_ctx[device] = Context(device)
    return _default_ctx[device]


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def candidate_plans_1d(precision, n, boundary=_lib.QSG_PERIOD, lib=None):
    """qsg_candidate_plans_1d: the Plan1D list of a 1D instance shape (host
    logic only; precision 0/1 or "fp64"/"mixed")."""
    lib = lib or _lib.load()
    prec = precision if isinstance(precision, int) else (1 if precision == "mixed" else 0)
    b = getattr(boundary, "value", boundary)
    k = lib.qsg_candidate_plans_1d(prec, n, b, None, 0)
    arr = (_lib.Plan1D * max(k, 1))()
    k = lib.qsg_candidate_plans_1d(prec, n, b, arr, k)
    return [arr[i] for i in range(k)]


class Instance:
    """One qsg_inst: a wavefunction resident on the device."""

    def __init__(self, ctx: Context, handle, shape, dv, prec=0):
        self.ctx = ctx
        self.h = handle
        self.shape = shape
        self.dv = dv
        self._prec = prec
        self._boundary = _lib.QSG_PERIOD
        ctx._adopt(self)

    @classmethod
    def create_1d(cls, ctx, psi0, V, dx, dt, order=2, precision="fp64", mass=1.0, hbar=1.0,
                  boundary=BoundaryCondition.Period):
        psi0 = np.ascontiguousarray(psi0, dtype=np.complex128)
        V = np.ascontiguousarray(V, dtype=np.float64)
        if psi0.ndim != 1 or V.shape != psi0.shape:
            raise ValueError("psi0 and V must be 1D arrays of the same length")
        dt = complex(dt)
        h = ctypes.c_void_p()
        check(ctx.lib.qsg_create_1d(ctx.h, psi0.size, dx, mass, hbar, dt.real, dt.imag, order,
                                    _lib.QSG_MIXED if precision == "mixed" else _lib.QSG_FP64,
                                    boundary.value, _dptr(psi0.view(np.float64)), _dptr(V),
                                    ctypes.byref(h)))
        inst = cls(ctx, h, psi0.shape, dx, 1 if precision == "mixed" else 0)
        inst._boundary = boundary.value
        return inst

    @classmethod
    def create_1d_spec(cls, ctx, spec, n, dx, dt, order=2, precision="fp64", mass=1.0, hbar=1.0,
                       boundary=BoundaryCondition.Period):
        """psi0 and V sampled on the device from a _lib.Spec (no host arrays)."""
        dt = complex(dt)
        h = ctypes.c_void_p()
        check(ctx.lib.qsg_create_1d_spec(ctx.h, n, dx, mass, hbar, dt.real, dt.imag, order,
                                         _lib.QSG_MIXED if precision == "mixed" else _lib.QSG_FP64,
                                         boundary.value, ctypes.byref(spec), ctypes.byref(h)))
        inst = cls(ctx, h, (n,), dx, 1 if precision == "mixed" else 0)
        inst._boundary = boundary.value
        return inst

    @classmethod
    def create_2d_spec(cls, ctx, spec, nx, ny, dx, dy, dt, order=2, precision="fp64", mass=1.0, hbar=1.0):
        dt = complex(dt)
        h = ctypes.c_void_p()
        check(ctx.lib.qsg_create_2d_spec(ctx.h, nx, ny, dx, dy, mass, hbar, dt.real, dt.imag, order,
                                         _lib.QSG_MIXED if precision == "mixed" else _lib.QSG_FP64,
                                         ctypes.byref(spec), ctypes.byref(h)))
        return cls(ctx, h, (nx, ny), dx * dy, 1 if precision == "mixed" else 0)

    @classmethod
    def create_1d_expr(cls, ctx, psi_expr, v_expr, n, x0, x1, dt, order=2, precision="fp64", mass=1.0, hbar=1.0,
                       boundary=BoundaryCondition.Period, normalize=True):
        """psi0 and V from expressions of the reference's calculator language
        (FunctorWrapper strings), sampled on the device at x_i = x0 + i dx."""
        dt = complex(dt)
        dx = (x1 - x0) / n
        h = ctypes.c_void_p()
        check(ctx.lib.qsg_create_1d_expr(ctx.h, n, x0, dx, mass, hbar, dt.real, dt.imag, order,
                                         _lib.QSG_MIXED if precision == "mixed" else _lib.QSG_FP64, boundary.value,
                                         psi_expr.encode(), v_expr.encode(), int(normalize), ctypes.byref(h)))
        inst = cls(ctx, h, (n,), dx, 1 if precision == "mixed" else 0)
        inst._boundary = boundary.value
        return inst

    @classmethod
    def create_2d_expr(cls, ctx, psi_expr, v_expr, nx, ny, x0, x1, y0, y1, dt, order=2, precision="fp64", mass=1.0,
                       hbar=1.0, normalize=True):
        """2D: Functor2DWrapper strings in x and y, sampled at (x0 + i dx, y0 + j dy)."""
        dt = complex(dt)
        dx, dy = (x1 - x0) / nx, (y1 - y0) / ny
        h = ctypes.c_void_p()
        check(ctx.lib.qsg_create_2d_expr(ctx.h, nx, ny, x0, y0, dx, dy, mass, hbar, dt.real, dt.imag, order,
                                         _lib.QSG_MIXED if precision == "mixed" else _lib.QSG_FP64,
                                         psi_expr.encode(), v_expr.encode(), int(normalize), ctypes.byref(h)))
        return cls(ctx, h, (nx, ny), dx * dy, 1 if precision == "mixed" else 0)

    @classmethod
    def create_3d(cls, ctx, psi0, V, dx, dy, dz, dt, order=2, precision="fp64", mass=1.0, hbar=1.0):
        """A 3D instance (index (ix*ny + iy)*nz + iz; qsg_create_3d)."""
        psi0 = np.ascontiguousarray(psi0, dtype=np.complex128)
        V = np.ascontiguousarray(V, dtype=np.float64)
        if psi0.ndim != 3 or V.shape != psi0.shape:
            raise ValueError("psi0 and V must be 3D arrays of the same shape (nx, ny, nz)")
        dt = complex(dt)
        nx, ny, nz = psi0.shape
        h = ctypes.c_void_p()
        check(ctx.lib.qsg_create_3d(ctx.h, nx, ny, nz, dx, dy, dz, mass, hbar, dt.real, dt.imag, order,
                                    _lib.QSG_MIXED if precision == "mixed" else _lib.QSG_FP64,
                                    _dptr(psi0.view(np.float64)), _dptr(V), ctypes.byref(h)))
        return cls(ctx, h, psi0.shape, dx * dy * dz, 1 if precision == "mixed" else 0)

    @classmethod
    def create_2d(cls, ctx, psi0, V, dx, dy, dt, order=2, precision="fp64", mass=1.0, hbar=1.0):
        psi0 = np.ascontiguousarray(psi0, dtype=np.complex128)
        V = np.ascontiguousarray(V, dtype=np.float64)
        if psi0.ndim != 2 or V.shape != psi0.shape:
            raise ValueError("psi0 and V must be 2D arrays of the same shape (nx, ny)")
        dt = complex(dt)
        nx, ny = psi0.shape
        h = ctypes.c_void_p()
        check(ctx.lib.qsg_create_2d(ctx.h, nx, ny, dx, dy, mass, hbar, dt.real, dt.imag, order,
                                    _lib.QSG_MIXED if precision == "mixed" else _lib.QSG_FP64,
                                    _dptr(psi0.view(np.float64)), _dptr(V), ctypes.byref(h)))
        return cls(ctx, h, psi0.shape, dx * dy, 1 if precision == "mixed" else 0)

    def step(self, nsteps: int, renormalize: bool = False):
        check(self.ctx.lib.qsg_step(self.h, nsteps, int(renormalize)))

    def sync(self):
        check(self.ctx.lib.qsg_sync(self.h))

    def norm2(self) -> float:
        v = ctypes.c_double()
        check(self.ctx.lib.qsg_norm2(self.h, ctypes.byref(v)))
        return v.value

    def step_norm2(self) -> float:
        """Norm2 as the last step summed it (qsg_step_norm2): no pass over psi
        for a 2D real-time instance; equal to norm2() up to rounding."""
        v = ctypes.c_double()
        check(self.ctx.lib.qsg_step_norm2(self.h, ctypes.byref(v)))
        return v.value

    def post_step_norm2(self) -> int:
        """Queue the step's Norm2 for reading without stalling the stream; returns a ticket."""
        t = ctypes.c_uint64()
        check(self.ctx.lib.qsg_step_norm2_post(self.h, ctypes.byref(t)))
        return t.value

    def get_step_norm2(self, ticket: int) -> float:
        """The Norm2 posted under `ticket` (waits for that copy only)."""
        v = ctypes.c_double()
        check(self.ctx.lib.qsg_step_norm2_get(self.h, ticket, ctypes.byref(v)))
        return v.value

    def energies(self):
        k, p = ctypes.c_double(), ctypes.c_double()
        check(self.ctx.lib.qsg_energies(self.h, ctypes.byref(k), ctypes.byref(p)))
        return k.value, p.value

    def xavg(self, x0: float) -> float:
        v = ctypes.c_double()
        check(self.ctx.lib.qsg_xavg(self.h, x0, ctypes.byref(v)))
        return v.value

    def norm2_range(self, x0, xa, xb) -> float:
        v = ctypes.c_double()
        check(self.ctx.lib.qsg_norm2_range(self.h, x0, xa, xb, ctypes.byref(v)))
        return v.value

    def get_psi(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.shape, dtype=np.complex128)
        check(self.ctx.lib.qsg_get_psi(self.h, _dptr(out.view(np.float64))))
        return out

    def set_psi(self, psi):
        psi = np.ascontiguousarray(psi, dtype=np.complex128).reshape(self.shape)
        check(self.ctx.lib.qsg_set_psi(self.h, _dptr(psi.view(np.float64))))

    def plan(self):
        """The execution plan in use: Plan2D for 2D instances, Plan1D for 1D."""
        if len(self.shape) == 1:
            p = _lib.Plan1D()
            check(self.ctx.lib.qsg_get_plan_1d(self.h, ctypes.byref(p)))
            return p
        p = _lib.Plan2D()
        check(self.ctx.lib.qsg_get_plan(self.h, ctypes.byref(p)))
        return p

    def set_plan(self, plan):
        """Switch plans between steps (a Plan2D / Plan1D or its tuple)."""
        if len(self.shape) == 1:
            if not isinstance(plan, _lib.Plan1D):
                plan = _lib.Plan1D(*plan)
            check(self.ctx.lib.qsg_set_plan_1d(self.h, ctypes.byref(plan)))
            return
        if not isinstance(plan, _lib.Plan2D):
            plan = _lib.Plan2D(*plan)
        check(self.ctx.lib.qsg_set_plan(self.h, ctypes.byref(plan)))

    def check_wait_timeout(self) -> int:
        """qsg_check_wait_timeout: run one column pass with its tensor copies
        withheld; returns the status code (4, QSG_ERR_TIMEOUT, when the bounded
        waits work)."""
        return int(self.ctx.lib.qsg_check_wait_timeout(self.h))

    @property
    def form(self):
        """"momentum" (complex64 2D default: state kept in momentum space,
        potential factors added as increments) or "direct"."""
        v = ctypes.c_int(0)
        check(self.ctx.lib.qsg_get_form(self.h, ctypes.byref(v)))
        return "momentum" if v.value == _lib.QSG_FORM_MOMENTUM else "direct"

    @form.setter
    def form(self, name):
        code = {"momentum": _lib.QSG_FORM_MOMENTUM, "direct": _lib.QSG_FORM_DIRECT}[name]
        check(self.ctx.lib.qsg_set_form(self.h, code))

    def candidate_plans(self, precision=None):
        lib = self.ctx.lib
        prec = self._prec if precision is None else (1 if precision == "mixed" else 0)
        if len(self.shape) == 1:
            return candidate_plans_1d(prec, self.shape[0], self._boundary, lib)
        nx, ny = self.shape
        n = lib.qsg_candidate_plans(prec, nx, ny, None, 0)
        arr = (_lib.Plan2D * max(n, 1))()
        n = lib.qsg_candidate_plans(prec, nx, ny, arr, n)
        return [arr[i] for i in range(n)]

    def autotune(self, trial_steps: int = 4, persist: bool = True):
        """Time every plan on a copy of the state, switch to the fastest; returns (plan, ms/step)."""
        ms = ctypes.c_double()
        if len(self.shape) == 1:
            p = _lib.Plan1D()
            check(self.ctx.lib.qsg_autotune_1d(self.h, trial_steps, int(persist), ctypes.byref(p),
                                               ctypes.byref(ms)))
            return p, ms.value
        p = _lib.Plan2D()
        check(self.ctx.lib.qsg_autotune(self.h, trial_steps, int(persist), ctypes.byref(p), ctypes.byref(ms)))
        return p, ms.value

    def steps_taken(self) -> int:
        v = ctypes.c_uint64()
        check(self.ctx.lib.qsg_steps_taken(self.h, ctypes.byref(v)))
        return v.value

    def close(self):
        # views of batch members (Batch.instance) do not own their handle
        if self.h and getattr(self, "_owned", True):
            self.ctx.lib.qsg_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """qsg_batch: many independent 1D instances (mixed sizes) advanced together."""

    def __init__(self, ctx: Context, psis, Vs, dxs, dts, order=2, precision="fp64", mass=1.0, hbar=1.0):
        lib = ctx.lib
        self.ctx = ctx
        psis = [np.ascontiguousarray(p, dtype=np.complex128) for p in psis]
        Vs = [np.ascontiguousarray(v, dtype=np.float64) for v in Vs]
        cnt = len(psis)
        if not (len(Vs) == len(dxs) == len(dts) == cnt):
            raise ValueError("psis, Vs, dxs, dts must have the same length")
        n = (ctypes.c_uint64 * cnt)(*[p.size for p in psis])
        dx = (ctypes.c_double * cnt)(*[float(v) for v in dxs])
        dtr = (ctypes.c_double * cnt)(*[complex(v).real for v in dts])
        dti = (ctypes.c_double * cnt)(*[complex(v).imag for v in dts])
        pp = (ctypes.POINTER(ctypes.c_double) * cnt)(*[_dptr(p.view(np.float64)) for p in psis])
        vp = (ctypes.POINTER(ctypes.c_double) * cnt)(*[_dptr(v) for v in Vs])
        h = ctypes.c_void_p()
        check(lib.qsg_batch_create_1d(ctx.h, cnt, n, dx, dtr, dti, mass, hbar, order,
                                      _lib.QSG_MIXED if precision == "mixed" else _lib.QSG_FP64, pp, vp,
                                      ctypes.byref(h)))
        self.h = h
        ctx._adopt(self)
        self._keep = (psis, Vs)
        self.count = cnt
        self.sizes = [p.size for p in psis]
        self._prec = 1 if precision == "mixed" else 0

    def step(self, nsteps: int):
        check(self.ctx.lib.qsg_batch_step(self.h, nsteps))

    def sync(self):
        check(self.ctx.lib.qsg_batch_sync(self.h))

    def sites(self) -> int:
        c, s = ctypes.c_int(), ctypes.c_uint64()
        check(self.ctx.lib.qsg_batch_size(self.h, ctypes.byref(c), ctypes.byref(s)))
        return s.value

    def plan(self, n: int):
        """The Plan1D of the members of length n."""
        p = _lib.Plan1D()
        check(self.ctx.lib.qsg_batch_get_plan_1d(self.h, n, ctypes.byref(p)))
        return p

    def set_plan(self, n: int, plan):
        """Switch the members of length n (a four-step class) to a four-step plan."""
        if not isinstance(plan, _lib.Plan1D):
            plan = _lib.Plan1D(*plan)
        check(self.ctx.lib.qsg_batch_set_plan_1d(self.h, n, ctypes.byref(plan)))

    def autotune(self, trial_steps: int = 8):
        """qsg_batch_autotune: each four-step class timed alone on every four-step
        plan, keeping its fastest; states unchanged.  Returns ({n: Plan1D}, ms/step
        summed over the tuned classes)."""
        ms = ctypes.c_double()
        check(self.ctx.lib.qsg_batch_autotune(self.h, trial_steps, ctypes.byref(ms)))
        return {n: self.plan(n) for n in sorted(set(self.sizes))}, ms.value

    def instance(self, i: int) -> "Instance":
        """A non-owning view of member i (get_psi, norm2, energies, ...)."""
        p = ctypes.c_void_p()
        check(self.ctx.lib.qsg_batch_instance(self.h, i, ctypes.byref(p)))
        v = Instance.__new__(Instance)
        v._owned = False
        v.__init__(self.ctx, p, (self.sizes[i],), 0.0, self._prec)
        return v

    def close(self):
        if self.h:
            self.ctx.lib.qsg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """qsg_server: evolution requests served with continuous batching."""

    QUEUED, RUNNING, DONE, FAILED = 0, 1, 2, 3

    def __init__(self, device: int = 0, hbm_budget: int = 0, max_running: int = 64):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        check(self.lib.qsg_server_create(device, hbm_budget, max_running, ctypes.byref(h)))
        self.h = h
        _live_contexts.add(self)  # closed at exit with the contexts
        self._shapes = {}

    def submit_spec(self, spec, shape, dx, dt, nsteps, order=2, precision="mixed", dy=None, mass=1.0, hbar=1.0):
        """A request whose psi0 and V are sampled on the device from a _lib.Spec."""
        shape = tuple(int(v) for v in shape)
        if len(shape) not in (1, 2):
            raise ValueError("shape: (n,) or (nx, ny)")
        dt = complex(dt)
        r = _lib.Request()
        r.dim = len(shape)
        r.order = order
        r.precision = _lib.QSG_MIXED if precision == "mixed" else _lib.QSG_FP64
        r.nx = shape[0]
        r.ny = shape[1] if len(shape) == 2 else 1
        r.dx = dx
        r.dy = dy if dy is not None else dx
        r.mass, r.hbar, r.dt_re, r.dt_im = mass, hbar, dt.real, dt.imag
        r.nsteps = nsteps
        r.spec = ctypes.pointer(spec)
        i = ctypes.c_uint64()
        check(self.lib.qsg_server_submit(self.h, ctypes.byref(r), ctypes.byref(i)))
        self._shapes[i.value] = shape
        return i.value

    def submit(self, psi0, V, dx, dt, nsteps, order=2, precision="mixed", dy=None, mass=1.0, hbar=1.0):
        psi0 = np.ascontiguousarray(psi0, dtype=np.complex128)
        V = np.ascontiguousarray(V, dtype=np.float64)
        if V.shape != psi0.shape or psi0.ndim not in (1, 2):
            raise ValueError("psi0 and V: same 1D or 2D shape")
        dt = complex(dt)
        r = _lib.Request()
        r.dim = psi0.ndim
        r.order = order
        r.precision = _lib.QSG_MIXED if precision == "mixed" else _lib.QSG_FP64
        r.nx = psi0.shape[0]
        r.ny = psi0.shape[1] if psi0.ndim == 2 else 1
        r.dx = dx
        r.dy = dy if dy is not None else dx
        r.mass, r.hbar, r.dt_re, r.dt_im = mass, hbar, dt.real, dt.imag
        r.nsteps = nsteps
        r.psi0 = _dptr(psi0.view(np.float64))
        r.V = _dptr(V)
        i = ctypes.c_uint64()
        check(self.lib.qsg_server_submit(self.h, ctypes.byref(r), ctypes.byref(i)))
        self._shapes[i.value] = psi0.shape
        return i.value

    def poll(self, rid):
        st = ctypes.c_int()
        check(self.lib.qsg_server_poll(self.h, rid, ctypes.byref(st)))
        return st.value

    def wait(self, rid, timeout=600.0):
        st = ctypes.c_int()
        check(self.lib.qsg_server_wait(self.h, rid, timeout, ctypes.byref(st)))
        return st.value

    def take(self, rid):
        """(psi, latency seconds); raises QsgError for a failed request."""
        out = np.empty(self._shapes[rid], dtype=np.complex128)
        lat = ctypes.c_double()
        rc = self.lib.qsg_server_take(self.h, rid, _dptr(out.view(np.float64)), ctypes.byref(lat))
        self._shapes.pop(rid, None)
        check(rc)
        return out, lat.value

    def stats(self):
        s = _lib.ServerInfo()
        check(self.lib.qsg_server_stats(self.h, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_ if f != "reserved"}

    def request_info(self, rid):
        """Progress of a request not yet taken: state, admitted_mid_flight, chunks,
        steps_dispatched and the t_submit / t_admit / t_first_dispatch / t_finish
        times (seconds since the server started, -1 where not reached)."""
        s = _lib.RequestInfo()
        check(self.lib.qsg_server_request_info(self.h, rid, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def close(self):
        if self.h:
            self.lib.qsg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _check_device(opts: Options):
    dev = opts.get("device", "CPU_SEQ")
    if dev != "GPU_GB300":
        # the reference's GetDeviceType raises std::invalid_argument for unknown
        # devices (src/DeviceType.h:21); here only GPU_GB300 is served
        raise ValueError(f"invalid device: {dev} (this package serves device GPU_GB300; "
                         "select it with Options().Gb300())")


class Evolver:
    def __init__(self):
        self._inst = None
        self._fnes = False
        self._batch = 1
        self._dt = 0j
        self._method = SolverMethod.Unknown
        self._psi_cache = None
        self._V = None

    def step(self):
        """Evolver::step (src/QuSim.cpp:39-42 -> EvolverImpl.cpp:56-68): `batch` steps,
        then renormalise if force_normalization_each_step."""
        self._inst.step(self._batch, self._fnes)
        self._psi_cache = None

    def Norm2(self, *args):
        return self._inst.norm2()

    def Time(self):
        return (self._inst.steps_taken() * self._dt).real

    def PotEn(self):
        return self._inst.energies()[1]

    def KinEn(self):
        return self._inst.energies()[0]

    def GetMethod(self):
        return self._method

    def _common(self, dt, fnes, solver, opts):
        _check_device(opts)
        if solver not in (SolverMethod.SplittingMethodO2, SolverMethod.SplittingMethodO4):
            raise RuntimeError("unspported solver")
        self._dt = complex(dt)
        self._fnes = bool(fnes)
        self._batch = int(opts.get("batch", 1))
        self._method = solver
        order = 2 if solver == SolverMethod.SplittingMethodO2 else 4
        precision = opts.get("precision", "fp64")
        ctx = default_context(opts.get("device_ordinal", 0))
        return ctx, order, precision


def _normalise(psi, dv):
    return psi / np.sqrt(np.sum(np.abs(psi) ** 2) * dv)


class Evolver1D(Evolver):
    def init(self, psi, force_normalization, dt, force_normalization_each_step, v, x0, x1, n,
             b, solver, mass, hbar, opts):
        ctx, order, precision = self._common(dt, force_normalization_each_step, solver, opts)
        n = int(n)
        dx = (x1 - x0) / n
        xs = dx * np.arange(n) + x0
        psi0 = np.asarray([psi(x) for x in xs] if callable(psi) else psi, dtype=np.complex128)
        V = np.real(np.asarray([v(x) for x in xs] if callable(v) else v)).astype(np.float64)
        if force_normalization:
            psi0 = _normalise(psi0, dx)
        self._x0, self._x1, self._n, self._dx = x0, x1, n, dx
        self._V = V
        self._inst = Instance.create_1d(ctx, psi0, V, dx, dt, order, precision, mass, hbar, b)

    def GetPsi(self):
        if self._psi_cache is None:
            self._psi_cache = self._inst.get_psi()
        return self._psi_cache

    def GetV(self):
        return self._V

    def Xavg(self):
        return self._inst.xavg(self._x0)

    def GetN(self):
        return self._n

    def GetX0(self):
        return self._x0

    def GetX1(self):
        return self._x1

    def Norm2(self, *args):
        if len(args) == 2:
            return self._inst.norm2_range(self._x0, args[0], args[1])
        return self._inst.norm2()


class Evolver2D(Evolver):
    def init(self, psi, force_normalization, dt, force_normalization_each_step, v, x0, x1, nx,
             y0, y1, ny, b, solver, mass, hbar, opts):
        ctx, order, precision = self._common(dt, force_normalization_each_step, solver, opts)
        if b != BoundaryCondition.Period:
            raise RuntimeError("unsupported boundary condition!")
        nx, ny = int(nx), int(ny)
        dx, dy = (x1 - x0) / nx, (y1 - y0) / ny
        if callable(psi) or callable(v):
            xs = dx * np.arange(nx) + x0
            ys = dy * np.arange(ny) + y0
        psi0 = (np.array([[psi(x, y) for y in ys] for x in xs], dtype=np.complex128)
                if callable(psi) else np.asarray(psi, dtype=np.complex128))
        V = (np.real(np.array([[v(x, y) for y in ys] for x in xs]))
             if callable(v) else np.real(np.asarray(v))).astype(np.float64)
        if force_normalization:
            psi0 = _normalise(psi0, dx * dy)
        self._nx, self._ny = nx, ny
        self._V = V
        self._inst = Instance.create_2d(ctx, psi0, V, dx, dy, dt, order, precision, mass, hbar)
        if precision == "mixed":
            self._inst.form = opts.get("form", "momentum")

    def GetPsi(self):
        if self._psi_cache is None:
            self._psi_cache = self._inst.get_psi()
        return self._psi_cache

    def GetV(self):
        return self._V

    def GetNx(self):
        return self._nx

    def GetNy(self):
        return self._ny


__all__ = ["BoundaryCondition", "SolverMethod", "Options", "Context", "Instance", "Batch", "Server", "Evolver1D",
           "Evolver2D", "QsgError", "default_context"]


class Calculator:
    """The reference's Calculator (include/QuSim.h:527-538): an expression of
    the calculator language with variables set by SetVaraible (the reference's
    spelling) and evaluated on the host by libqsg.so (qsg_expr_eval)."""

    def __init__(self, expr: str):
        self.expr = expr
        self.vars = {}
        self.lib = _lib.load()
        # syntax errors surface here, as the reference's constructor throws;
        # variables are set after construction, so an undefined one waits for Evaluate
        self._eval(allow_undefined=True)

    def SetVaraible(self, name, value):
        self.vars[name] = complex(value)
        return self.vars[name]

    def GetVaraible(self, name):
        return self.vars[name]

    def _eval(self, allow_undefined=False):
        names = (ctypes.c_char_p * max(1, len(self.vars)))(*[k.encode() for k in self.vars])
        vals = np.array([[v.real, v.imag] for v in self.vars.values()] or [[0.0, 0.0]], dtype=np.float64)
        out = np.zeros(2)
        rc = self.lib.qsg_expr_eval(self.expr.encode(), len(self.vars), names, _dptr(vals), _dptr(out))
        if allow_undefined and rc == _lib.QSG_ERR_ARG and b"var not defined" in self.lib.qsg_last_error():
            return None
        check(rc)
        return complex(out[0], out[1])

    def Evaluate(self):
        return self._eval()


class FunctorWrapper:
    """psi(x) / V(x) from an expression string (include/QuSim.h:506-516)."""

    def __init__(self, expr: str):
        self.expr = expr
        self._c = Calculator(expr)

    def __call__(self, x):
        self._c.SetVaraible("x", x)
        return self._c.Evaluate()


class Functor2DWrapper:
    """psi(x, y) / V(x, y) from an expression string (include/QuSim.h:518-525)."""

    def __init__(self, expr: str):
        self.expr = expr
        self._c = Calculator(expr)

    def __call__(self, x, y):
        self._c.SetVaraible("x", x)
        self._c.SetVaraible("y", y)
        return self._c.Evaluate()
