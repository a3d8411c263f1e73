"""ctypes binding of libqsg.so (include/qsg.h).

The library is the product: there is no fallback.  ``load()`` raises
``QsgError`` if libqsg.so is missing or cannot be loaded.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libqsg.so")

QSG_OK = 0
QSG_ERR_ARG = 1
QSG_ERR_BUDGET = 2
QSG_ERR_CUDA = 3
QSG_ERR_TIMEOUT = 4
QSG_ERR_UNSUPPORTED = 5
QSG_ERR_STATE = 6
QSG_FP64 = 0
QSG_MIXED = 1
QSG_PERIOD = 0
QSG_INFINITE_WALL = 1

STATUS_NAMES = {0: "ok", 1: "bad argument", 2: "out of budget", 3: "cuda error", 4: "timeout",
                5: "unsupported", 6: "bad state"}

# every symbol include/qsg.h declares
EXPORTS = [
    "qsg_version", "qsg_last_error", "qsg_init", "qsg_ctx_destroy", "qsg_ctx_stream",
    "qsg_ctx_bytes_in_use", "qsg_create_1d", "qsg_create_2d", "qsg_step", "qsg_sync",
    "qsg_norm2", "qsg_energies", "qsg_xavg", "qsg_norm2_range", "qsg_get_psi", "qsg_set_psi",
    "qsg_steps_taken", "qsg_destroy", "qsg_candidate_plans", "qsg_get_plan", "qsg_set_plan",
    "qsg_autotune", "qsg_batch_create_1d", "qsg_batch_step", "qsg_batch_sync", "qsg_batch_size",
    "qsg_batch_instance", "qsg_batch_destroy", "qsg_server_create", "qsg_server_submit",
    "qsg_server_poll", "qsg_server_wait", "qsg_server_take", "qsg_server_stats", "qsg_server_request_info",
    "qsg_server_destroy",
    "qsg_profile_enable", "qsg_profile_read", "qsg_norm2_noalloc", "qsg_create_1d_spec", "qsg_create_2d_spec",
    "qsg_born_default_opts", "qsg_born_create_1d", "qsg_born_create_2d", "qsg_born_compute", "qsg_born_get",
    "qsg_born_rt", "qsg_born_delta_norm", "qsg_born_epsilon", "qsg_born_xsection", "qsg_born_total_xsection",
    "qsg_born_destroy", "qsg_step_norm2", "qsg_create_3d", "qsg_step_norm2_post", "qsg_step_norm2_get",
    "qsg_set_form", "qsg_get_form", "qsg_check_wait_timeout", "qsg_create_1d_expr", "qsg_create_2d_expr",
    "qsg_expr_eval", "qsg_candidate_plans_1d", "qsg_get_plan_1d", "qsg_set_plan_1d", "qsg_autotune_1d",
    "qsg_batch_autotune", "qsg_batch_get_plan_1d", "qsg_batch_set_plan_1d",
]

# qsg_form: how a complex64 2D instance holds its state between passes
QSG_FORM_MOMENTUM, QSG_FORM_DIRECT = 0, 1

# qsg_born_preconditioner / qsg_born_field
QSG_BORN_IDENTITY, QSG_BORN_VELLEKOOP, QSG_BORN_HAO1, QSG_BORN_HAO2 = 0, 1, 2, 3
QSG_BORN_PSI, QSG_BORN_PSI0, QSG_BORN_V = 0, 1, 2


SPEC_MAX_BUMPS = 32


class Spec(ctypes.Structure):
    """qsg_spec: psi0 = exp(i k.r) exp(-|r-c|^2/(4 s^2)) (normalised if asked),
    V = v0 + sum_b h exp(-|r-b|^2/(2 w^2)), sampled on the device at x0 + i*dx (, y0 + j*dy)."""
    _fields_ = [("x0", ctypes.c_double), ("y0", ctypes.c_double), ("kx", ctypes.c_double), ("ky", ctypes.c_double),
                ("cx", ctypes.c_double), ("cy", ctypes.c_double), ("s", ctypes.c_double), ("v0", ctypes.c_double),
                ("normalize", ctypes.c_int32), ("nbumps", ctypes.c_int32),
                ("bumps", (ctypes.c_double * 4) * SPEC_MAX_BUMPS)]

    @classmethod
    def make(cls, x0, s, kx=0.0, cx=0.0, y0=0.0, ky=0.0, cy=0.0, bumps=(), v0=0.0, normalize=True):
        """bumps: rows (h, bx, by, w) (by unused in 1D)."""
        sp = cls()
        sp.x0, sp.y0, sp.kx, sp.ky, sp.cx, sp.cy, sp.s, sp.v0 = x0, y0, kx, ky, cx, cy, s, v0
        sp.normalize = 1 if normalize else 0
        bumps = [tuple(float(v) for v in b) for b in bumps]
        if len(bumps) > SPEC_MAX_BUMPS:
            raise ValueError(f"at most {SPEC_MAX_BUMPS} bumps")
        sp.nbumps = len(bumps)
        for i, b in enumerate(bumps):
            for k in range(4):
                sp.bumps[i][k] = b[k]
        return sp


class Request(ctypes.Structure):
    """qsg_request."""
    _fields_ = [("dim", ctypes.c_int32), ("order", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("nx", ctypes.c_uint64), ("ny", ctypes.c_uint64),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("mass", ctypes.c_double),
                ("hbar", ctypes.c_double), ("dt_re", ctypes.c_double), ("dt_im", ctypes.c_double),
                ("nsteps", ctypes.c_uint64), ("psi0", ctypes.POINTER(ctypes.c_double)),
                ("V", ctypes.POINTER(ctypes.c_double)), ("spec", ctypes.POINTER(Spec))]


class ServerInfo(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64), ("site_steps", ctypes.c_uint64),
                ("peak_device_bytes", ctypes.c_size_t), ("budget_bytes", ctypes.c_size_t),
                ("admitted_mid_flight", ctypes.c_uint64), ("max_in_flight", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class RequestInfo(ctypes.Structure):
    """qsg_request_info: one served request's progress (times in s since the server started; -1 = not yet)."""
    _fields_ = [("state", ctypes.c_int32), ("admitted_mid_flight", ctypes.c_int32), ("chunks", ctypes.c_uint64),
                ("steps_dispatched", ctypes.c_uint64), ("t_submit", ctypes.c_double), ("t_admit", ctypes.c_double),
                ("t_first_dispatch", ctypes.c_double), ("t_finish", ctypes.c_double)]


class Plan2D(ctypes.Structure):
    """qsg_plan2d: x split g, row radix and CTA threads, column radix and tile width, row-pass kind."""
    _fields_ = [("g", ctypes.c_int32), ("row_e", ctypes.c_int32), ("row_nt", ctypes.c_int32),
                ("col_e", ctypes.c_int32), ("col_w", ctypes.c_int32), ("row_kind", ctypes.c_int32)]

    def as_tuple(self):
        return (self.g, self.row_e, self.row_nt, self.col_e, self.col_w, self.row_kind)

    def __repr__(self):
        return (f"Plan2D(g={self.g}, row_e={self.row_e}, row_nt={self.row_nt}, col_e={self.col_e}, "
                f"col_w={self.col_w}, row_kind={self.row_kind})")


class Plan1D(ctypes.Structure):
    """qsg_plan1d: kind 0 resident (one CTA) / 1 four-step (n = n1 * n2), row length n1, tensor-copy columns."""
    _fields_ = [("kind", ctypes.c_int32), ("n1", ctypes.c_int32), ("tma", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]

    def as_tuple(self):
        return (self.kind, self.n1, self.tma)

    def __repr__(self):
        return f"Plan1D(kind={self.kind}, n1={self.n1}, tma={self.tma})"


class BornOpts(ctypes.Structure):
    """qsg_born_opts: the order / preconditional / preconditioner / slow options."""
    _fields_ = [("order", ctypes.c_int), ("preconditional", ctypes.c_int), ("preconditioner", ctypes.c_int),
                ("slow", ctypes.c_double)]


class QsgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{STATUS_NAMES.get(code, code)}] {msg}")
        self.code = code


_lib = None
_lock = threading.Lock()

_vp = ctypes.c_void_p
_d = ctypes.c_double
_dp = ctypes.POINTER(ctypes.c_double)
_u64 = ctypes.c_uint64
_i = ctypes.c_int
_sz = ctypes.c_size_t


def _declare(lib):
    lib.qsg_version.restype = ctypes.c_char_p
    lib.qsg_last_error.restype = ctypes.c_char_p
    lib.qsg_init.argtypes = [_i, _sz, ctypes.POINTER(_vp)]
    lib.qsg_ctx_destroy.argtypes = [_vp]
    lib.qsg_ctx_destroy.restype = None
    lib.qsg_ctx_stream.argtypes = [_vp]
    lib.qsg_ctx_stream.restype = _vp
    lib.qsg_ctx_bytes_in_use.argtypes = [_vp]
    lib.qsg_ctx_bytes_in_use.restype = _sz
    lib.qsg_create_1d.argtypes = [_vp, _u64, _d, _d, _d, _d, _d, _i, _i, _i, _dp, _dp, ctypes.POINTER(_vp)]
    lib.qsg_create_1d_spec.argtypes = [_vp, _u64, _d, _d, _d, _d, _d, _i, _i, _i, ctypes.POINTER(Spec),
                                       ctypes.POINTER(_vp)]
    lib.qsg_create_2d_spec.argtypes = [_vp, _u64, _u64, _d, _d, _d, _d, _d, _d, _i, _i, ctypes.POINTER(Spec),
                                       ctypes.POINTER(_vp)]
    lib.qsg_create_2d.argtypes = [_vp, _u64, _u64, _d, _d, _d, _d, _d, _d, _i, _i, _dp, _dp,
                                  ctypes.POINTER(_vp)]
    lib.qsg_create_3d.argtypes = [_vp, _u64, _u64, _u64, _d, _d, _d, _d, _d, _d, _d, _i, _i, _dp, _dp,
                                  ctypes.POINTER(_vp)]
    lib.qsg_step.argtypes = [_vp, _u64, _i]
    lib.qsg_sync.argtypes = [_vp]
    lib.qsg_norm2.argtypes = [_vp, _dp]
    lib.qsg_step_norm2.argtypes = [_vp, _dp]
    lib.qsg_step_norm2_post.argtypes = [_vp, ctypes.POINTER(_u64)]
    lib.qsg_step_norm2_get.argtypes = [_vp, _u64, _dp]
    lib.qsg_energies.argtypes = [_vp, _dp, _dp]
    lib.qsg_xavg.argtypes = [_vp, _d, _dp]
    lib.qsg_norm2_range.argtypes = [_vp, _d, _d, _d, _dp]
    lib.qsg_get_psi.argtypes = [_vp, _dp]
    lib.qsg_set_psi.argtypes = [_vp, _dp]
    lib.qsg_steps_taken.argtypes = [_vp, ctypes.POINTER(_u64)]
    lib.qsg_destroy.argtypes = [_vp]
    lib.qsg_destroy.restype = None
    lib.qsg_candidate_plans.argtypes = [_i, _u64, _u64, ctypes.POINTER(Plan2D), _i]
    lib.qsg_get_plan.argtypes = [_vp, ctypes.POINTER(Plan2D)]
    lib.qsg_set_plan.argtypes = [_vp, ctypes.POINTER(Plan2D)]
    lib.qsg_set_form.argtypes = [_vp, _i]
    lib.qsg_get_form.argtypes = [_vp, ctypes.POINTER(_i)]
    lib.qsg_check_wait_timeout.argtypes = [_vp]
    lib.qsg_autotune.argtypes = [_vp, _i, _i, ctypes.POINTER(Plan2D), _dp]
    lib.qsg_candidate_plans_1d.argtypes = [_i, _u64, _i, ctypes.POINTER(Plan1D), _i]
    lib.qsg_get_plan_1d.argtypes = [_vp, ctypes.POINTER(Plan1D)]
    lib.qsg_set_plan_1d.argtypes = [_vp, ctypes.POINTER(Plan1D)]
    lib.qsg_autotune_1d.argtypes = [_vp, _i, _i, ctypes.POINTER(Plan1D), _dp]
    lib.qsg_batch_autotune.argtypes = [_vp, _i, _dp]
    lib.qsg_batch_get_plan_1d.argtypes = [_vp, _u64, ctypes.POINTER(Plan1D)]
    lib.qsg_batch_set_plan_1d.argtypes = [_vp, _u64, ctypes.POINTER(Plan1D)]
    _pp = ctypes.POINTER(_dp)
    lib.qsg_batch_create_1d.argtypes = [_vp, _i, ctypes.POINTER(_u64), _dp, _dp, _dp, _d, _d, _i, _i, _pp, _pp,
                                        ctypes.POINTER(_vp)]
    lib.qsg_batch_step.argtypes = [_vp, _u64]
    lib.qsg_batch_sync.argtypes = [_vp]
    lib.qsg_batch_size.argtypes = [_vp, ctypes.POINTER(_i), ctypes.POINTER(_u64)]
    lib.qsg_batch_instance.argtypes = [_vp, _i, ctypes.POINTER(_vp)]
    lib.qsg_batch_destroy.argtypes = [_vp]
    lib.qsg_batch_destroy.restype = None
    lib.qsg_server_create.argtypes = [_i, _sz, _i, ctypes.POINTER(_vp)]
    lib.qsg_server_submit.argtypes = [_vp, ctypes.POINTER(Request), ctypes.POINTER(_u64)]
    lib.qsg_server_poll.argtypes = [_vp, _u64, ctypes.POINTER(_i)]
    lib.qsg_server_wait.argtypes = [_vp, _u64, _d, ctypes.POINTER(_i)]
    lib.qsg_server_take.argtypes = [_vp, _u64, _dp, _dp]
    lib.qsg_server_stats.argtypes = [_vp, ctypes.POINTER(ServerInfo)]
    lib.qsg_server_request_info.argtypes = [_vp, _u64, ctypes.POINTER(RequestInfo)]
    _cp = ctypes.c_char_p
    lib.qsg_create_1d_expr.argtypes = [_vp, _u64, _d, _d, _d, _d, _d, _d, _i, _i, _i, _cp, _cp, _i,
                                       ctypes.POINTER(_vp)]
    lib.qsg_create_2d_expr.argtypes = [_vp, _u64, _u64, _d, _d, _d, _d, _d, _d, _d, _d, _i, _i, _cp, _cp, _i,
                                       ctypes.POINTER(_vp)]
    lib.qsg_expr_eval.argtypes = [_cp, _i, ctypes.POINTER(_cp), _dp, _dp]
    lib.qsg_server_destroy.argtypes = [_vp]
    lib.qsg_server_destroy.restype = None
    lib.qsg_profile_enable.argtypes = [_vp, _i]
    lib.qsg_profile_read.argtypes = [_vp, _i, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(_u64), _dp]
    lib.qsg_norm2_noalloc.argtypes = [_vp, _u64, _i, _d, _vp, _dp]
    lib.qsg_born_default_opts.argtypes = [ctypes.POINTER(BornOpts)]
    lib.qsg_born_default_opts.restype = None
    lib.qsg_born_create_1d.argtypes = [_vp, _u64, _d, _d, _dp, _d, _d, _d, _d, _d, ctypes.POINTER(BornOpts), _i,
                                       ctypes.POINTER(_vp)]
    lib.qsg_born_create_2d.argtypes = [_vp, _i, _i, _d, _d, _d, _d, _dp, _d, _d, _d, _d, _d, _d,
                                       ctypes.POINTER(BornOpts), _i, ctypes.POINTER(_vp)]
    lib.qsg_born_compute.argtypes = [_vp]
    lib.qsg_born_get.argtypes = [_vp, _i, _dp]
    lib.qsg_born_rt.argtypes = [_vp, _dp, _dp]
    lib.qsg_born_delta_norm.argtypes = [_vp, _dp]
    lib.qsg_born_epsilon.argtypes = [_vp, _dp]
    lib.qsg_born_xsection.argtypes = [_vp, _i, _dp, _dp]
    lib.qsg_born_total_xsection.argtypes = [_vp, _i, _dp]
    lib.qsg_born_destroy.argtypes = [_vp]
    lib.qsg_born_destroy.restype = None


def load(path: str = LIB_PATH):
    """Load libqsg.so (once).  Raises QsgError if it is not there."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(path):
                raise QsgError(QSG_ERR_STATE, f"{path} not built: run `python -m qusim_gb300.build`")
            lib = ctypes.CDLL(path)
            _declare(lib)
            _lib = lib
        return _lib


def check(rc: int):
    if rc != QSG_OK:
        raise QsgError(rc, load().qsg_last_error().decode())
    return rc
