"""qsg_norm2_noalloc: Norm2 of a caller-owned device buffer with no device allocation.

Callers whose GPU memory is reserved up front by another runtime's pool, or
whose real-time loop may not call cudaMalloc / cudaFree (those calls can stall
the whole device), hold the wavefunction themselves and cannot let the library
allocate its reduction scratch.  This entry point keeps that scratch in a fixed
array inside libqsg.so.  Here a torch tensor plays the caller's buffer, and each
result is checked against qsg_norm2 on an engine instance in the same state.

The file name makes pytest collect it last, so a run that stops at the first
failure has already run every other test.  It also passes alone in a fresh
process: the first call on the device does the array's one-time set-up.
"""
import ctypes

import numpy as np
import pytest

from tests.workloads import gauss_packet_1d, gauss_packet_2d, gaussian_bumps_2d

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the complex128 parity bar of the GPU tests


@pytest.fixture(scope="module")
def lib():
    import qusim_gb300 as q
    return q.load()


def caller_buffer(torch, psi, precision):
    """psi as a device tensor owned by the caller (complex64 for the mixed form)."""
    a = np.ascontiguousarray(psi, dtype=np.complex64 if precision == "mixed" else np.complex128)
    t = torch.from_numpy(a.view(np.float32 if precision == "mixed" else np.float64)).to("cuda")
    torch.cuda.synchronize()
    return t


def norm2_noalloc(lib, torch, t, n, precision, dv):
    from qusim_gb300 import _lib
    out = ctypes.c_double(-1.0)
    prec = _lib.QSG_MIXED if precision == "mixed" else _lib.QSG_FP64
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.qsg_norm2_noalloc(ctypes.c_void_p(t.data_ptr()), n, prec, dv, ctypes.c_void_p(stream),
                               ctypes.byref(out))
    assert rc == 0, lib.qsg_last_error().decode()
    return out.value


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_noalloc_norm2_matches_qsg_norm2_on_two_calls(lib, precision):
    """Two calls in a row, the second on a smaller state than the first, so a
    stale partial sum or counter left by the first call would show."""
    torch = pytest.importorskip("torch")
    import qusim_gb300 as q
    ctx = q.Context(0)
    psi2, dx, dy = gauss_packet_2d(1024, 1024, -100, 100, -100, 100, 1.5, 0.0, -40.0, 0.0, 8.0)
    V2 = gaussian_bumps_2d(1024, 1024, -100, 100, -100, 100, seed=3)
    big = q.Instance.create_2d(ctx, psi2 * 1.7, V2, dx, dy, 0.01, order=4, precision=precision)
    big.step(3)
    psi1, V1, dx1 = gauss_packet_1d(65536, -3000.0, 3000.0, 1.5, -500.0, 300.0, barrier=0.7)
    small = q.Instance.create_1d(ctx, psi1 * 0.6, V1, dx1, 0.01, order=2, precision=precision)
    small.step(5)

    for inst, dv in ((big, dx * dy), (small, dx1)):
        want = inst.norm2()
        psi = inst.get_psi()
        t = caller_buffer(torch, psi, precision)
        got = norm2_noalloc(lib, torch, t, psi.size, precision, dv)
        assert abs(got - want) <= TOL * abs(want), (got, want)
    big.close()
    small.close()
    ctx.close()


def test_noalloc_rejects_bad_arguments(lib):
    """Sizes beyond the fixed array and buffers that are not device memory are
    refused on the host, before any launch."""
    from qusim_gb300 import _lib
    torch = pytest.importorskip("torch")
    out = ctypes.c_double()
    t = torch.zeros(64, dtype=torch.float64, device="cuda")
    rc = lib.qsg_norm2_noalloc(ctypes.c_void_p(t.data_ptr()), (1 << 26) + 1, _lib.QSG_FP64, 1.0, None,
                               ctypes.byref(out))
    assert rc == 1 and b"exceeds" in lib.qsg_last_error()
    host = np.zeros(64, np.complex128)
    rc = lib.qsg_norm2_noalloc(ctypes.c_void_p(host.ctypes.data), 64, _lib.QSG_FP64, 1.0, None,
                               ctypes.byref(out))
    assert rc == 1 and b"not device memory" in lib.qsg_last_error()
    rc = lib.qsg_norm2_noalloc(ctypes.c_void_p(t.data_ptr()), 16, 7, 1.0, None, ctypes.byref(out))
    assert rc == 1
