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


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_noalloc_at_the_limit_then_a_ragged_length(lib, precision):
    """A call at the maximum size (2^26 sites: every block of the fixed array in
    use), then one whose length is not a multiple of a block's 16,384 sites, so
    the last block is partial and fewer partial sums are read than the first
    call wrote.  Each is compared with a float64 sum of the same buffer."""
    torch = pytest.importorskip("torch")
    dt = torch.float32 if precision == "mixed" else torch.float64
    gen = torch.Generator(device="cuda").manual_seed(5)
    n_max = 1 << 26
    big = torch.rand(2 * n_max, dtype=dt, device="cuda", generator=gen) - 0.5
    want = float((big.double() ** 2).sum())
    got = norm2_noalloc(lib, torch, big, n_max, precision, 0.25)
    assert abs(got - 0.25 * want) <= 1e-12 * 0.25 * want, (got, want)
    n_rag = 16384 * 5 + 37
    rag = big[: 2 * n_rag] * 3.0
    torch.cuda.synchronize()
    want = float((rag.double() ** 2).sum())
    got = norm2_noalloc(lib, torch, rag, n_rag, precision, 1.0)
    assert abs(got - want) <= 1e-12 * want, (got, want)
    del big, rag


def test_noalloc_refuses_a_stream_being_captured(lib):
    """The call waits for its result on the host, so a stream under graph
    capture is refused (QSG_ERR_STATE) before anything is queued on it."""
    from qusim_gb300 import _lib
    torch = pytest.importorskip("torch")
    t = torch.ones(2 * 4096, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    out = ctypes.c_double(-1.0)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s, capture_error_mode="relaxed"):
            rc = lib.qsg_norm2_noalloc(ctypes.c_void_p(t.data_ptr()), 4096, _lib.QSG_FP64, 1.0,
                                       ctypes.c_void_p(s.cuda_stream), ctypes.byref(out))
            t.mul_(1.0)  # something for the graph to hold
    assert rc == _lib.QSG_ERR_STATE and b"captured" in lib.qsg_last_error()
    assert out.value == -1.0
    # outside the capture the same call works: 4096 sites of 1 + 1i, dv = 2
    rc = lib.qsg_norm2_noalloc(ctypes.c_void_p(t.data_ptr()), 4096, _lib.QSG_FP64, 2.0, None, ctypes.byref(out))
    assert rc == 0 and out.value == 2.0 * 4096 * 2.0
