// qsg_noalloc.cu -- qsg_norm2_noalloc: Norm2 of a caller-owned device buffer
// without allocating device memory.
//
// Some callers cannot allocate device memory at all: applications whose GPU
// memory is reserved up front and handed out by another runtime's pool (where
// a cudaMalloc from a library fails or is forbidden), and real-time loops that
// may not call cudaMalloc / cudaFree because those calls can synchronise the
// whole device.  They already own the wavefunction buffer; this entry point
// sums |psi|^2 over it with its scratch (the per-block partial sums, a
// completion counter and the result) in one fixed array compiled into this
// file, instead of the context's allocated partials buffer that qsg_norm2 uses.
//
// The array costs every device that loads the library its 33,024 bytes until
// the process exits, and bounds the input at QSG_NORM2_NOALLOC_MAX_SITES.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/qsg.h"
#include "qsg_launch.h"

namespace {

constexpr int kThreads = 256;
constexpr uint64_t kSitesPerBlock = 16384;  // 64 sites per thread
constexpr int kMaxBlocks = 4096;            // one partial sum per block
static_assert(kSitesPerBlock * kMaxBlocks == QSG_NORM2_NOALLOC_MAX_SITES, "limit and scratch disagree");
// [0, kMaxBlocks): partial sums; [kMaxBlocks]: completion counter (as an
// unsigned int); [kMaxBlocks + 1]: the result; the rest pads to 256 bytes
constexpr int kCounterSlot = kMaxBlocks;
constexpr int kResultSlot = kMaxBlocks + 1;
constexpr int kScratchDoubles = kMaxBlocks + 32;
constexpr int kMaxDevices = 64;

}  // namespace

// The scratch.  In host code this name is only a stand-in for the symbol, not
// a device address: kernels get the address that cudaGetSymbolAddress returns.
static __device__ __align__(256) double g_norm2_scratch[kScratchDoubles];

namespace {

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// every thread returns the sum over the block (fixed order)
__device__ __forceinline__ double cta_sum(double v, double *red)
{
    v = warp_sum(v);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = threadIdx.x < kThreads / 32 ? red[threadIdx.x] : 0.0;
    if (threadIdx.x < 32) s = warp_sum(s);
    if (threadIdx.x == 0) red[0] = s;
    __syncthreads();
    return red[0];
}

template <class C> __device__ __forceinline__ double abs2_wide(C a)
{
    return double(a.x) * double(a.x) + double(a.y) * double(a.y);
}

// Block b sums sites [b*kSitesPerBlock, (b+1)*kSitesPerBlock) into
// scratch[b]; the last block to finish adds the partials in block order, so
// the result does not depend on which block finishes last.
template <class C>
__global__ void __launch_bounds__(kThreads) k_norm2_noalloc(const C *__restrict__ psi, uint64_t n, double *scratch)
{
    __shared__ double red[32];
    __shared__ bool is_last;
    const uint64_t lo = (uint64_t)blockIdx.x * kSitesPerBlock;
    const uint64_t hi = lo + kSitesPerBlock < n ? lo + kSitesPerBlock : n;
    double s = 0;
    for (uint64_t i = lo + threadIdx.x; i < hi; i += kThreads) s += abs2_wide(psi[i]);
    s = cta_sum(s, red);
    unsigned int *counter = reinterpret_cast<unsigned int *>(scratch + kCounterSlot);
    if (threadIdx.x == 0) {
        scratch[blockIdx.x] = s;
        __threadfence();  // the partial is visible device-wide before the count
        is_last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double t = 0;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += kThreads) t += __ldcg(scratch + b);
    t = cta_sum(t, red);
    if (threadIdx.x == 0) {
        scratch[kResultSlot] = t;
        *counter = 0u;
    }
}

std::mutex g_addr_mu;
double *g_addr[kMaxDevices] = {};

// Device address of g_norm2_scratch on `dev` (the current device), looked up
// once per device on its first call.
int scratch_address(int dev, double **out)
{
    std::lock_guard<std::mutex> lk(g_addr_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_norm2_scratch);
        if (e != cudaSuccess)
            return qsg::set_last_error(QSG_ERR_CUDA, std::string("qsg_norm2_noalloc: cudaGetSymbolAddress: ") +
                                                         cudaGetErrorString(e));
        g_addr[dev] = static_cast<double *>(p);
    }
    *out = g_addr[dev];
    return QSG_OK;
}

#define NA_CUDA(call)                                                                                   \
    do {                                                                                                \
        const cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) {                                                                        \
            rc = qsg::set_last_error(QSG_ERR_CUDA, std::string("qsg_norm2_noalloc: ") + #call + ": " + \
                                                       cudaGetErrorString(e_));                         \
            goto done;                                                                                  \
        }                                                                                               \
    } while (0)

}  // namespace

extern "C" int qsg_norm2_noalloc(const void *psi, uint64_t n, int precision, double dv, void *stream, double *out)
{
    if (!out || (!psi && n)) return qsg::set_last_error(QSG_ERR_ARG, "qsg_norm2_noalloc: null argument");
    if (precision != QSG_FP64 && precision != QSG_MIXED)
        return qsg::set_last_error(QSG_ERR_ARG, "qsg_norm2_noalloc: precision must be QSG_FP64 or QSG_MIXED");
    if (n > QSG_NORM2_NOALLOC_MAX_SITES)
        return qsg::set_last_error(QSG_ERR_ARG, "qsg_norm2_noalloc: n = " + std::to_string(n) +
                                                    " exceeds the limit of its fixed scratch array (" +
                                                    std::to_string(QSG_NORM2_NOALLOC_MAX_SITES) + " sites)");
    if (n == 0) {
        *out = 0;
        return QSG_OK;
    }
    const size_t esize = precision == QSG_MIXED ? 8 : 16;
    if (reinterpret_cast<uintptr_t>(psi) % esize)
        return qsg::set_last_error(QSG_ERR_ARG, "qsg_norm2_noalloc: psi is not aligned to its element size");
    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    {
        // The call waits for its result on the host, which a stream being
        // captured cannot do.  Checked first: any other query of a capturing
        // stream would end the caller's capture with an error.
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
            cudaGetLastError();
            return qsg::set_last_error(QSG_ERR_STATE, "qsg_norm2_noalloc: the stream is being captured; this call "
                                                      "is synchronous and cannot be part of a graph");
        }
    }
    cudaPointerAttributes attr{};
    if (cudaPointerGetAttributes(&attr, psi) != cudaSuccess || attr.device < 0 || attr.device >= kMaxDevices ||
        (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged)) {
        cudaGetLastError();
        return qsg::set_last_error(QSG_ERR_ARG, "qsg_norm2_noalloc: psi is not device memory");
    }

    if (st) {
        // the launch goes to the caller's stream: it must belong to psi's device
        int sdev = -1;
        if (cudaStreamGetDevice(st, &sdev) != cudaSuccess) {
            cudaGetLastError();
            return qsg::set_last_error(QSG_ERR_ARG, "qsg_norm2_noalloc: stream is not a valid CUDA stream");
        }
        if (sdev != attr.device)
            return qsg::set_last_error(QSG_ERR_ARG, "qsg_norm2_noalloc: stream belongs to device " +
                                                        std::to_string(sdev) + ", psi to device " +
                                                        std::to_string(attr.device));
    }

    int prev = -1, rc = QSG_OK;
    double *scratch = nullptr, sum = 0;
    const unsigned blocks = (unsigned)((n + kSitesPerBlock - 1) / kSitesPerBlock);
    NA_CUDA(cudaGetDevice(&prev));
    if (prev != attr.device) NA_CUDA(cudaSetDevice(attr.device));
    if ((rc = scratch_address(attr.device, &scratch))) goto done;
    // the completion counter must start at zero; partials and result are overwritten
    NA_CUDA(cudaMemsetAsync(scratch + kCounterSlot, 0, sizeof(double), st));
    if (precision == QSG_MIXED)
        k_norm2_noalloc<float2><<<blocks, kThreads, 0, st>>>(static_cast<const float2 *>(psi), n, scratch);
    else
        k_norm2_noalloc<double2><<<blocks, kThreads, 0, st>>>(static_cast<const double2 *>(psi), n, scratch);
    NA_CUDA(cudaGetLastError());
    NA_CUDA(cudaMemcpyAsync(&sum, scratch + kResultSlot, sizeof(double), cudaMemcpyDeviceToHost, st));
    NA_CUDA(cudaStreamSynchronize(st));
    *out = sum * dv;
done:
    if (prev >= 0 && prev != attr.device) cudaSetDevice(prev);
    return rc;
}
