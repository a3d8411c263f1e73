// 1D four-step column pass fed by tensor copies: instantiations, launcher and
// the per-instance tensor maps.
#include <algorithm>
#include <atomic>
#include "qsg_fs_tma.cuh"
#include "qsg_dispatch.cuh"

namespace qsg {

bool fs_tma_supported(int prec, int n2) { return prec == 1 && (n2 == 128 || n2 == 256 || n2 == 512); }

template <int N2>
static cudaError_t run_fs_tma(const FsColArgs &a, cudaStream_t st)
{
    constexpr int W = 4096 / N2;  // 256 threads: W * N2 / 16
    auto k = k_fs_col_tma<N2, W>;
    const size_t smem = fs_tma_smem(N2, W) + 128;
    static std::atomic<uint64_t> ready{0};
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = dev < 64 ? 1ull << dev : 0;
    if (!bit || !(ready.load() & bit)) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        ready.fetch_or(bit);
    }
    static int occ = 0;
    const unsigned grid = persistent_grid(k, W * (N2 / 16), smem, a.tiles, occ);
    k<<<grid, W * (N2 / 16), smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_fs_col_tma(const FsGeom &g, const FsColArgs &a, cudaStream_t st)
{
    if (g.n2 == 128) return run_fs_tma<128>(a, st);
    if (g.n2 == 256) return run_fs_tma<256>(a, st);
    if (g.n2 == 512) return run_fs_tma<512>(a, st);
    return cudaErrorNotSupported;
}

namespace {
using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiled encode_fn()
{
    static EncodeTiled fn = nullptr;
    static std::atomic<bool> tried{false};
    if (!tried.load()) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
        cudaGetLastError();
        tried.store(true);
    }
    return fn;
}
}  // namespace

// one instance's n2 x n1 complex64 buffer (row-major) as a 2D tensor of
// 8-byte elements, boxes of W = 4096 / n2 columns x min(n2, 256) rows
bool encode_fs_map(void *base, int n1, int n2, void *out)
{
    EncodeTiled fn = encode_fn();
    if (!fn || !base || (reinterpret_cast<uintptr_t>(base) & 15) || ((size_t)n1 * 8) % 16) return false;
    const int w = 4096 / n2;
    if (n1 % w) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)n1, (cuuint64_t)n2};
    const cuuint64_t strides[1] = {(cuuint64_t)n1 * 8};
    const cuuint32_t box[2] = {(cuuint32_t)w, (cuuint32_t)(n2 < 256 ? n2 : 256)};
    const cuuint32_t estr[2] = {1, 1};
    return fn(static_cast<CUtensorMap *>(out), CU_TENSOR_MAP_DATA_TYPE_INT64, 2, base, dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace qsg
