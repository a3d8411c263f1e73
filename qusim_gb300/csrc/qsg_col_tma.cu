// Momentum-form column pass fed by tensor copies: instantiations, launcher and
// the tensor maps of the two buffers it reads.
#include <algorithm>
#include "qsg_col_tma.cuh"
#include <atomic>
#include "qsg_dispatch.cuh"

namespace qsg {

bool col_tma_supported(int m, int e, int w) { return e == 32 && ((m == 1024 && w == 8) || (m == 512 && w == 16)); }

template <int M, int E, int W, bool PL>
static cudaError_t run_col_tma(const ColPassArgs &a, const CUtensorMap *mw, const CUtensorMap *mp, cudaStream_t st)
{
    auto k = k_col_pass_tma<M, E, W, PL>;
    const size_t smem = col_tma_smem(M, W, E) + 128;
    // the attribute belongs to the device's context: set once per device
    static std::atomic<uint64_t> ready{0};
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = dev < 64 ? 1ull << dev : 0;
    if (!bit || !(ready.load() & bit)) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        ready.fetch_or(bit);
    }
    // persistent: one CTA per SM (the staging buffers take most of its shared memory)
    const int grid = std::min(a.tiles, sm_count());
    k<<<grid, W * (M / E), smem, st>>>(a, *mw, *mp);
    return cudaGetLastError();
}

cudaError_t launch_col_pass_tma(const Geom2D &g, const ColPassArgs &a, const void *maps, cudaStream_t st)
{
    const CUtensorMap *m = static_cast<const CUtensorMap *>(maps);
    if (g.m == 1024 && g.col_e == 32 && g.col_w == 8)
        return a.plain ? run_col_tma<1024, 32, 8, true>(a, m, m + 1, st) : run_col_tma<1024, 32, 8, false>(a, m, m + 1, st);
    if (g.m == 512 && g.col_e == 32 && g.col_w == 16)
        return a.plain ? run_col_tma<512, 32, 16, true>(a, m, m + 1, st) : run_col_tma<512, 32, 16, false>(a, m, m + 1, st);
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

bool encode_2d_map(void *base, uint64_t inner, uint64_t outer, uint32_t box_inner, uint32_t box_outer, void *out)
{
    EncodeTiled fn = encode_fn();
    if (!fn || !base || (reinterpret_cast<uintptr_t>(base) & 15) || (inner * 8) % 16 || (box_inner * 8) % 16 ||
        box_inner == 0 || box_inner > 256 || box_outer == 0 || box_outer > 256 || outer < box_outer ||
        inner % box_inner || outer % box_outer)
        return false;
    const cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
    const cuuint64_t strides[1] = {(cuuint64_t)inner * 8};
    const cuuint32_t box[2] = {box_inner, box_outer};
    const cuuint32_t estr[2] = {1, 1};
    return fn(static_cast<CUtensorMap *>(out), CU_TENSOR_MAP_DATA_TYPE_INT64, 2, base, dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool encode_col_tma_maps(void *work, void *psi, int nx, int ny, int w, void *out)
{
    CUtensorMap *m = static_cast<CUtensorMap *>(out);
    return encode_2d_map(work, (uint64_t)ny, (uint64_t)nx, (uint32_t)w, 256, m) &&
           encode_2d_map(psi, (uint64_t)ny, (uint64_t)nx, (uint32_t)w, 256, m + 1);
}

}  // namespace qsg
