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

// one instance's n2 x n1 complex64 buffer (row-major) as a 2D tensor of
// 8-byte elements, boxes of W = 4096 / n2 columns x min(n2, 256) rows
bool encode_fs_map(void *base, int n1, int n2, void *out)
{
    return encode_2d_map(base, (uint64_t)n1, (uint64_t)n2, (uint32_t)(4096 / n2), (uint32_t)(n2 < 256 ? n2 : 256), out);
}

}  // namespace qsg
