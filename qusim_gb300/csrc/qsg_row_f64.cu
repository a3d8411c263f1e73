// 2D row passes (double): instantiations + launcher.
#include "qsg_dispatch.cuh"

namespace qsg {

template <int NY, int G, bool IS, bool OS>
static cudaError_t run_row_f64(const Geom2D &g, const RowPassArgs &a, cudaStream_t st)
{
    constexpr int E = 8;
    constexpr int B = row_b_for(NY, E, G);
    constexpr int RS = row_rs_for(NY, E, G);
    auto k = k_row_pass<double, NY, E, G, B, RS, IS, OS>;
    cudaError_t e = prepare_smem(k, g.row_smem);
    if (e != cudaSuccess) return e;
    k<<<g.row_blocks, g.row_threads, g.row_smem, st>>>(a);
    return cudaGetLastError();
}

template <int NY, int G>
static cudaError_t row_modes_f64(const Geom2D &g, bool is, bool os, const RowPassArgs &a, cudaStream_t st)
{
    if (!is && os) return run_row_f64<NY, G, false, true>(g, a, st);
    if (is && os) return run_row_f64<NY, G, true, true>(g, a, st);
    if (is && !os) return run_row_f64<NY, G, true, false>(g, a, st);
    return run_row_f64<NY, G, false, false>(g, a, st);
}

cudaError_t launch_row_pass_f64(const Geom2D &g, bool is, bool os, const RowPassArgs &a, cudaStream_t st)
{
#define X(NY) \
    case NY: \
        if (g.g == 1) return row_modes_f64<NY, 1>(g, is, os, a, st); \
        if (g.g == 2) return row_modes_f64<NY, 2>(g, is, os, a, st); \
        break;
    switch (g.ny) { X(128) X(256) X(512) X(1024) X(2048) X(4096) default: break; }
#undef X
    return cudaErrorNotSupported;
}

}  // namespace qsg
