// 2D column passes (float): instantiations + launcher.
#include "qsg_dispatch.cuh"

namespace qsg {

template <class T, int M, int E, int W, bool PL>
static cudaError_t run_col_f32(const Geom2D &g, const ColPassArgs &a, cudaStream_t st)
{
    auto k = k_col_pass<T, M, E, W, PL>;
    cudaError_t e = prepare_smem(k, g.col_smem);
    if (e != cudaSuccess) return e;
    k<<<(unsigned)a.tiles, W * (M / E), g.col_smem, st>>>(a);  // one tile per CTA
    return cudaGetLastError();
}

template <bool PL> cudaError_t launch_col_pass_f32_t(const Geom2D &g, const ColPassArgs &a, cudaStream_t st)
{
#define C(T, M, E, W) \
    if (g.m == M && g.col_e == E && g.col_w == W) return run_col_f32<T, M, E, W, PL>(g, a, st);
    QSG_COL_VARIANTS_F32(C)
#undef C
    return cudaErrorNotSupported;
}

// this unit instantiates the hi + lo twiddle variants, qsg_colpass_f32_plain.cu
// (which includes it) the plain ones
#ifndef QSG_PLAIN_UNIT
template cudaError_t launch_col_pass_f32_t<false>(const Geom2D &, const ColPassArgs &, cudaStream_t);
#else
template cudaError_t launch_col_pass_f32_t<true>(const Geom2D &, const ColPassArgs &, cudaStream_t);
#endif

}  // namespace qsg
