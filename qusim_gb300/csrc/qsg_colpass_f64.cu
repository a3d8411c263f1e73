// 2D column passes (double): instantiations + launcher.
#include "qsg_dispatch.cuh"

namespace qsg {

template <class T, int M, int E, int W>
static cudaError_t run_col_f64(const Geom2D &g, const ColPassArgs &a, cudaStream_t st)
{
    auto k = k_col_pass<T, M, E, W>;
    cudaError_t e = prepare_smem(k, g.col_smem);
    if (e != cudaSuccess) return e;
    k<<<(unsigned)a.tiles, W * (M / E), g.col_smem, st>>>(a);  // one tile per CTA
    return cudaGetLastError();
}

cudaError_t launch_col_pass_f64(const Geom2D &g, const ColPassArgs &a, cudaStream_t st)
{
#define C(T, M, E, W) \
    if (g.m == M && g.col_e == E && g.col_w == W) return run_col_f64<T, M, E, W>(g, a, st);
    QSG_COL_VARIANTS_F64(C)
#undef C
    return cudaErrorNotSupported;
}

}  // namespace qsg
