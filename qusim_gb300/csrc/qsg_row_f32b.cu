// 2D row passes (float, radix 8): instantiations + launcher.
// Packed f32x2 arithmetic in the transforms (qsg_fft.cuh).  Measured on the 4096^2
// momentum-form step: this row pass 134.3 -> 128.8 us per launch.  Its plain 45-degree
// rotations are no longer fused by the compiler into the next butterfly add, so the
// rounding differs from the scalar build (not the accuracy: 3.8e-9 after 6 steps).
#define QSG_PACKED_F32 1
#include "qsg_dispatch.cuh"

namespace qsg {

template <int NY, int E, int G, int NT, bool PL>
static cudaError_t run_row_f32b(const Geom2D &g, const RowPassArgs &a, cudaStream_t st)
{
    constexpr int B = row_b_for(NY, E, G);
    constexpr int RS = row_work_for(NY, E, G) / NT;
    static_assert(RS * NT == row_work_for(NY, E, G), "NT must divide the CTA's line work");
    auto k = k_row_pass<float, NY, E, G, B, RS, PL>;
    cudaError_t e = prepare_smem(k, g.row_smem);
    if (e != cudaSuccess) return e;
    static int occ = 0;
    k<<<persistent_grid(k, NT, g.row_smem, a.units, occ), NT, g.row_smem, st>>>(a);
    return cudaGetLastError();
}

template <bool PL> cudaError_t launch_row_pass_f32b_t(const Geom2D &g, const RowPassArgs &a, cudaStream_t st)
{
#define X(T, NY, E, G, NT) \
    if (g.ny == NY && g.row_e == E && g.g == G && g.row_threads == NT) return run_row_f32b<NY, E, G, NT, PL>(g, a, st);
    QSG_ROW_VARIANTS_F32B(X)
#undef X
    return cudaErrorNotSupported;
}

// this unit instantiates the hi + lo twiddle variants; qsg_row_f32b_plain.cu
// (which includes it) the plain ones, in parallel
#ifndef QSG_PLAIN_UNIT
template cudaError_t launch_row_pass_f32b_t<false>(const Geom2D &, const RowPassArgs &, cudaStream_t);

bool row_variant_exists_f32b(int ny, int e, int g, int nt)
{
#define X(T, NY, E, G, NT) \
    if (ny == NY && e == E && g == G && nt == NT) return true;
    QSG_ROW_VARIANTS_F32B(X)
#undef X
    return false;
}

#else
template cudaError_t launch_row_pass_f32b_t<true>(const Geom2D &, const RowPassArgs &, cudaStream_t);
#endif

}  // namespace qsg
