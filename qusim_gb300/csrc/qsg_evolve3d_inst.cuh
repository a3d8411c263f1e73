// qsg_evolve3d_inst.cuh -- launchers of the 3D passes, instantiated per
// precision by qsg_evolve3d_f32.cu / qsg_evolve3d_f64.cu.
#pragma once
#include "qsg_dispatch.cuh"
#include "qsg_evolve3d.cuh"

namespace qsg {

constexpr int e3(int prec) { return prec == 1 ? 16 : 8; }
// z lines: B per CTA, B * L / E = 256 threads
constexpr int b3(int prec, int l) { return (prec == 1 ? 4096 : 2048) / l > 1 ? (prec == 1 ? 4096 : 2048) / l : 1; }
// strided lines: W adjacent ones per CTA, W * L / E <= 512 threads, W <= 16
constexpr int w3(int prec, int l) { return (prec == 1 ? 8192 : 4096) / l > 16 ? 16 : (prec == 1 ? 8192 : 4096) / l; }

template <class T, int L>
static cudaError_t run3_row(size_t lines, const Pass3Args &a, cudaStream_t st)
{
    constexpr int P = sizeof(T) == 4 ? 1 : 0, E = e3(P), B = b3(P, L);
    constexpr int PADS = P ? 4 : 3;
    const size_t smem = sizeof(cplx_t<T>) * B * padded<L, PADS>(L);
    auto k = k3_row<T, L, E, B>;
    cudaError_t e = prepare_smem(k, smem);
    if (e != cudaSuccess) return e;
    k<<<(unsigned)(lines / B), B * (L / E), smem, st>>>(a);
    return cudaGetLastError();
}

template <class T, int L>
static cudaError_t run3_col(int inner, int outer, const Pass3Args &a, cudaStream_t st)
{
    constexpr int P = sizeof(T) == 4 ? 1 : 0, E = e3(P), W = w3(P, L);
    const size_t smem = sizeof(cplx_t<T>) * col_tile_elems(sizeof(cplx_t<T>), L, W, E);
    auto k = k3_col<T, L, E, W>;
    cudaError_t e = prepare_smem(k, smem);
    if (e != cudaSuccess) return e;
    k<<<dim3(inner / W, outer), W * (L / E), smem, st>>>(a);
    return cudaGetLastError();
}

#define QSG_3D_SIZES(X) X(16) X(32) X(64) X(128) X(256) X(512) X(1024)

template <class T> cudaError_t launch3_row(int l, size_t lines, const Pass3Args &a, cudaStream_t st)
{
#define X(N) case N: return run3_row<T, N>(lines, a, st);
    switch (l) { QSG_3D_SIZES(X) default: break; }
#undef X
    return cudaErrorNotSupported;
}

template <class T> cudaError_t launch3_col(int l, int inner, int outer, const Pass3Args &a, cudaStream_t st)
{
#define X(N) case N: return run3_col<T, N>(inner, outer, a, st);
    switch (l) { QSG_3D_SIZES(X) default: break; }
#undef X
    return cudaErrorNotSupported;
}

#define QSG_3D_INSTANTIATE(T)                                                                   \
    template cudaError_t launch3_row<T>(int, size_t, const Pass3Args &, cudaStream_t);         \
    template cudaError_t launch3_col<T>(int, int, int, const Pass3Args &, cudaStream_t);

}  // namespace qsg
