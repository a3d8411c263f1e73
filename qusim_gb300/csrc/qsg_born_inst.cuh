// qsg_born_inst.cuh -- launchers of the Born-series kernels, instantiated per
// precision by qsg_born_f32.cu / qsg_born_f64.cu.
#pragma once
#include "qsg_born.cuh"
#include "qsg_born_launch.h"
#include "qsg_dispatch.cuh"

namespace qsg {

template <class T> constexpr int born_prec() { return sizeof(T) == 4 ? 1 : 0; }

// 2D row pass: B groups of G rows per CTA, B * G * NY / E >= 256 threads where
// the rows are short (one group of G rows otherwise)
constexpr int born_row_b(int prec, int ny, int g)
{
    return (prec == 1 ? 4096 : 2048) / (ny * g) > 1 ? (prec == 1 ? 4096 : 2048) / (ny * g) : 1;
}
// G = nx / (1024 complex64, 512 complex128 rows), at most 4, and at most
// 512 / (ny / E) so that one group of G rows fits a CTA of 512 threads
constexpr int born_split_g0(int prec, int nx)
{
    return (prec == 1 ? (nx > 1024 ? nx / 1024 : 1) : (nx > 512 ? nx / 512 : 1)) > 4
               ? 4
               : (prec == 1 ? (nx > 1024 ? nx / 1024 : 1) : (nx > 512 ? nx / 512 : 1));
}
constexpr int born_split_c(int prec, int nx, int ny)
{
    return born_split_g0(prec, nx) * (ny / born_e(prec)) <= 512 ? born_split_g0(prec, nx) : 512 / (ny / born_e(prec));
}
// 2D column pass: W adjacent columns of M rows, W * M / E <= 512 threads
constexpr int born_col_w(int prec, int m)
{
    return prec == 1 ? (m <= 512 ? 16 : (m <= 1024 ? 8 : 4))
                     : (m <= 256 ? 16 : (m == 512 ? 8 : (m <= 2048 ? 4 : 2)));
}
// four-step column pass: W * N2 / E = 512 threads
constexpr int born_fs_w(int prec, int n2) { return (prec == 1 ? 8192 : 4096) / n2; }
// four-step row pass: B * N1 / E = 256 threads
constexpr int born_fs_b(int prec, int n1)
{
    return (prec == 1 ? 4096 : 2048) / n1 > 1 ? (prec == 1 ? 4096 : 2048) / n1 : 1;
}

template <class T, int NY, int G>
static cudaError_t run_born_row(int nx, const BornRowArgs &a, cudaStream_t st)
{
    constexpr int P = born_prec<T>(), E = born_e(P), B = born_row_b(P, NY, G);
    constexpr int PADS = P ? 4 : 3;
    const size_t smem = sizeof(cplx_t<T>) * B * G * padded<NY, PADS>(NY);
    auto k = k_born_row<T, NY, E, G, B>;
    cudaError_t e = prepare_smem(k, smem);
    if (e != cudaSuccess) return e;
    k<<<nx / (G * B), B * G * (NY / E), smem, st>>>(a);
    return cudaGetLastError();
}

template <class T, int M>
static cudaError_t run_born_col(int ny, int g, const BornColArgs &a, cudaStream_t st)
{
    constexpr int P = born_prec<T>(), E = born_col_e(P, M), W = born_col_w(P, M);
    const size_t smem = sizeof(cplx_t<T>) * col_tile_elems(sizeof(cplx_t<T>), M, W, E);
    auto k = k_born_col<T, M, E, W>;
    cudaError_t e = prepare_smem(k, smem);
    if (e != cudaSuccess) return e;
    k<<<g * (ny / W), W * (M / E), smem, st>>>(a);
    return cudaGetLastError();
}

template <class T, int L>
static cudaError_t run_born_1d(const Born1DArgs &a, cudaStream_t st)
{
    constexpr int P = born_prec<T>(), E = born_e(P);
    constexpr int PADS = P ? 4 : 3;
    const size_t smem = sizeof(cplx_t<T>) * padded<L, PADS>(L);
    auto k = k_born1d<T, L, E>;
    cudaError_t e = prepare_smem(k, smem);
    if (e != cudaSuccess) return e;
    k<<<1, L / E, smem, st>>>(a);
    return cudaGetLastError();
}

template <class T, int N2>
static cudaError_t run_born_fs_col(int n1, const BornFsColArgs &a, cudaStream_t st)
{
    constexpr int P = born_prec<T>(), E = born_e(P), W = born_fs_w(P, N2);
    const size_t smem = sizeof(cplx_t<T>) * col_tile_elems(sizeof(cplx_t<T>), N2, W, E);
    auto k = k_born_fs_col<T, N2, E, W>;
    cudaError_t e = prepare_smem(k, smem);
    if (e != cudaSuccess) return e;
    k<<<n1 / W, W * (N2 / E), smem, st>>>(a);
    return cudaGetLastError();
}

template <class T, int N1>
static cudaError_t run_born_fs_row(int n2, const BornFsRowArgs &a, cudaStream_t st)
{
    constexpr int P = born_prec<T>(), E = born_e(P), B = born_fs_b(P, N1);
    constexpr int PADS = P ? 4 : 3;
    const size_t smem = sizeof(cplx_t<T>) * B * padded<N1, PADS>(N1);
    auto k = k_born_fs_row<T, N1, E, B>;
    cudaError_t e = prepare_smem(k, smem);
    if (e != cudaSuccess) return e;
    k<<<n2 / B, B * (N1 / E), smem, st>>>(a);
    return cudaGetLastError();
}

#define QSG_BORN_2D_SIZES(X) X(64) X(128) X(256) X(512) X(1024) X(2048) X(4096)

template <class T, int NY>
static cudaError_t run_born_row_g(int nx, const BornRowArgs &a, cudaStream_t st)
{
    constexpr int P = born_prec<T>(), TL = NY / born_e(P);
    switch (born_split(P, nx, NY)) {
    case 1: return run_born_row<T, NY, 1>(nx, a, st);
    case 2: if constexpr (2 * TL <= 512) return run_born_row<T, NY, 2>(nx, a, st); break;
    case 4: if constexpr (4 * TL <= 512) return run_born_row<T, NY, 4>(nx, a, st); break;
    default: break;
    }
    return cudaErrorNotSupported;
}

template <class T> cudaError_t born_row(int nx, int ny, const BornRowArgs &a, cudaStream_t st)
{
#define X(N) case N: return run_born_row_g<T, N>(nx, a, st);
    switch (ny) { QSG_BORN_2D_SIZES(X) default: break; }
#undef X
    return cudaErrorNotSupported;
}

// the column pass runs on blocks of M = nx / G rows
template <class T> cudaError_t born_col(int nx, int ny, const BornColArgs &a, cudaStream_t st)
{
    const int g = born_split(born_prec<T>(), nx, ny);
#define X(N) case N: return run_born_col<T, N>(ny, g, a, st);
    switch (nx / g) { QSG_BORN_2D_SIZES(X) default: break; }
#undef X
    return cudaErrorNotSupported;
}

template <class T> cudaError_t born_1d(int n, const Born1DArgs &a, cudaStream_t st)
{
#define X(N) case N: return run_born_1d<T, N>(a, st);
    if constexpr (sizeof(T) == 4) {
        switch (n) { X(128) X(256) X(512) X(1024) X(2048) X(4096) X(8192) default: break; }
    } else {
        switch (n) { X(128) X(256) X(512) X(1024) X(2048) X(4096) default: break; }
    }
#undef X
    return cudaErrorNotSupported;
}

template <class T> cudaError_t born_fs_col(int n1, int n2, const BornFsColArgs &a, cudaStream_t st)
{
#define X(N) case N: return run_born_fs_col<T, N>(n1, a, st);
    switch (n2) { X(64) X(128) X(256) X(512) X(1024) X(2048) default: break; }
#undef X
    return cudaErrorNotSupported;
}

template <class T> cudaError_t born_fs_row(int n1, int n2, const BornFsRowArgs &a, cudaStream_t st)
{
#define X(N) case N: return run_born_fs_row<T, N>(n2, a, st);
    switch (n1) { X(128) X(256) X(512) X(1024) X(2048) default: break; }
#undef X
    return cudaErrorNotSupported;
}

template <class T> cudaError_t born_xsec(int nx, const BornXsecArgs &a, cudaStream_t st)
{
    k_born_xsec<T><<<born_xsec_blocks(nx), kXsecThreads, 0, st>>>(a);
    return cudaGetLastError();
}

#define QSG_BORN_INSTANTIATE(T)                                                                      \
    template cudaError_t born_row<T>(int, int, const BornRowArgs &, cudaStream_t);                \
    template cudaError_t born_col<T>(int, int, const BornColArgs &, cudaStream_t);                \
    template cudaError_t born_1d<T>(int, const Born1DArgs &, cudaStream_t);                       \
    template cudaError_t born_fs_col<T>(int, int, const BornFsColArgs &, cudaStream_t);           \
    template cudaError_t born_fs_row<T>(int, int, const BornFsRowArgs &, cudaStream_t);           \
    template cudaError_t born_xsec<T>(int, const BornXsecArgs &, cudaStream_t);

}  // namespace qsg
