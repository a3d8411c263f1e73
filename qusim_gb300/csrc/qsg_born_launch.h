// qsg_born_launch.h -- launch geometry and launchers of the Born-series
// kernels (qsg_born.cuh).  Each launcher picks the instantiation for the
// runtime size; sizes without one return cudaErrorNotSupported.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector_types.h>

namespace qsg {

// post-update kinds
enum BornPost : int {
    BORN_POST_NEW = 0,        // dpsi = new
    BORN_POST_LINEAR = 1,     // dpsi = dpsi (1 - slow) + new slow      (op_LinearUpdate)
    BORN_POST_VELLEKOOP = 2,  // g = (1 - i V / eps) slow               (op_Vellekoop)
    BORN_POST_HAO1 = 3,       // g = (1 - i conj(V) / eps) slow         (op_Hao1)
    BORN_POST_HAO2 = 4,       // g = 2 / (1 + i V / eps) slow           (op_Hao2)
};

struct BornOps {
    double eps, slow;
    int pre;   // 0 naive, 1 preconditioned
    int post;  // BornPost
};

// 2D real-space pass (k_born_row)
struct BornRowArgs {
    const void *in;       // in_k: rows of the k-space scratch; else dpsi (natural)
    void *tmp;            // out_k: where pre(dpsi) goes after the row FFT
    const void *dold;     // dpsi before the update (post reads it), or null
    void *dnew;           // where the updated dpsi goes, or null
    const void *dstart;   // dpsi at the start of Compute (delta-psi norm), with partials
    const void *V;
    const void *ex, *ey;  // psi0 = ex[row] * ey[col]
    const void *tw;       // stage twiddles (NY, E)
    const void *tw_nx;    // exp(-2 pi i m / Nx), m < Nx (x-split twiddles)
    double *partials;     // 2 per CTA: sum |dnew - dstart|^2, sum |dnew|^2 (or null)
    BornOps ops;
    int m;                // Nx / G
    int in_k, out_k;      // input in split-k space / output to split-k space
};

// 2D k-space pass (k_born_col)
struct BornColArgs {
    void *tmp;           // in/out, natural k layout (kx row, ky column)
    const double *gx;    // E - fold(kx)^2 DPx^2/2m, Nx entries
    const double *gy;    // fold(ky)^2 DPy^2/2m, Ny entries
    const float2 *gx2;   // the same tables as float hi + lo pairs (complex64 path)
    const float2 *gy2;
    const void *tw;      // stage twiddles (M, E)
    double eps, inv_n;
    int ny, g;           // g: the x split (M = Nx / g)
};

// 1D, one CTA per instance (k_born1d)
struct Born1DArgs {
    void *dpsi;           // in/out, natural
    const void *psi0;     // exp(i dir k0 x)
    const void *V;
    const void *tw;       // stage twiddles (L, E)
    double en, dk2;       // E and (2 pi hbar / (dx n))^2 / 2m
    float2 enf, dkf;      // the same as float hi + lo pairs (complex64 path)
    double inv_n;
    double *sums;         // 4 doubles: r (re, im), t (re, im) before the prefactor
    BornOps ops;
    int order;
};

// 1D four-step passes (k_born_fs_col / k_born_fs_row)
struct BornFsColArgs {
    const void *in;       // in_k: the k-layout scratch; else dpsi (natural)
    void *tmp;            // out_k: where pre(dpsi) goes (column FFT + twiddle)
    const void *dold;     // dpsi before the update, or null
    void *dnew;           // updated dpsi, or null
    const void *psi0, *V; // natural
    const void *tw;       // stage twiddles (N2, E)
    const void *tw_n;     // exp(-2 pi i r c / N) at r * n1 + c (row r < n2, column c < n1)
    double *partials;     // last pass: 4 per CTA, the ComputeRT sums (or null)
    BornOps ops;
    int n1;
    int in_k, out_k;
};

struct BornFsRowArgs {
    void *tmp;            // in/out, k layout
    const void *tw;       // stage twiddles (N1, E)
    double en, dk2, eps, inv_n;
    float2 enf, dkf;      // en, dk2 as float hi + lo pairs (complex64 path)
    int n, n2;
};

// 2D scattering amplitudes (k_born_xsec)
struct BornXsecArgs {
    const void *dpsi, *V, *ex, *ey;
    const double2 *ax;    // na x nx
    const double2 *ay;    // na x ny
    double *partials;     // per CTA: na complex (re, im)
    int nx, ny, na;
};

// elements per thread: 16 (complex64), 8 (complex128)
constexpr int born_e(int prec) { return prec == 1 ? 16 : 8; }

// 2D: nx, ny in 64 .. 4096 (powers of two)
bool born2d_supported(int nx, int ny);
// 1D: one CTA holds the instance (n <= 8192 complex64, 4096 complex128), or
// four-step n = n1 * n2 up to 2^22
bool born1d_resident(int prec, uint64_t n);
bool born1d_supported(int prec, uint64_t n);
void born_fs_split(uint64_t n, int *n1, int *n2);

// column-transform radix of the 2D k-space pass
constexpr int born_col_e(int prec, int m) { return prec == 1 ? (m >= 512 ? 32 : 16) : (m >= 2048 ? 16 : 8); }
// the x split of an nx x ny grid: column blocks of <= 1024 rows (complex64) /
// 512 (complex128), as far as a CTA of G rows of ny stays within 512 threads
int born_split(int prec, int nx, int ny);

int born_row_blocks(int prec, int nx, int ny);       // CTAs of a 2D row pass
int born_fs_col_blocks(int prec, int n1, int n2);    // CTAs of a four-step column pass

template <class T> cudaError_t born_row(int nx, int ny, const BornRowArgs &a, cudaStream_t st);
template <class T> cudaError_t born_col(int nx, int ny, const BornColArgs &a, cudaStream_t st);
template <class T> cudaError_t born_1d(int n, const Born1DArgs &a, cudaStream_t st);
template <class T> cudaError_t born_fs_col(int n1, int n2, const BornFsColArgs &a, cudaStream_t st);
template <class T> cudaError_t born_fs_row(int n1, int n2, const BornFsRowArgs &a, cudaStream_t st);
template <class T> cudaError_t born_xsec(int nx, const BornXsecArgs &a, cudaStream_t st);
int born_xsec_blocks(int nx);

}  // namespace qsg
