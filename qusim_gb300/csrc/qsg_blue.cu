// Split-operator steps on lengths that are not powers of two (Bluestein,
// qsg_blue.cuh): instantiations, launchers and the host-side tables.
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "qsg_blue.cuh"
#include "qsg_dispatch.cuh"

namespace qsg {

namespace {

constexpr int blue_e(int prec) { return prec == 1 ? 16 : 8; }

template <class T, int M>
cudaError_t run_blue(const BlueArgs &a, cudaStream_t st)
{
    constexpr int E = sizeof(T) == 4 ? 16 : 8;
    constexpr int PADS = sizeof(T) == 4 ? 4 : 3;
    const size_t smem = sizeof(cplx_t<T>) * padded<M, PADS>(M);
    auto k = k_evolve1d_blue<T, M, E>;
    cudaError_t e = prepare_smem(k, smem);
    if (e != cudaSuccess) return e;
    k<<<1, M / E, smem, st>>>(a);
    return cudaGetLastError();
}

template <class T, int M>
cudaError_t run_blue_kin(const BlueArgs &a, double dtk, double *sums, cudaStream_t st)
{
    constexpr int E = sizeof(T) == 4 ? 16 : 8;
    constexpr int PADS = sizeof(T) == 4 ? 4 : 3;
    const size_t smem = sizeof(cplx_t<T>) * padded<M, PADS>(M);
    auto k = k_kinetic1d_blue<T, M, E>;
    cudaError_t e = prepare_smem(k, smem);
    if (e != cudaSuccess) return e;
    k<<<1, M / E, smem, st>>>(a, dtk, sums);
    return cudaGetLastError();
}

// in-place forward DFT of a power-of-two length in long double (iterative
// radix 2, twiddles from cosl / sinl of the exact angle)
void dft_ld(std::vector<std::complex<long double>> &a)
{
    const size_t m = a.size();
    for (size_t i = 1, j = 0; i < m; ++i) {
        size_t bit = m >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(a[i], a[j]);
    }
    const long double two_pi = 6.283185307179586476925286766559005768L;
    for (size_t len = 2; len <= m; len <<= 1) {
        for (size_t k = 0; k < len / 2; ++k) {
            const long double ang = -two_pi * (long double)k / (long double)len;
            const std::complex<long double> wk(cosl(ang), sinl(ang));
            for (size_t i = 0; i < m; i += len) {
                const auto u = a[i + k], v = a[i + k + len / 2] * wk;
                a[i + k] = u + v;
                a[i + k + len / 2] = u - v;
            }
        }
    }
}

}  // namespace

int blue_m_for(int prec, uint64_t n)
{
    if (n < 2) return 0;
    uint64_t m = 256;
    while (m < 2 * n - 1) m <<= 1;
    return m <= 8192 ? (int)m : 0;
}

void blue_tables(uint64_t n, int m, std::vector<std::complex<long double>> &w,
                 std::vector<std::complex<long double>> &hs)
{
    const long double pi = 3.141592653589793238462643383279502884197L;
    w.assign(m, 0.0L);
    std::vector<std::complex<long double>> h(m, 0.0L);
    for (uint64_t j = 0; j < n; ++j) {
        // j^2 mod 2n keeps the angle small (the chirp has period 2n in j^2)
        const uint64_t q = (j * j) % (2 * n);
        const long double ang = -pi * (long double)q / (long double)n;
        w[j] = std::complex<long double>(cosl(ang), sinl(ang));
        h[j] = std::conj(w[j]);
        if (j) h[m - j] = std::conj(w[j]);
    }
    dft_ld(h);
    hs.resize(m);
    for (int k = 0; k < m; ++k) hs[k] = h[k] / (long double)m;
}

cudaError_t launch_evolve1d_blue(int prec, int m, const BlueArgs &a, cudaStream_t st)
{
#define X(T, M) case M: return run_blue<T, M>(a, st);
    if (prec == 1) {
        switch (m) { X(float, 256) X(float, 512) X(float, 1024) X(float, 2048) X(float, 4096) X(float, 8192) default: break; }
    } else {
        switch (m) { X(double, 256) X(double, 512) X(double, 1024) X(double, 2048) X(double, 4096) X(double, 8192) default: break; }
    }
#undef X
    return cudaErrorNotSupported;
}

cudaError_t launch_kinetic1d_blue(int prec, int m, const BlueArgs &a, double dtk, double *sums, cudaStream_t st)
{
#define X(T, M) case M: return run_blue_kin<T, M>(a, dtk, sums, st);
    if (prec == 1) {
        switch (m) { X(float, 256) X(float, 512) X(float, 1024) X(float, 2048) X(float, 4096) X(float, 8192) default: break; }
    } else {
        switch (m) { X(double, 256) X(double, 512) X(double, 1024) X(double, 2048) X(double, 4096) X(double, 8192) default: break; }
    }
#undef X
    return cudaErrorNotSupported;
}

int blue_elems(int prec) { return blue_e(prec); }

// 2D: rows per row-pass CTA (a CTA of >= 256 threads), columns per column-pass CTA
// (a tile of <= 64 KB), for a transform length m
int blue_rows_per_cta(int prec, int m) { return std::max(1, 256 / (m / blue_e(prec))); }
int blue_cols_per_cta(int prec, int m) { return std::max(1, std::min(16, 65536 / (m * (prec == 1 ? 8 : 16)))); }

namespace {

template <class T, int M>
cudaError_t run_row_blue(const Blue2DArgs &a, cudaStream_t st)
{
    constexpr int E = sizeof(T) == 4 ? 16 : 8;
    constexpr int PADS = sizeof(T) == 4 ? 4 : 3;
    constexpr int RPC = (256 / (M / E)) > 1 ? 256 / (M / E) : 1;
    const size_t smem = sizeof(cplx_t<T>) * padded<M, PADS>(M) * RPC;
    auto k = k_row_blue<T, M, E, RPC>;
    cudaError_t e = prepare_smem(k, smem);
    if (e != cudaSuccess) return e;
    k<<<(a.nx + RPC - 1) / RPC, RPC * (M / E), smem, st>>>(a);
    return cudaGetLastError();
}

template <class T, int M> constexpr int col_w_of()
{
    constexpr int w = 65536 / (M * (int)sizeof(cplx_t<T>));
    return w < 1 ? 1 : (w > 16 ? 16 : w);
}

template <class T, int M>
cudaError_t run_col_blue(const Blue2DArgs &a, bool kinetic, double dtx, double dty, double *partials, cudaStream_t st)
{
    constexpr int E = sizeof(T) == 4 ? 16 : 8;
    constexpr int W = col_w_of<T, M>();
    const size_t smem = sizeof(cplx_t<T>) * col_tile_elems(sizeof(cplx_t<T>), M, W);
    const unsigned grid = (unsigned)((a.ny + W - 1) / W);
    if (kinetic) {
        auto k = k_col_blue_kinetic<T, M, E, W>;
        cudaError_t e = prepare_smem(k, smem);
        if (e != cudaSuccess) return e;
        k<<<grid, W * (M / E), smem, st>>>(a, dtx, dty, partials);
    } else {
        auto k = k_col_blue<T, M, E, W>;
        cudaError_t e = prepare_smem(k, smem);
        if (e != cudaSuccess) return e;
        k<<<grid, W * (M / E), smem, st>>>(a);
    }
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_row_blue(int prec, int m, const Blue2DArgs &a, cudaStream_t st)
{
#define X(T, MM) case MM: return run_row_blue<T, MM>(a, st);
    if (prec == 1) {
        switch (m) { X(float, 256) X(float, 512) X(float, 1024) X(float, 2048) X(float, 4096) X(float, 8192) default: break; }
    } else {
        switch (m) { X(double, 256) X(double, 512) X(double, 1024) X(double, 2048) X(double, 4096) X(double, 8192) default: break; }
    }
#undef X
    return cudaErrorNotSupported;
}

cudaError_t launch_col_blue(int prec, int m, const Blue2DArgs &a, bool kinetic, double dtx, double dty,
                            double *partials, cudaStream_t st)
{
#define X(T, MM) case MM: return run_col_blue<T, MM>(a, kinetic, dtx, dty, partials, st);
    if (prec == 1) {
        switch (m) { X(float, 256) X(float, 512) X(float, 1024) X(float, 2048) X(float, 4096) X(float, 8192) default: break; }
    } else {
        switch (m) { X(double, 256) X(double, 512) X(double, 1024) X(double, 2048) X(double, 4096) X(double, 8192) default: break; }
    }
#undef X
    return cudaErrorNotSupported;
}

}  // namespace qsg
