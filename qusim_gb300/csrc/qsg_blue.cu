// Split-operator steps on lengths that are not powers of two (Bluestein,
// qsg_blue.cuh): instantiations, launchers and the host-side tables.
#include <algorithm>
#include <cmath>
#include <complex>
#include <thread>
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

namespace {

// Double-double numbers (an unevaluated sum hi + lo, |lo| <= ulp(hi) / 2, about
// 106 bits): Knuth's two-sum and the fused-multiply-add exact product
// (Dekker 1971; Hida, Li and Bailey's QD library describes the same operations).
// The long tables need more than double's 53 bits: an error in FFT_M(h) repeats
// at every kinetic factor, and binary128 long double is software arithmetic on
// some hosts (tens of seconds for 2^22 entries).
struct dd {
    double hi, lo;
};
inline dd quick_two_sum(double a, double b)
{
    const double s = a + b;
    return dd{s, b - (s - a)};
}
inline dd two_sum(double a, double b)
{
    const double s = a + b;
    const double bb = s - a;
    return dd{s, (a - (s - bb)) + (b - bb)};
}
inline dd dd_add(dd a, dd b)
{
    dd s = two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return quick_two_sum(s.hi, s.lo);
}
inline dd dd_neg(dd a) { return dd{-a.hi, -a.lo}; }
inline dd dd_mul(dd a, dd b)
{
    // the rounded product as an fma with zero: a plain product could be contracted
    // with the sum below into one fused operation, which the error term assumes it is not
    const double p = std::fma(a.hi, b.hi, 0.0);
    const double e = std::fma(a.hi, b.hi, -p) + (a.hi * b.lo + a.lo * b.hi);
    return quick_two_sum(p, e);
}
inline dd dd_from_ld(long double x)
{
    const double hi = (double)x;
    return dd{hi, (double)(x - (long double)hi)};
}
struct cdd {
    dd re, im;
};
inline cdd c_add(cdd a, cdd b) { return cdd{dd_add(a.re, b.re), dd_add(a.im, b.im)}; }
inline cdd c_sub(cdd a, cdd b) { return cdd{dd_add(a.re, dd_neg(b.re)), dd_add(a.im, dd_neg(b.im))}; }
inline cdd c_mul(cdd a, cdd b)
{
    return cdd{dd_add(dd_mul(a.re, b.re), dd_neg(dd_mul(a.im, b.im))),
               dd_add(dd_mul(a.re, b.im), dd_mul(a.im, b.re))};
}
inline cdd c_conj(cdd a) { return cdd{a.re, dd_neg(a.im)}; }

// exp(-i pi q / half) for q < 2 half as products A[q / S] B[q % S] of two short
// tables from cosl / sinl (a few thousand calls instead of one per entry)
struct RootTable {
    uint64_t half, S;
    std::vector<cdd> A, B;
    explicit RootTable(uint64_t half_) : half(half_), S(1)
    {
        while (S * S < 2 * half) S <<= 1;
        const long double pi = 3.141592653589793238462643383279502884197L;
        auto root = [&](uint64_t q) {
            const long double ang = -pi * (long double)q / (long double)half;
            return cdd{dd_from_ld(cosl(ang)), dd_from_ld(sinl(ang))};
        };
        for (uint64_t a = 0; a * S < 2 * half; ++a) A.push_back(root(a * S));
        for (uint64_t b = 0; b < S; ++b) B.push_back(root(b));
    }
    cdd operator()(uint64_t q) const { return c_mul(A[q / S], B[q % S]); }
};

// run f(lo, hi) over [0, count) on the host's threads
template <class F> void parallel_for(uint64_t count, F f)
{
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const uint64_t nt = count < 4096 ? 1 : std::min<uint64_t>(hw, count / 4096);
    if (nt <= 1) {
        f(uint64_t(0), count);
        return;
    }
    std::vector<std::thread> th;
    for (uint64_t t = 0; t < nt; ++t)
        th.emplace_back(f, count * t / nt, count * (t + 1) / nt);
    for (auto &x : th) x.join();
}

// in-place forward DFT of a power-of-two length in double-double: bit reversal,
// then radix-2 stages whose twiddles exp(-2 pi i k / len) are entries of one
// root table of the full length (stride m / len)
void dft_dd(std::vector<cdd> &a)
{
    const uint64_t m = a.size();
    for (uint64_t i = 1, j = 0; i < m; ++i) {
        uint64_t bit = m >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) std::swap(a[i], a[j]);
    }
    // roots of the full length: exp(-2 pi i k / m) = exp(-i pi k / (m / 2)), k < m / 2
    const RootTable rt(m / 2);
    std::vector<cdd> roots(m / 2);
    parallel_for(m / 2, [&](uint64_t lo, uint64_t hi) {
        for (uint64_t k = lo; k < hi; ++k) roots[k] = rt(k);
    });
    for (uint64_t len = 2; len <= m; len <<= 1) {
        const uint64_t half = len / 2, stride = m / len;
        // butterflies (block i, position k) numbered b = (i / len) * half + k
        parallel_for(m / 2, [&](uint64_t lo, uint64_t hi) {
            for (uint64_t b = lo; b < hi; ++b) {
                const uint64_t i = (b / half) * len, k = b % half;
                const cdd u = a[i + k], v = c_mul(a[i + k + half], roots[k * stride]);
                a[i + k] = c_add(u, v);
                a[i + k + half] = c_sub(u, v);
            }
        });
    }
}

std::complex<double> to_c(const cdd &z) { return {z.re.hi + z.re.lo, z.im.hi + z.im.lo}; }

}  // namespace

void blue_tables_dd(uint64_t n, uint64_t m, std::vector<std::complex<double>> &w,
                    std::vector<std::complex<double>> &hs)
{
    // chirp w_j = exp(-i pi (j^2 mod 2n) / n), h = conj(w) laid out circularly
    const RootTable rt(n);
    std::vector<cdd> wd(n), h(m, cdd{dd{0, 0}, dd{0, 0}});
    parallel_for(n, [&](uint64_t lo, uint64_t hi) {
        for (uint64_t j = lo; j < hi; ++j) {
            wd[j] = rt((j * j) % (2 * n));
            h[j] = c_conj(wd[j]);
            if (j) h[m - j] = c_conj(wd[j]);
        }
    });
    dft_dd(h);
    w.assign(m, 0.0);
    for (uint64_t j = 0; j < n; ++j) w[j] = to_c(wd[j]);
    hs.resize(m);
    const double inv_m = 1.0 / (double)m;  // a power of two: exact
    for (uint64_t k = 0; k < m; ++k) hs[k] = to_c(h[k]) * inv_m;
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
