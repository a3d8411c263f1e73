// qsg_aux.cu -- phase tables, reductions, conversions.
#include "qsg_aux.h"
#include <type_traits>
#include "qsg_kernels.cuh"

namespace qsg {

namespace {

constexpr int kThreads = 256;

inline unsigned blocks_for(size_t n, int per_block = kThreads)
{
    size_t b = (n + per_block - 1) / per_block;
    return (unsigned)(b > 1048576 ? 1048576 : (b ? b : 1));
}

// sin and cos in fp64.  The phase arguments of the potential tables are small
// (|V dt c / hbar| is 0.07 on the 4096^2 benchmark), where the Taylor series of
// sin and cos, summed in Horner form to the y^13 / y^14 terms, is within an ulp
// or two for |y| <= 1/4 (the first dropped terms are below 2^-56 relative) at
// about a third of the general routine's cost; larger arguments take sincos.
__device__ __forceinline__ void sincos_d(double y, double *s, double *c)
{
    if (fabs(y) > 0.25) {
        sincos(y, s, c);
        return;
    }
    const double z = y * y;
    double ps = -1.0 / 6227020800.0;                     // -1/13!
    ps = fma(ps, z, 1.0 / 39916800.0);                   //  1/11!
    ps = fma(ps, z, -1.0 / 362880.0);                    // -1/9!
    ps = fma(ps, z, 1.0 / 5040.0);                       //  1/7!
    ps = fma(ps, z, -1.0 / 120.0);                       // -1/5!
    ps = fma(ps, z, 1.0 / 6.0);                          //  1/3!
    *s = fma(-y * z, ps, y);                             // y - y^3/3! + y^5/5! - ...
    double pc = 1.0 / 87178291200.0;                     //  1/14!
    pc = fma(pc, z, -1.0 / 479001600.0);                 // -1/12!
    pc = fma(pc, z, 1.0 / 3628800.0);                    //  1/10!
    pc = fma(pc, z, -1.0 / 40320.0);                     // -1/8!
    pc = fma(pc, z, 1.0 / 720.0);                        //  1/6!
    pc = fma(pc, z, -1.0 / 24.0);                        // -1/4!
    pc = fma(pc, z, 0.5);                                //  1/2!
    *c = fma(-z, pc, 1.0);                               // 1 - y^2/2! + y^4/4! - ...
}

// exp(z) and exp(z) - 1 in fp64.  The "-1" form keeps relative accuracy for
// small |z|: re = expm1(x) - 2 e^x sin^2(y/2), im = e^x sin y.
// A real time step (x == 0, the usual case) needs no exp / expm1, and the
// "-1" form then needs a single sincos of y/2 (sin y = 2 sin(y/2) cos(y/2)).
// FP64 transcendentals are the whole cost of building a table on this part.
__device__ __forceinline__ double2 cexp_d(double x, double y)
{
    double s, c;
    sincos_d(y, &s, &c);
    const double ex = x == 0.0 ? 1.0 : exp(x);
    return make_double2(ex * c, ex * s);
}
__device__ __forceinline__ float2 cexpm1_f(double x, double y)
{
    if (x == 0.0 && fabs(y) <= 0.5) {
        // half angle h = y/2 (|h| <= 1/4): sin h = h - h^3 P(h^2), cos h = 1 - h^2 Q(h^2).
        // Only the corrections h^3 P (at most 1.1% of sin h) and h^2 Q (at most 3.2% of
        // cos h) are summed in fp32: their rounding moves the fp64 sums by under 3e-9
        // relative, a twentieth of the fp32 ulp the table entries are rounded to.
        // (Series through h^9 / h^10: the first terms left out are below 1e-12 relative.)
        const double h = 0.5 * y;
        const float hf = (float)h, z = hf * hf;
        const float P = fmaf(fmaf(fmaf(-1.0f / 362880.0f, z, 1.0f / 5040.0f), z, -1.0f / 120.0f), z, 1.0f / 6.0f);
        const float Q = fmaf(fmaf(fmaf(fmaf(1.0f / 3628800.0f, z, -1.0f / 40320.0f), z, 1.0f / 720.0f), z,
                                 -1.0f / 24.0f),
                            z, 0.5f);
        const double sh = h - (double)(hf * z * P), ch = 1.0 - (double)(z * Q);
        return make_float2(float(-2.0 * sh * sh), float(2.0 * sh * ch));
    }
    double sh, ch;
    sincos_d(0.5 * y, &sh, &ch);
    if (x == 0.0) return make_float2(float(-2.0 * sh * sh), float(2.0 * sh * ch));
    double s, c;
    sincos_d(y, &s, &c);
    const double ex = exp(x);
    return make_float2(float(expm1(x) - 2.0 * ex * sh * sh), float(ex * s));
}

template <class C> __device__ __forceinline__ C phase_entry(double x, double y, double scale);
template <> __device__ __forceinline__ double2 phase_entry<double2>(double x, double y, double scale)
{
    double2 r = cexp_d(x, y);
    return make_double2(r.x * scale, r.y * scale);
}
template <> __device__ __forceinline__ float2 phase_entry<float2>(double x, double y, double)
{
    return cexpm1_f(x, y);
}

template <class C>
__global__ void k_vtable(C *out, const double *V, size_t n, double fre, double fim)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double v = V[i];
        out[i] = phase_entry<C>(fre * v, fim * v, 1.0);
    }
}

template <class C>
__global__ void k_ktable1d(C *out, int n, double fre, double fim, double scale)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double f = double(i > n / 2 ? n - i : i);
        const double s = f * f;
        out[i] = phase_entry<C>(fre * s, fim * s, scale);
    }
}

template <class C>
__global__ void k_ktable_wall(C *out, int n, double fre, double fim, double scale)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double s = double(i) * double(i);
        out[i] = phase_entry<C>(fre * s, fim * s, scale);
    }
}

template <class C>
__global__ void k_ktable_fs(C *out, int n1, int n2, double fre, double fim, double scale)
{
    const long n = (long)n1 * n2;
    for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < n; idx += (long)gridDim.x * blockDim.x) {
        const long k2 = idx / n1, k1 = idx % n1;
        const long k = k2 + (long)n2 * k1;
        const double f = double(k > n / 2 ? n - k : k);
        const double s = f * f;
        out[idx] = phase_entry<C>(fre * s, fim * s, scale);
    }
}

__global__ void k_ktable2d(double2 *out, int nx, int ny, double are, double aim, double dtx, double dty,
                           double scale)
{
    const size_t n = (size_t)nx * ny;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int i = int(idx / ny), j = int(idx % ny);
        const double fi = double(i > nx / 2 ? nx - i : i), fj = double(j > ny / 2 ? ny - j : j);
        const double s = (fi * fi) * dtx + (fj * fj) * dty;
        out[idx] = phase_entry<double2>(are * s, aim * s, scale);
    }
}

__global__ void k_c128_to_c64(float2 *out, const double2 *in, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double2 v = in[i];
        out[i] = make_float2(float(v.x), float(v.y));
    }
}
__global__ void k_c64_to_c128(double2 *out, const float2 *in, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float2 v = in[i];
        out[i] = make_double2(double(v.x), double(v.y));
    }
}

// Sum of |psi|^2 in FP32 with no rounding loss that matters: each square is
// split exactly into p + e (p = x*x, e = fma(x, x, -p)) and the running sum is
// a float pair (hi, lo) updated by two-sum (Knuth), so the per-thread result
// carries about 48 bits before it is handed to the FP64 block sum.  FP64 runs
// at 1/64 of the FP32 rate on this part: summing float2 values in FP64 made
// the reduction issue-bound at a fraction of HBM bandwidth.
struct SumF2 {
    float hi = 0.f, lo = 0.f;
    // explicit round-to-nearest intrinsics: the compiler may not contract
    // or reassociate them, which the two-sum identities rely on
    __device__ __forceinline__ void add(float v)
    {
        const float s = __fadd_rn(hi, v);
        const float bv = __fsub_rn(s, hi);
        lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bv)), __fsub_rn(v, bv)));
        hi = s;
    }
    __device__ __forceinline__ void add_sq(float x)
    {
        const float p = __fmul_rn(x, x);
        add(p);
        lo = __fadd_rn(lo, fmaf(x, x, -p));
    }
    __device__ __forceinline__ double value() const { return double(hi) + double(lo); }
};

template <class C, int MODE>
__device__ __forceinline__ void reduce_add(double &s, SumF2 &f, C a, const double *V, size_t i, size_t lo)
{
    if constexpr (MODE == 0 && std::is_same<C, float2>::value) {
        f.add_sq(a.x);
        f.add_sq(a.y);
    } else {
        const double a2 = abs2d(a);
        s += MODE == 0 ? a2 : (MODE == 1 ? a2 * V[i] : a2 * double(i - lo));
    }
}

template <class C, int MODE>
__global__ void __launch_bounds__(kThreads) k_reduce(const C *__restrict__ psi, const double *__restrict__ V,
                                                     size_t lo, size_t hi, double *partials)
{
    __shared__ double red[32];
    double s = 0;
    SumF2 f;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t i = lo + blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    // four independent loads in flight per thread
    for (; i + 3 * stride < hi; i += 4 * stride) {
        const C a0 = psi[i], a1 = psi[i + stride], a2 = psi[i + 2 * stride], a3 = psi[i + 3 * stride];
        reduce_add<C, MODE>(s, f, a0, V, i, lo);
        reduce_add<C, MODE>(s, f, a1, V, i + stride, lo);
        reduce_add<C, MODE>(s, f, a2, V, i + 2 * stride, lo);
        reduce_add<C, MODE>(s, f, a3, V, i + 3 * stride, lo);
    }
    for (; i < hi; i += stride) reduce_add<C, MODE>(s, f, psi[i], V, i, lo);
    s += f.value();
    s = block_sum<kThreads>(s, red);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kThreads) k_finalize(const double *partials, int nparts, int stride,
                                                       double *out)
{
    __shared__ double red[32];
    for (int k = 0; k < stride; ++k) {
        double s = 0;
        for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += partials[(size_t)i * stride + k];
        s = block_sum<kThreads>(s, red);
        if (threadIdx.x == 0) out[k] = s;
    }
}

template <class C, class T>
__global__ void k_renorm(C *psi, size_t n, const double *sum, double dv)
{
    const T sc = T(1.0 / sqrt(sum[0] * dv));
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        C v = psi[i];
        v.x *= sc;
        v.y *= sc;
        psi[i] = v;
    }
}

}  // namespace

cudaError_t launch_vtable(int prec, void *out, const double *V, size_t n, double fre, double fim,
                          cudaStream_t st)
{
    if (prec == 1)
        k_vtable<float2><<<blocks_for(n), kThreads, 0, st>>>((float2 *)out, V, n, fre, fim);
    else
        k_vtable<double2><<<blocks_for(n), kThreads, 0, st>>>((double2 *)out, V, n, fre, fim);
    return cudaGetLastError();
}

cudaError_t launch_ktable1d(int prec, void *out, int n, double fre, double fim, double scale,
                            cudaStream_t st)
{
    if (prec == 1)
        k_ktable1d<float2><<<blocks_for(n), kThreads, 0, st>>>((float2 *)out, n, fre, fim, scale);
    else
        k_ktable1d<double2><<<blocks_for(n), kThreads, 0, st>>>((double2 *)out, n, fre, fim, scale);
    return cudaGetLastError();
}

__global__ void k_sample_spec(SpecArgs a, int nx, int ny, double2 *psi, double *V)
{
    const size_t n = (size_t)nx * ny;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(idx / ny), j = (int)(idx - (size_t)i * ny);
        const double x = a.x0 + i * a.dx;
        const double y = a.dim == 2 ? a.y0 + j * a.dy : 0.0;
        const double rx = x - a.cx, ry = a.dim == 2 ? y - a.cy : 0.0;
        const double env = exp(-(rx * rx + ry * ry) / (4.0 * a.s * a.s));
        double sp, cp;
        sincos(a.kx * x + (a.dim == 2 ? a.ky * y : 0.0), &sp, &cp);
        psi[idx] = make_double2(env * cp, env * sp);
        double v = a.v0;
        for (int b = 0; b < a.nbumps; ++b) {
            const double bx = x - a.bumps[b][1], by = a.dim == 2 ? y - a.bumps[b][2] : 0.0;
            const double w = a.bumps[b][3];
            v += a.bumps[b][0] * exp(-(bx * bx + by * by) / (2.0 * w * w));
        }
        V[idx] = v;
    }
}

cudaError_t launch_sample_spec(const SpecArgs &a, int nx, int ny, void *psi, double *V, cudaStream_t st)
{
    k_sample_spec<<<blocks_for((size_t)nx * ny), kThreads, 0, st>>>(a, nx, ny, (double2 *)psi, V);
    return cudaGetLastError();
}

cudaError_t launch_ktable_wall(int prec, void *out, int n, double fre, double fim, double scale, cudaStream_t st)
{
    if (prec == 1)
        k_ktable_wall<float2><<<blocks_for(n), kThreads, 0, st>>>((float2 *)out, n, fre, fim, scale);
    else
        k_ktable_wall<double2><<<blocks_for(n), kThreads, 0, st>>>((double2 *)out, n, fre, fim, scale);
    return cudaGetLastError();
}

cudaError_t launch_ktable_fs(int prec, void *out, int n1, int n2, double fre, double fim, double scale,
                             cudaStream_t st)
{
    const size_t n = (size_t)n1 * n2;
    if (prec == 1)
        k_ktable_fs<float2><<<blocks_for(n), kThreads, 0, st>>>((float2 *)out, n1, n2, fre, fim, scale);
    else
        k_ktable_fs<double2><<<blocks_for(n), kThreads, 0, st>>>((double2 *)out, n1, n2, fre, fim, scale);
    return cudaGetLastError();
}

cudaError_t launch_ktable2d(void *out, int nx, int ny, double are, double aim, double dtx,
                            double dty, double scale, cudaStream_t st)
{
    k_ktable2d<<<blocks_for((size_t)nx * ny), kThreads, 0, st>>>((double2 *)out, nx, ny, are, aim, dtx,
                                                                  dty, scale);
    return cudaGetLastError();
}

cudaError_t launch_c128_to_c64(void *out, const void *in, size_t n, cudaStream_t st)
{
    k_c128_to_c64<<<blocks_for(n), kThreads, 0, st>>>((float2 *)out, (const double2 *)in, n);
    return cudaGetLastError();
}

cudaError_t launch_c64_to_c128(void *out, const void *in, size_t n, cudaStream_t st)
{
    k_c64_to_c128<<<blocks_for(n), kThreads, 0, st>>>((double2 *)out, (const float2 *)in, n);
    return cudaGetLastError();
}

cudaError_t launch_reduce(int prec, const void *psi, const double *V, size_t lo, size_t hi, int mode,
                          double *partials, int max_parts, int *nparts, cudaStream_t st)
{
    // at least 16 sites per thread, at most 8 CTAs per SM of a 152-SM part
    unsigned b = blocks_for(hi > lo ? hi - lo : 1, kThreads * 16);
    if (b > 1216) b = 1216;
    if ((int)b > max_parts) b = (unsigned)max_parts;
    *nparts = (int)b;
#define QSG_REDUCE(C, M) k_reduce<C, M><<<b, kThreads, 0, st>>>((const C *)psi, V, lo, hi, partials)
    if (prec == 1) {
        if (mode == 0) QSG_REDUCE(float2, 0);
        else if (mode == 1) QSG_REDUCE(float2, 1);
        else QSG_REDUCE(float2, 2);
    } else {
        if (mode == 0) QSG_REDUCE(double2, 0);
        else if (mode == 1) QSG_REDUCE(double2, 1);
        else QSG_REDUCE(double2, 2);
    }
#undef QSG_REDUCE
    return cudaGetLastError();
}

cudaError_t launch_finalize(const double *partials, int nparts, int stride, double *out,
                            cudaStream_t st)
{
    k_finalize<<<1, kThreads, 0, st>>>(partials, nparts, stride, out);
    return cudaGetLastError();
}

cudaError_t launch_renorm(int prec, void *psi, size_t n, const double *sum, double dv, cudaStream_t st)
{
    if (prec == 1)
        k_renorm<float2, float><<<blocks_for(n), kThreads, 0, st>>>((float2 *)psi, n, sum, dv);
    else
        k_renorm<double2, double><<<blocks_for(n), kThreads, 0, st>>>((double2 *)psi, n, sum, dv);
    return cudaGetLastError();
}

}  // namespace qsg
