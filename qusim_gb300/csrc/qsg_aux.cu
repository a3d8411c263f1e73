// qsg_aux.cu -- phase tables, reductions, conversions.
#include "qsg_aux.h"
#include "qsg_kernels.cuh"

namespace qsg {

namespace {

constexpr int kThreads = 256;

inline unsigned blocks_for(size_t n, int per_block = kThreads)
{
    size_t b = (n + per_block - 1) / per_block;
    return (unsigned)(b > 1048576 ? 1048576 : (b ? b : 1));
}

// exp(z) and exp(z) - 1 in fp64.  The "-1" form keeps relative accuracy for
// small |z|: re = expm1(x) - 2 e^x sin^2(y/2), im = e^x sin y.
__device__ __forceinline__ double2 cexp_d(double x, double y)
{
    double s, c;
    sincos(y, &s, &c);
    const double ex = exp(x);
    return make_double2(ex * c, ex * s);
}
__device__ __forceinline__ float2 cexpm1_f(double x, double y)
{
    double s, c, sh, ch;
    sincos(y, &s, &c);
    sincos(0.5 * y, &sh, &ch);
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

template <class C>
__global__ void __launch_bounds__(kThreads) k_reduce(const C *psi, const double *V, size_t lo, size_t hi,
                                                     int mode, double *partials)
{
    __shared__ double red[32];
    double s = 0;
    for (size_t i = lo + blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < hi;
         i += (size_t)gridDim.x * blockDim.x) {
        const double a2 = abs2d(psi[i]);
        s += mode == 0 ? a2 : (mode == 1 ? a2 * V[i] : a2 * double(i - lo));
    }
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
    unsigned b = blocks_for(hi > lo ? hi - lo : 1, kThreads * 8);
    if ((int)b > max_parts) b = (unsigned)max_parts;
    *nparts = (int)b;
    if (prec == 1)
        k_reduce<float2><<<b, kThreads, 0, st>>>((const float2 *)psi, V, lo, hi, mode, partials);
    else
        k_reduce<double2><<<b, kThreads, 0, st>>>((const double2 *)psi, V, lo, hi, mode, partials);
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
