// qsg_evolve3d.cuh -- 3D split-operator passes.
//
// The reference has a 3D transform (KissFourierTransform3D,
// src/FourierTransform.cpp:379-440; z contiguous, index (ix*ny + iy)*nz + iz)
// and a 3D kinetic multiply (MulExpK3D, src/DeviceTemplate.h:851-879), but no 3D
// evolver; this is SplittingMethod2D's step (src/SplittingMethod2D.cpp:38-121)
// with a third axis.  The kinetic factor exp(a (kx^2 DTx + ky^2 DTy + kz^2 DTz))
// is a product of one factor per axis, so the kinetic operator is the product
// of three commuting one-axis operators F_a^-1 K_a F_a: each is one pass over
// the lines along its axis (transform, factor, inverse transform, all on chip),
// and V multiplies fuse into the passes.  A step never leaves natural
// real-space layout:
//
//   O2: z[V V', Kz] y[Ky] x[Kx, (V)]                   3 passes
//   O4: z[V1 V1', Kz1] y[Ky1] x[Kx1, V2] z[Kz2] y[Ky2] x[Kx2, V2]
//       z[Kz1] y[Ky1] x[Kx1, (V1)]                     9 passes
//
// (V' = the previous step's closing factor, merged; (V) only on the last step
// of a call.)  z lines are contiguous (k3_row); y and x lines are strided by nz
// and ny*nz (k3_col, W adjacent z positions per CTA so every access is a W-wide
// contiguous segment).
#pragma once
#include "qsg_kernels.cuh"

namespace qsg {

struct Pass3Args {
    void *psi;
    const void *vpre;      // V factor before the line transforms (or null) ...
    const void *vpost;     // ... and after (or null); natural layout, n entries
    int vpre_twice, vpost_twice;
    const void *k;         // the axis factor: complex64 factor - 1, complex128 factor / L
    const void *tw;        // stage twiddles (L, E)
    float inv_l;           // 1/L (complex64)
    long long s_line;      // stride between a line's elements (strided kernel)
    long long s_outer;     // stride between line groups (strided kernel)
    double *partials;      // kinetic mode: 2 per CTA, sum |X|^2 fold(k)^2 and sum |X|^2
    int kinetic;           // 1: forward transform and the kinetic sums only (no store)
};

template <class C> __device__ __forceinline__ C v3_apply(C x, const C *vt, size_t i, int twice)
{
    const C v = ld_stream(vt + i);
    x = PhaseOps<C>::apply(x, v);
    return twice ? PhaseOps<C>::apply(x, v) : x;
}

// x * K[k] (with 1/L): complex64 cmul1p on the factor - 1 table
template <class C> __device__ __forceinline__ C k3_apply(C x, const C *kt, int k, float inv_l)
{
    if constexpr (sizeof(C) == 8) return cmul1p(cscale(x, inv_l), ld_c(kt + k));
    else return cmul(x, ld_c(kt + k));
}

// B contiguous lines (z) of L per CTA
// strided passes: three 256-thread CTAs per SM (registers capped at 85), as
// they are bound by the latency of their scattered loads, not by issue
constexpr int min_blocks3(int threads) { return threads <= 256 ? 3 : 1; }

template <class T, int L, int E, int B>
__global__ void __launch_bounds__(B *(L / E)) k3_row(Pass3Args a)
{
    using C = cplx_t<T>;
    constexpr int TL = Plan<L, E>::TL;
    constexpr int NT = B * TL;
    constexpr int PADS = sizeof(C) == 8 ? 4 : 3;
    constexpr int LINE = padded<L, PADS>(L);
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[32];
    C *sm = reinterpret_cast<C *>(smraw);
    const int tid = threadIdx.x;
    const int line = tid / TL, t = tid - line * TL;
    const size_t base = ((size_t)blockIdx.x * B + line) * L + t;
    const RowLayout<PADS> lay{line * LINE};
    const auto lbar = LineBarrierOf<TL, B>::make(line);
    C *psi = static_cast<C *>(a.psi);
    const tw_t<C> *tw = static_cast<const tw_t<C> *>(a.tw);
    const C *kt = static_cast<const C *>(a.k);

    C x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) x[e] = ld_stream(psi + base + e * TL);
    if (a.kinetic) {
        line_fft<C, L, E, false>(x, sm, lay, lbar, t, tw);
        double s1 = 0, s0 = 0;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int k = t + e * TL;
            const double f = (double)(k > L / 2 ? L - k : k);
            const double m = abs2d(x[e]);
            s1 += m * f * f;
            s0 += m;
        }
        s1 = block_sum<NT>(s1, red);
        s0 = block_sum<NT>(s0, red);
        if (tid == 0) {
            a.partials[2 * blockIdx.x] = s1;
            a.partials[2 * blockIdx.x + 1] = s0;
        }
        return;
    }
    if (a.vpre) {
        const C *vt = opaque(static_cast<const C *>(a.vpre));
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = v3_apply(x[e], vt, base + e * TL, a.vpre_twice);
    }
    // F^-1 K F, the inverse as conj(F(conj(.)))
#pragma unroll 1
    for (int q = 0; q < 2; ++q) {
        line_fft<C, L, E, false>(x, sm, lay, lbar, t, tw);
        if (q == 1) continue;
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = cconj(k3_apply(x[e], kt, t + e * TL, a.inv_l));
    }
#pragma unroll
    for (int e = 0; e < E; ++e) x[e] = cconj(x[e]);
    if (a.vpost) {
        const C *vt = opaque(static_cast<const C *>(a.vpost));
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = v3_apply(x[e], vt, base + e * TL, a.vpost_twice);
    }
    C *o = const_cast<C *>(opaque(psi));
#pragma unroll
    for (int e = 0; e < E; ++e) st_stream(o + base + e * TL, x[e]);
}

// strided lines (y or x): W adjacent z positions, line element i at
// o * s_outer + c + i * s_line (blockIdx.y = o, blockIdx.x * W + lane = c)
template <class T, int L, int E, int W>
__global__ void __launch_bounds__(W *(L / E), min_blocks3(W *(L / E))) k3_col(Pass3Args a)
{
    using C = cplx_t<T>;
    constexpr int TM = Plan<L, E>::TL;
    constexpr int NT = W * TM;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[32];
    C *sm = reinterpret_cast<C *>(smraw);
    const int tid = threadIdx.x;
    const int c = tid % W, t = tid / W;
    const size_t base = (size_t)blockIdx.y * a.s_outer + (size_t)blockIdx.x * W + c + (size_t)t * a.s_line;
    const size_t stride = (size_t)TM * a.s_line;
    constexpr ColPad CP = col_pad(sizeof(C), L, W, E);
    const ColLayout<W, CP.sh, CP.p> lay{c};
    const CtaBarrier bar{};
    C *psi = static_cast<C *>(a.psi);
    const tw_t<C> *tw = static_cast<const tw_t<C> *>(a.tw);
    const C *kt = static_cast<const C *>(a.k);

    C x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) x[e] = ld_stream(psi + base + e * stride);
    if (a.kinetic) {
        line_fft<C, L, E, false>(x, sm, lay, bar, t, tw);
        double s1 = 0, s0 = 0;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int k = t + e * TM;
            const double f = (double)(k > L / 2 ? L - k : k);
            const double m = abs2d(x[e]);
            s1 += m * f * f;
            s0 += m;
        }
        s1 = block_sum<NT>(s1, red);
        s0 = block_sum<NT>(s0, red);
        if (tid == 0) {
            const size_t cta = (size_t)blockIdx.y * gridDim.x + blockIdx.x;
            a.partials[2 * cta] = s1;
            a.partials[2 * cta + 1] = s0;
        }
        return;
    }
    if (a.vpre) {
        const C *vt = opaque(static_cast<const C *>(a.vpre));
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = v3_apply(x[e], vt, base + e * stride, a.vpre_twice);
    }
#pragma unroll 1
    for (int q = 0; q < 2; ++q) {
        line_fft<C, L, E, false>(x, sm, lay, bar, t, tw);
        if (q == 1) continue;
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = cconj(k3_apply(x[e], kt, t + e * TM, a.inv_l));
    }
#pragma unroll
    for (int e = 0; e < E; ++e) x[e] = cconj(x[e]);
    if (a.vpost) {
        const C *vt = opaque(static_cast<const C *>(a.vpost));
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = v3_apply(x[e], vt, base + e * stride, a.vpost_twice);
    }
    C *o = const_cast<C *>(opaque(psi));
#pragma unroll
    for (int e = 0; e < E; ++e) st_stream(o + base + e * stride, x[e]);
}

}  // namespace qsg
