// qsg_born.cuh -- kernel templates of the Born-series scattering solvers.
//
// Reference path (lhprojects/QuSim): QuPerturbation1DImpl / 2DImpl::Compute
// (src/Perturbation1DImpl.cpp:45-71, src/Perturbation2DImpl.cpp:49-83) run
// `order` updates of BornSeries (src/Perburbation.h:238-287) or
// PreconditionalBornSeries (src/Perburbation.h:349-417).  One update is
//
//   a    = pre(dpsi)                 naive: (dpsi + psi0) V            (op_AddMul)
//                                    preconditioned: (Re V + i(Im V + eps)) dpsi
//                                                    + Re V psi0       (op_Add3)
//   dpsi = post(F^-1[G0 F[a]] / N)   G0(k) = 1 / (E - T(k) + i eps)    (G01D / G02D)
//
// with post the identity (naive series; identity preconditioner with slow = 1),
// the linear update dpsi (1 - slow) + new slow (identity preconditioner), or
// (1 - g) dpsi + g new with g(V) of the Vellekoop / Hao1 / Hao2 preconditioners
// (src/DeviceTemplate.h:1021-1078).  The reference spends five device ops and
// two FFTs (each several HBM passes) per update; here an update is
//
//   2D:  real-space row pass   [row iFFT] -> post -> pre -> [row FFT]
//        k-space column pass   column FFT -> G0 / N -> column iFFT
//   1D, n <= 8192:  one CTA runs every update of a Compute in registers
//   1D, larger n:   four-step, the real-space pass strided (column iFFT, post,
//                   pre, column FFT, twiddles), the k-space pass contiguous
//
// and the real-space pass of one update is fused with that of the next, so an
// update costs two HBM round trips of the scratch array plus the reads of V
// (and of dpsi where the post-update needs the old value).  psi0 is
// exp(i k0.r): a table in 1D, the product of an x and a y table in 2D.
// G0 is formed on the fly from E - T(k), the kinetic part in FP64.
#pragma once
#include "qsg_born_launch.h"
#include "qsg_kernels.cuh"

namespace qsg {



// a = pre(d) at one site; p0 = psi0, v = V there
template <class C> __device__ __forceinline__ C born_pre(const BornOps &o, C d, C p0, C v)
{
    using R = typename RealOf<C>::type;
    if (o.pre == 0) return cmul(cadd(d, p0), v);
    const C a = cmk<C>(v.x, v.y + (R)o.eps);
    const C r = cmul(a, d);
    return cmk<C>(r.x + v.x * p0.x, r.y + v.x * p0.y);
}

// dpsi after the update; f = the transform result (1/N applied), d = dpsi before
template <class C> __device__ __forceinline__ C born_post(const BornOps &o, C f, C d, C v)
{
    using R = typename RealOf<C>::type;
    if (o.post == BORN_POST_NEW) return f;
    const R s = (R)o.slow;
    if (o.post == BORN_POST_LINEAR) return cmk<C>(d.x * (1 - s) + f.x * s, d.y * (1 - s) + f.y * s);
    const R e = (R)o.eps;
    C g;
    if (o.post == BORN_POST_VELLEKOOP) {
        g = cmk<C>(1 + v.y / e, -v.x / e);
    } else if (o.post == BORN_POST_HAO1) {
        g = cmk<C>(1 - v.y / e, -v.x / e);
    } else {
        // 2 / (a + i b), a = 1 - Im V / eps, b = Re V / eps
        const R a = 1 - v.y / e, b = v.x / e;
        const R q = 2 / (a * a + b * b);
        g = cmk<C>(a * q, -b * q);
    }
    g = cscale(g, s);
    const C h = cmk<C>(1 - g.x, -g.y);
    return cadd(cmul(h, d), cmul(g, f));
}

// x * G0 / N for the kinetic term t (FP64): x (e - t - i eps) / ((e - t)^2 + eps^2) / N
template <class C> __device__ __forceinline__ C born_g0(C x, double dr, double eps, double inv_n)
{
    using R = typename RealOf<C>::type;
    if constexpr (sizeof(R) == 8) {
        const double q = inv_n / (dr * dr + eps * eps);
        return cmul(x, cmk<C>(dr * q, -eps * q));
    } else {
        const float d = (float)dr, ef = (float)eps;
        const float q = (float)inv_n / (d * d + ef * ef);
        return cmul(x, cmk<C>(d * q, -ef * q));
    }
}

// complex64 form from float hi + lo tables: E - T = (gx - gy), gx = E - Tx(kx),
// gy = Ty(ky).  The hi difference is exact wherever gx and gy are close
// (Sterbenz), i.e. near the resonance E = T where G0 is large, so the
// denominator keeps its float precision there without FP64 arithmetic.
__device__ __forceinline__ float2 born_g0f(float2 x, float2 gx, float2 gy, float eps, float inv_n)
{
    const float d = __fsub_rn(gx.x, gy.x) + __fsub_rn(gx.y, gy.y);
    const float q = inv_n * __frcp_rn(__fmaf_rn(d, d, eps * eps));
    return cmul(x, make_float2(d * q, -eps * q));
}

__device__ __forceinline__ int born_fold(int i, int n) { return i > n / 2 ? n - i : i; }

// 1D G0 / N at k index fold f, complex64 form: E - f^2 D with E = (eh, el),
// D = (dh, dl) given as float hi + lo pairs and f^2 split exactly into two
// floats, the product formed with an FMA error term (Dekker's two-product),
// so E - T keeps ~1e-14 relative accuracy (of E) in FP32 arithmetic.
__device__ __forceinline__ float2 born_g0_1d(float2 x, int f, float2 en, float2 dk, float eps, float inv_n)
{
    const long long f2 = (long long)f * f;
    const float ah = __ll2float_rz(f2);
    const float al = (float)(f2 - (long long)ah);
    const float p = ah * dk.x;
    const float pe = __fmaf_rn(ah, dk.x, -p);
    const float tl = pe + __fmaf_rn(ah, dk.y, al * dk.x);
    const float d = __fsub_rn(en.x, p) + __fsub_rn(en.y, tl);
    const float q = inv_n * __frcp_rn(__fmaf_rn(d, d, eps * eps));
    return cmul(x, make_float2(d * q, -eps * q));
}
template <class C> __device__ __forceinline__ C born_g0_k(C x, int f, double en, double dk2, float2 enf, float2 dkf,
                                                          double eps, double inv_n)
{
    if constexpr (sizeof(C) == 8) {
        return born_g0_1d(x, f, enf, dkf, (float)eps, (float)inv_n);
    } else {
        const double fd = (double)f;
        return born_g0(x, en - fd * fd * dk2, eps, inv_n);
    }
}

// two CTAs per SM where a CTA has at most 256 threads (registers capped at 128)
constexpr int born_min_blocks(int threads) { return threads <= 256 ? 2 : 1; }

// ---------------------------------------------------------------------------
// 2D real-space pass: B rows of NY per CTA
// ---------------------------------------------------------------------------


// The x split (as in the split-operator passes): a column transform of
// length Nx = G*M is a radix-G decimation-in-frequency stage across the G rows
// n1 + j*M, twiddled by exp(-2 pi i n1 q / Nx), then M-point transforms over
// each block q of M consecutive rows (the k-space pass), where kx = G*k2 + q.
// A CTA holds B groups of those G rows; the stage runs here through shared
// memory, so the column pass reads W-column tiles of length M instead of Nx.
template <class T, int NY, int E, int G, int B>
__global__ void __launch_bounds__(B *G *(NY / E), born_min_blocks(B *G *(NY / E))) k_born_row(BornRowArgs a)
{
    using C = cplx_t<T>;
    constexpr int TL = Plan<NY, E>::TL;
    constexpr int NL = B * G;
    constexpr int NT = NL * TL;
    constexpr int PADS = sizeof(C) == 8 ? 4 : 3;
    constexpr int LINE = padded<NY, PADS>(NY);
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[32];
    C *sm = reinterpret_cast<C *>(smraw);
    const int tid = threadIdx.x;
    const int line = tid / TL, t = tid - line * TL;
    const int b = line / G, j = line - b * G;
    const int m = a.m;
    const int row = blockIdx.x * B + b + j * m;
    const RowLayout<PADS> lay{line * LINE};
    const auto lbar = LineBarrierOf<TL, NL>::make(line);
    const CtaBarrier cbar{};
    const tw_t<C> *tw = static_cast<const tw_t<C> *>(a.tw);
    const tw_t<C> *twx = static_cast<const tw_t<C> *>(a.tw_nx);
    const size_t base = (size_t)row * NY + t;
    const C *V = static_cast<const C *>(a.V) + base;

    C x[E];
    if (a.in_k && G > 1) {
        // inverse x-split stage over every column of the CTA's groups
#pragma unroll 2
        for (int v = 0; v < B * NY / NT; ++v) {
            const int gc = tid + v * NT;
            const int bb = gc / NY, c = gc - bb * NY;
            const int nn1 = blockIdx.x * B + bb;
            C y[G];
#pragma unroll
            for (int q = 0; q < G; ++q) {
                y[q] = ld_stream(static_cast<const C *>(a.in) + (size_t)(q * m + nn1) * NY + c);
                if (q > 0) y[q] = twmul<true>(y[q], __ldg(twx + nn1 * q));
            }
            dftg<G, true>(y);
#pragma unroll
            for (int q = 0; q < G; ++q) sm[(bb * G + q) * LINE + c + (c >> PADS)] = y[q];
        }
        cbar();
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = sm[lay(t + e * TL)];
    } else {
        const C *p = static_cast<const C *>(a.in) + base;
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = ld_stream(p + e * TL);
    }
    double s0 = 0, s1 = 0;
    if (a.in_k) {
        // the inverse row transform as conj(FFT(conj(x)))
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = cconj(x[e]);
        line_fft<C, NY, E, false>(x, sm, lay, lbar, t, tw);
        C v[E], d[E];
#pragma unroll
        for (int e = 0; e < E; ++e) v[e] = ld_stream(V + e * TL);
        if (a.dold) {
            const C *p = static_cast<const C *>(a.dold) + base;
#pragma unroll
            for (int e = 0; e < E; ++e) d[e] = ld_stream(p + e * TL);
        } else {
#pragma unroll
            for (int e = 0; e < E; ++e) d[e] = cmk<C>(0, 0);
        }
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = born_post(a.ops, cconj(x[e]), d[e], v[e]);
        if (a.dnew) {
            C *p = static_cast<C *>(a.dnew) + base;
#pragma unroll
            for (int e = 0; e < E; ++e) st_stream(p + e * TL, x[e]);
        }
        if (a.partials) {
            // complex64: a thread's sums in FP32 (FP64 per element is slow here)
            const C *p = static_cast<const C *>(a.dstart) + base;
            using R = typename RealOf<C>::type;
            R f0 = 0, f1 = 0;
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const C d = csub(x[e], ld_stream(p + e * TL));
                f0 += d.x * d.x + d.y * d.y;
                f1 += x[e].x * x[e].x + x[e].y * x[e].y;
            }
            s0 = f0;
            s1 = f1;
        }
    }
    if (a.out_k) {
        const C ex = __ldg(static_cast<const C *>(a.ex) + row);
        const C *ey = static_cast<const C *>(a.ey) + t;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const C v = ld_stream(opaque(V) + e * TL);
            x[e] = born_pre(a.ops, x[e], cmul(ex, __ldg(ey + e * TL)), v);
        }
        line_fft<C, NY, E, false>(x, sm, lay, lbar, t, opaque(tw));
        if constexpr (G > 1) {
            lbar();  // this line's readers of the last exchange are done
#pragma unroll
            for (int e = 0; e < E; ++e) sm[lay(t + e * TL)] = x[e];
            cbar();
            // forward x-split stage
#pragma unroll 2
            for (int v = 0; v < B * NY / NT; ++v) {
                const int gc = tid + v * NT;
                const int bb = gc / NY, c = gc - bb * NY;
                const int nn1 = blockIdx.x * B + bb;
                C y[G];
#pragma unroll
                for (int q = 0; q < G; ++q) y[q] = sm[(bb * G + q) * LINE + c + (c >> PADS)];
                dftg<G, false>(y);
#pragma unroll
                for (int q = 0; q < G; ++q) {
                    if (q > 0) y[q] = twmul<false>(y[q], __ldg(twx + nn1 * q));
                    st_stream(static_cast<C *>(a.tmp) + (size_t)(q * m + nn1) * NY + c, y[q]);
                }
            }
        } else {
            C *p = static_cast<C *>(a.tmp) + base;
#pragma unroll
            for (int e = 0; e < E; ++e) st_stream(p + e * TL, x[e]);
        }
    }
    if (a.partials) {
        s0 = block_sum<NT>(s0, red);
        s1 = block_sum<NT>(s1, red);
        if (tid == 0) {
            a.partials[2 * blockIdx.x] = s0;
            a.partials[2 * blockIdx.x + 1] = s1;
        }
    }
}

// ---------------------------------------------------------------------------
// 2D k-space pass: W columns of one x-split block (M = Nx / G rows) per CTA,
// column FFT -> G0/N -> column iFFT
// ---------------------------------------------------------------------------


template <class T, int M, int E, int W>
__global__ void __launch_bounds__(W *(M / E), born_min_blocks(W *(M / E))) k_born_col(BornColArgs a)
{
    using C = cplx_t<T>;
    constexpr int TM = Plan<M, E>::TL;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C *>(smraw);
    const int tid = threadIdx.x;
    const int c = tid % W, t = tid / W;
    const int ny = a.ny;
    const int ntx = ny / W;
    const int qb = blockIdx.x / ntx;  // x-split block: rows qb*M .. qb*M + M - 1, kx = G*k2 + qb
    const int col = (blockIdx.x - qb * ntx) * W + c;
    C *p = static_cast<C *>(a.tmp) + ((size_t)qb * M + t) * ny + col;
    const size_t stride = (size_t)TM * ny;
    const tw_t<C> *tw = static_cast<const tw_t<C> *>(a.tw);
    constexpr ColPad CP = col_pad(sizeof(C), M, W, E);
    const ColLayout<W, CP.sh, CP.p> lay{c};
    const CtaBarrier bar{};

    C x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) x[e] = ld_stream(p + e * stride);
#pragma unroll 1
    for (int q = 0; q < 2; ++q) {
        line_fft<C, M, E, false>(x, sm, lay, bar, t, tw);
        if (q == 1) continue;
        if constexpr (sizeof(T) == 4) {
            const float2 gy = __ldg(a.gy2 + col);
            const float ef = (float)a.eps, inf = (float)a.inv_n;
#pragma unroll
            for (int e = 0; e < E; ++e) x[e] = cconj(born_g0f(x[e], __ldg(a.gx2 + a.g * (t + e * TM) + qb), gy, ef, inf));
        } else {
            const double gy = __ldg(a.gy + col);
#pragma unroll
            for (int e = 0; e < E; ++e) x[e] = cconj(born_g0(x[e], __ldg(a.gx + a.g * (t + e * TM) + qb) - gy, a.eps, a.inv_n));
        }
    }
    C *o = const_cast<C *>(opaque(p));
#pragma unroll
    for (int e = 0; e < E; ++e) st_stream(o + e * stride, cconj(x[e]));
}

// ---------------------------------------------------------------------------
// 1D, one CTA per instance: every update of a Compute on chip, then the
// reflection / transmission sums (ComputeRT, src/ScatteringSolverImpl.cpp:40-55)
// ---------------------------------------------------------------------------


template <class T, int L, int E>
__global__ void __launch_bounds__(L / E) k_born1d(Born1DArgs a)
{
    using C = cplx_t<T>;
    constexpr int TL = Plan<L, E>::TL;
    constexpr int PADS = sizeof(C) == 8 ? 4 : 3;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[32];
    C *sm = reinterpret_cast<C *>(smraw);
    const int t = threadIdx.x;
    const RowLayout<PADS> lay{0};
    const CtaBarrier bar{};
    const tw_t<C> *tw = static_cast<const tw_t<C> *>(a.tw);
    C *dp = static_cast<C *>(a.dpsi) + t;
    const C *p0 = static_cast<const C *>(a.psi0) + t;
    const C *V = static_cast<const C *>(a.V) + t;

    // dpsi stays in its global buffer between updates (a thread reads back only
    // what it wrote itself; the instance is L2-resident), which keeps the
    // registers for the transforms
#pragma unroll 1
    for (int it = 0; it < a.order; ++it) {
        C x[E];
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = born_pre(a.ops, dp[e * TL], __ldg(opaque(p0) + e * TL), __ldg(opaque(V) + e * TL));
#pragma unroll 1
        for (int q = 0; q < 2; ++q) {
            line_fft<C, L, E, false>(x, sm, lay, bar, t, opaque(tw));
            if (q == 1) continue;
#pragma unroll
            for (int e = 0; e < E; ++e)
                x[e] = cconj(born_g0_k(x[e], born_fold(t + e * TL, L), a.en, a.dk2, a.enf, a.dkf, a.ops.eps, a.inv_n));
        }
#pragma unroll
        for (int e = 0; e < E; ++e) dp[e * TL] = born_post(a.ops, cconj(x[e]), dp[e * TL], __ldg(opaque(V) + e * TL));
    }
    double r0 = 0, r1 = 0, t0 = 0, t1 = 0;
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const C d = dp[e * TL];
        const C p = __ldg(p0 + e * TL), v = __ldg(V + e * TL);
        const double vr = v.x;
        const double sr = ((double)p.x + d.x) * vr, si = ((double)p.y + d.y) * vr;
        r0 += sr * p.x - si * p.y;  // s psi0
        r1 += sr * p.y + si * p.x;
        t0 += sr * p.x + si * p.y;  // s conj(psi0)
        t1 += si * p.x - sr * p.y;
    }
    r0 = block_sum<L / E>(r0, red);
    r1 = block_sum<L / E>(r1, red);
    t0 = block_sum<L / E>(t0, red);
    t1 = block_sum<L / E>(t1, red);
    if (t == 0) {
        a.sums[0] = r0;
        a.sums[1] = r1;
        a.sums[2] = t0;
        a.sums[3] = t1;
    }
}

// ---------------------------------------------------------------------------
// 1D four-step: psi[n], n = n1 + N1 n2, as an N2 x N1 row-major array.
// Forward transform: column FFTs (length N2), twiddle exp(-2 pi i n1 k2 / N),
// row FFTs (length N1); frequency k = k2 + N2 k1 at row k2, column k1.
// ---------------------------------------------------------------------------


template <class T, int N2, int E, int W>
__global__ void __launch_bounds__(W *(N2 / E)) k_born_fs_col(BornFsColArgs a)
{
    using C = cplx_t<T>;
    constexpr int TM = Plan<N2, E>::TL;
    constexpr int NT = W * TM;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[32];
    C *sm = reinterpret_cast<C *>(smraw);
    const int tid = threadIdx.x;
    const int c = tid % W, t = tid / W;
    const int col = blockIdx.x * W + c;
    const int n1 = a.n1;
    const tw_t<C> *tw = static_cast<const tw_t<C> *>(a.tw);
    const tw_t<C> *twn = static_cast<const tw_t<C> *>(a.tw_n);
    constexpr ColPad CP = col_pad(sizeof(C), N2, W, E);
    const ColLayout<W, CP.sh, CP.p> lay{c};
    const CtaBarrier bar{};
    const size_t base = (size_t)t * n1 + col;
    const size_t stride = (size_t)TM * n1;
    const C *V = static_cast<const C *>(a.V) + base;
    const C *P0 = static_cast<const C *>(a.psi0) + base;

    C x[E];
    {
        const C *p = static_cast<const C *>(a.in) + base;
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = ld_stream(p + e * stride);
    }
    double r0 = 0, r1 = 0, t0 = 0, t1 = 0;
    if (a.in_k) {
        // iFFT(y conj(w)) = conj(FFT(conj(y) w))
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = twmul<false>(cconj(x[e]), __ldg(twn + base + e * stride));
        line_fft<C, N2, E, false>(x, sm, lay, bar, t, tw);
        C v[E], d[E];
#pragma unroll
        for (int e = 0; e < E; ++e) v[e] = ld_stream(V + e * stride);
        if (a.dold) {
            const C *p = static_cast<const C *>(a.dold) + base;
#pragma unroll
            for (int e = 0; e < E; ++e) d[e] = ld_stream(p + e * stride);
        } else {
#pragma unroll
            for (int e = 0; e < E; ++e) d[e] = cmk<C>(0, 0);
        }
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = born_post(a.ops, cconj(x[e]), d[e], v[e]);
        if (a.dnew) {
            C *p = static_cast<C *>(a.dnew) + base;
#pragma unroll
            for (int e = 0; e < E; ++e) st_stream(p + e * stride, x[e]);
        }
        if (a.partials) {
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const C p = ld_stream(P0 + e * stride);
                const double vr = v[e].x;
                const double sr = ((double)p.x + x[e].x) * vr, si = ((double)p.y + x[e].y) * vr;
                r0 += sr * p.x - si * p.y;
                r1 += sr * p.y + si * p.x;
                t0 += sr * p.x + si * p.y;
                t1 += si * p.x - sr * p.y;
            }
        }
    }
    if (a.out_k) {
#pragma unroll
        for (int e = 0; e < E; ++e)
            x[e] = born_pre(a.ops, x[e], ld_stream(opaque(P0) + e * stride), ld_stream(opaque(V) + e * stride));
        line_fft<C, N2, E, false>(x, sm, lay, bar, t, opaque(tw));
        C *p = static_cast<C *>(a.tmp) + base;
#pragma unroll
        for (int e = 0; e < E; ++e)
            st_stream(p + e * stride, twmul<false>(x[e], __ldg(opaque(twn) + base + e * stride)));
    }
    if (a.partials) {
        r0 = block_sum<NT>(r0, red);
        r1 = block_sum<NT>(r1, red);
        t0 = block_sum<NT>(t0, red);
        t1 = block_sum<NT>(t1, red);
        if (tid == 0) {
            double *o = a.partials + 4 * blockIdx.x;
            o[0] = r0;
            o[1] = r1;
            o[2] = t0;
            o[3] = t1;
        }
    }
}


// B rows of N1 per CTA: row FFT -> G0/N -> row iFFT
template <class T, int N1, int E, int B>
__global__ void __launch_bounds__(B *(N1 / E)) k_born_fs_row(BornFsRowArgs a)
{
    using C = cplx_t<T>;
    constexpr int TL = Plan<N1, E>::TL;
    constexpr int PADS = sizeof(C) == 8 ? 4 : 3;
    constexpr int LINE = padded<N1, PADS>(N1);
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C *>(smraw);
    const int tid = threadIdx.x;
    const int line = tid / TL, t = tid - line * TL;
    const int row = blockIdx.x * B + line;
    const RowLayout<PADS> lay{line * LINE};
    const auto lbar = LineBarrierOf<TL, B>::make(line);
    const tw_t<C> *tw = static_cast<const tw_t<C> *>(a.tw);
    C *p = static_cast<C *>(a.tmp) + (size_t)row * N1 + t;

    C x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) x[e] = ld_stream(p + e * TL);
#pragma unroll 1
    for (int q = 0; q < 2; ++q) {
        line_fft<C, N1, E, false>(x, sm, lay, lbar, t, tw);
        if (q == 1) continue;
#pragma unroll
        for (int e = 0; e < E; ++e)
            x[e] = cconj(born_g0_k(x[e], born_fold(row + a.n2 * (t + e * TL), a.n), a.en, a.dk2, a.enf, a.dkf,
                                   a.eps, a.inv_n));
    }
    C *o = const_cast<C *>(opaque(p));
#pragma unroll
    for (int e = 0; e < E; ++e) st_stream(o + e * TL, cconj(x[e]));
}

// ---------------------------------------------------------------------------
// 2D scattering amplitudes r(theta) = sum (psi0 + dpsi) Re V exp(-i (kx x + ky y))
// for a batch of directions (ComputeXSection, src/ScatteringSolverImpl.cpp:218-250),
// the phase split as ax[a][ix] ay[a][iy].
// ---------------------------------------------------------------------------


constexpr int kXsecRows = 4;      // rows per CTA
constexpr int kXsecThreads = 256;
constexpr int kXsecChunk = 8;     // directions per sweep

template <class T>
__global__ void __launch_bounds__(kXsecThreads) k_born_xsec(BornXsecArgs a)
{
    using C = cplx_t<T>;
    __shared__ double red[32];
    const int tid = threadIdx.x;
    const C *dpsi = static_cast<const C *>(a.dpsi);
    const C *V = static_cast<const C *>(a.V);
    const C *ex = static_cast<const C *>(a.ex);
    const C *ey = static_cast<const C *>(a.ey);
    const int r0 = blockIdx.x * kXsecRows;
#pragma unroll 1
    for (int a0 = 0; a0 < a.na; a0 += kXsecChunk) {
        double acc[kXsecChunk][2];
#pragma unroll
        for (int k = 0; k < kXsecChunk; ++k) acc[k][0] = acc[k][1] = 0;
#pragma unroll 1
        for (int r = r0; r < r0 + kXsecRows && r < a.nx; ++r) {
            double row[kXsecChunk][2];
#pragma unroll
            for (int k = 0; k < kXsecChunk; ++k) row[k][0] = row[k][1] = 0;
            const C exr = ex[r];
#pragma unroll 1
            for (int j = tid; j < a.ny; j += kXsecThreads) {
                const size_t i = (size_t)r * a.ny + j;
                const C p = cmul(exr, ey[j]), d = dpsi[i];
                const double vr = V[i].x;
                const double sr = ((double)p.x + d.x) * vr, si = ((double)p.y + d.y) * vr;
#pragma unroll
                for (int k = 0; k < kXsecChunk; ++k) {
                    if (a0 + k < a.na) {
                        const double2 w = a.ay[(size_t)(a0 + k) * a.ny + j];
                        row[k][0] += sr * w.x - si * w.y;
                        row[k][1] += sr * w.y + si * w.x;
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < kXsecChunk; ++k) {
                if (a0 + k < a.na) {
                    const double2 w = a.ax[(size_t)(a0 + k) * a.nx + r];
                    acc[k][0] += row[k][0] * w.x - row[k][1] * w.y;
                    acc[k][1] += row[k][0] * w.y + row[k][1] * w.x;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < kXsecChunk; ++k) {
            const double s0 = block_sum<kXsecThreads>(acc[k][0], red);
            const double s1 = block_sum<kXsecThreads>(acc[k][1], red);
            if (tid == 0 && a0 + k < a.na) {
                a.partials[((size_t)blockIdx.x * a.na + a0 + k) * 2] = s0;
                a.partials[((size_t)blockIdx.x * a.na + a0 + k) * 2 + 1] = s1;
            }
        }
    }
}

}  // namespace qsg
