// qsg_kernels.cuh -- kernel templates of the split-operator step.
//
// Reference path (lhprojects/QuSim): QuUpdatePsi (src/SplittingUtils.h:14-64)
// drives ExpV / ExpT of SplittingMethod1D (src/SplittingMethod1D.cpp:40-89)
// and SplittingMethod2D (src/SplittingMethod2D.cpp:81-121), each of which is a
// separate Device op (src/DeviceTemplate.h:1458-1579) plus FFT calls.  Here
// one kernel owns several of those ops at once:
//
//   k_evolve1d_resident  whole O2/O4 step sequence of a 1D instance that fits
//                        in one CTA's shared memory, for any number of steps,
//                        psi kept in registers/shared memory between steps.
//   k_row_pass           2D real-space pass: [inverse x-split stage, row iFFT]
//                        -> V phase(s) -> [row FFT, forward x-split stage].
//   k_col_pass           2D k-space pass: column FFT -> kinetic phase -> column
//                        iFFT, over one x-split block.
//
// The x-split: a column transform of length Nx = G*M is a radix-G
// decimation-in-frequency stage across the G rows n1 + j*M (done in the row
// pass, with twiddles exp(-2 pi i n1 q / Nx)) followed by M-point transforms
// over each block q of M consecutive rows (the column pass).  Output
// frequency of block q, position k2 is kx = G*k2 + q.  The inverse runs the
// same stages backwards.
#pragma once
#include <type_traits>
#include "qsg_fft.cuh"

namespace qsg {

// ---------------------------------------------------------------------------
// shared helpers
// ---------------------------------------------------------------------------

template <class C> struct PhaseOps;
// complex128: tables hold the factor itself (the reference's own exp(f V)),
// multiplied in as a plain complex product with explicit roundings (one product
// rounded, one fused): the same bits in every pass that applies a factor, once
// or twice in a row, so a step split across calls equals the step in one call
// (left to the compiler, the contraction of a.x m.x - a.y m.y can differ
// between two inlined copies).
template <> struct PhaseOps<double2> {
    static __device__ __forceinline__ double2 apply(double2 a, double2 m)
    {
        return double2{__fma_rn(a.x, m.x, -__dmul_rn(a.y, m.y)), __fma_rn(a.x, m.y, __dmul_rn(a.y, m.x))};
    }
    static __device__ __forceinline__ double2 increment(double2 a, double2, int) { return a; }  // unused
};
// complex64: tables hold factor - 1 (see cmul1p).
template <> struct PhaseOps<float2> {
    static __device__ __forceinline__ float2 apply(float2 a, float2 m) { return cmul1p(a, m); }
    // the increment a * (f - 1) of a factor f = 1 + m, or of f^2 (twice):
    // (1 + m)^2 - 1 = m (2 + m)
    static __device__ __forceinline__ float2 increment(float2 a, float2 m, int twice)
    {
        if (twice) m = cmulw_f<false>(m, cmk<float2>(m.x + 2.f, m.y));
        return cmulw_f<false>(a, m);
    }
};

template <class C> __device__ __forceinline__ C ld_c(const C *p) { return __ldg(p); }
// Streaming loads of psi and of the V tables bypass L1: each element is read
// once per pass, and letting them allocate evicts the twiddle tables that
// every butterfly stage re-reads from L1.
__device__ __forceinline__ float2 ld_stream(const float2 *p)
{
    float2 r;
    asm volatile("ld.global.nc.L1::no_allocate.v2.f32 {%0, %1}, [%2];" : "=f"(r.x), "=f"(r.y) : "l"(p));
    return r;
}
__device__ __forceinline__ double2 ld_stream(const double2 *p)
{
    double2 r;
    asm volatile("ld.global.nc.L1::no_allocate.v2.f64 {%0, %1}, [%2];" : "=d"(r.x), "=d"(r.y) : "l"(p));
    return r;
}
template <class C> __device__ __forceinline__ void st_stream(C *p, C v) { __stcs(p, v); }
__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }
// bulk L2 prefetch of `bytes` (a multiple of 16) from a 16-byte aligned address
__device__ __forceinline__ void prefetch_l2_bulk(const void *p, unsigned bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}
template <class C> __device__ __forceinline__ C cconj(C a) { return cmk<C>(a.x, -a.y); }

// Every inverse transform here is computed as conj(FFT(conj(x))), which is
// bit-identical to running the transform with conjugated twiddles and
// constants (negation is exact), and every kernel runs its transforms in a
// non-unrolled loop over one forward-transform body: two inlined transform
// bodies roughly triple the register demand (the scheduler interleaves them).
// The conjugations fold into the neighbouring phase multiplies.

template <class C> __device__ __forceinline__ double abs2d(C a)
{
    return double(a.x) * double(a.x) + double(a.y) * double(a.y);
}

// block-wide sum of a double; every thread gets the result
template <int NT> __device__ __forceinline__ double block_sum(double v, double *red)
{
    // a CTA narrower than a warp shuffles only among its own lanes
    constexpr int O0 = NT < 32 ? NT / 2 : 16;
    constexpr unsigned MASK = NT < 32 ? (1u << NT) - 1u : 0xffffffffu;
#pragma unroll
    for (int o = O0; o > 0; o >>= 1) v += __shfl_xor_sync(MASK, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double s = 0;
    if (NT >= 32 && threadIdx.x < 32) {
        s = threadIdx.x < (NT + 31) / 32 ? red[threadIdx.x] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) red[0] = s;
    }
    __syncthreads();
    s = red[0];
    __syncthreads();
    return s;
}

// G-point DFT on registers (G = 1, 2, 4)
template <int G, bool INV, class C> __device__ __forceinline__ void dftg(C (&v)[G])
{
    if constexpr (G == 2) dft2<INV>(v[0], v[1]);
    if constexpr (G == 4) dft4<INV>(v[0], v[1], v[2], v[3]);
}

// ---------------------------------------------------------------------------
// 1D resident evolution
// ---------------------------------------------------------------------------

struct FsInst;
struct Evolve1DBatchArgs;

// NI instances per CTA (instance blockIdx.x*NI + line); all instances of one
// launch share N and the order.  V tables vtab[0..1], kinetic tables ktab[0..1] (natural layout,
// 1/N folded in for complex128, factor - 1 for complex64).
template <class T, int L, int E, int NI>
__global__ void __launch_bounds__(NI *(L / E)) k_evolve1d_resident(Evolve1DBatchArgs a);

// ---------------------------------------------------------------------------
// 2D passes
// ---------------------------------------------------------------------------

struct RowPassArgs {
    const void *in;
    void *out;
    const void *vtab;       // V phase table (Nx*Ny), or null (plain transform)
    int vtwice;             // apply it twice (the two ExpV calls at a step boundary)
    int vdiff;              // complex64: multiply by factor - 1 (the increment (V - 1) psi)
    int plain;              // complex64: tw_row / tw_nx are float2 tables (plain twiddles)
    const void *tw_row;     // stage-major twiddles for (Ny, E)
    const void *tw_nx;      // full circle exp(-2 pi i m / Nx), m < Nx (x-split twiddles)
    double *partials;       // per-unit sum |psi|^2 (natural-output passes), or null
    int nx, m;              // Nx and M = Nx / G
    int in_split, out_split;
    int units;              // row-group units (M / B); CTAs loop over them
};

// in_split:  input is in split-k space (inverse x-split stage + row iFFT first);
//            otherwise natural real-space rows.
// out_split: output goes back to split-k space (row FFT + forward x-split
//            stage); otherwise natural real-space rows (+ norm partials).
// (Runtime flags: one instantiation serves the three pass kinds of a step.)
// A unit is B row groups; group b has the G rows n1 + j*M, j < G,
// n1 = u*B + b, i.e. NL = B*G lines of NY.  The NT threads work on NL/RS lines
// at a time and go over the unit's lines in RS rounds.  CTAs are persistent
// (CTA i takes units i, i + gridDim.x, ...).  When the split-k input of a unit
// fits in 32 registers per thread, it is loaded while the previous unit's
// forward x-split stage runs, so its HBM latency overlaps that stage.
// The body, for a compile-time in_split (see k_row_pass).
// the twiddle table type of a pass: PL (complex64 only) selects plain float2 tables
template <class C, bool PL> using pass_tw_t = std::conditional_t<PL, float2, tw_t<C>>;

template <class T, int NY, int E, int G, int B, int RS, bool IN, bool PL>
__device__ __forceinline__ void row_pass_units(const RowPassArgs &a, unsigned char *smraw, double *red)
{
    using C = cplx_t<T>;
    using TW = pass_tw_t<C, PL>;
    static_assert(!PL || sizeof(C) == 8, "plain twiddles are a complex64 form");
    using P = Plan<NY, E>;
    constexpr int TL = P::TL;
    constexpr int NL = B * G;
    constexpr int NT = NL * TL / RS;
    constexpr int LPR = NL / RS;  // lines per round
    static_assert(NL % RS == 0, "");
    constexpr int PADS = sizeof(C) == 8 ? 4 : 3;
    constexpr int LINE = padded<NY, PADS>(NY);
    C *sm = reinterpret_cast<C *>(smraw);

    constexpr bool in_split = IN;
    const bool out_split = a.out_split != 0;
    const int tid = threadIdx.x;
    const int grp = tid / TL;  // line slot within a round
    const int t = tid - grp * TL;
    const C *in = static_cast<const C *>(a.in);
    C *out = static_cast<C *>(a.out);
    const TW *tw = static_cast<const TW *>(a.tw_row);
    const TW *twx = static_cast<const TW *>(a.tw_nx);
    const C *vt = static_cast<const C *>(a.vtab);
    const CtaBarrier cbar{};
    // lines of whole warps synchronise among themselves; otherwise CTA-wide
    const auto lbar = LineBarrierOf<TL, LPR>::make(grp);
    constexpr bool via_smem_in = in_split && G > 1;
    const bool via_smem_out = out_split && G > 1;
    constexpr int XV = B * NY / NT;                       // x-split columns per thread
    // split-k input held in registers (not with 1024 threads: 64 registers per thread)
    constexpr bool XPF = via_smem_in && XV * G <= 32 && NT <= 512;
    C pf[XPF ? XV : 1][G];
    // issue the loads of unit uu's split-k input (consumed by the next x-split
    // stage).  Every path defines pf (zeros when !live), so the consumed values
    // are dead during the transforms.
    auto xs_load = [&](int uu, bool live) {
        if constexpr (XPF) {
#pragma unroll
            for (int v = 0; v < XV; ++v) {
                const int gc = tid + v * NT;
                const int bb = gc / NY, c = gc - bb * NY;
                const int nn1 = uu * B + bb;
#pragma unroll
                for (int q = 0; q < G; ++q)
                    pf[v][q] = live ? ld_stream(in + (size_t)(q * a.m + nn1) * NY + c) : cmk<C>(0, 0);
            }
        }
    };
    if constexpr (XPF) xs_load(blockIdx.x, true);

#pragma unroll 1
    for (int u = blockIdx.x; u < a.units; u += gridDim.x) {
    const int unext = u + gridDim.x;
    if (u != (int)blockIdx.x) cbar();  // the previous unit's readers of sm are done
    if (vt && tid < NL) {
        // each line's potential row is read right after its inverse transform:
        // start pulling the unit's rows into L2 now, one bulk prefetch per row
        // (4096^2 complex64: 129.0 -> 128.0 us per launch)
        const int b = tid / G, j = tid - b * G;
        prefetch_l2_bulk(vt + (size_t)(u * B + b + j * a.m) * NY, NY * (unsigned)sizeof(C));
    }

    if constexpr (XPF) {
        {
            // inverse x-split stage from the registers loaded in advance
#pragma unroll
            for (int v = 0; v < XV; ++v) {
                const int gc = tid + v * NT;
                const int bb = gc / NY, c = gc - bb * NY;
                const int nn1 = u * B + bb;
                C y[G];
#pragma unroll
                for (int q = 0; q < G; ++q) y[q] = q > 0 ? twmul<true>(pf[v][q], __ldg(twx + nn1 * q)) : pf[v][q];
                dftg<G, true>(y);
#pragma unroll
                for (int q = 0; q < G; ++q) sm[(bb * G + q) * LINE + c + (c >> PADS)] = y[q];
            }
        }
        cbar();
    } else if constexpr (via_smem_in) {
        {
            // inverse x-split stage over every column of every group of this unit
#pragma unroll 2
            for (int v = 0; v < B * NY / NT; ++v) {
                const int gc = tid + v * NT;
                const int bb = gc / NY, c = gc - bb * NY;
                const int nn1 = u * B + bb;
                C y[G];
#pragma unroll
                for (int q = 0; q < G; ++q) {
                    y[q] = ld_stream(in + (size_t)(q * a.m + nn1) * NY + c);
                    if (q > 0) y[q] = twmul<true>(y[q], __ldg(twx + nn1 * q));
                }
                dftg<G, true>(y);
#pragma unroll
                for (int q = 0; q < G; ++q) sm[(bb * G + q) * LINE + c + (c >> PADS)] = y[q];
            }
        }
        cbar();
    }

    double nsum = 0;
#pragma unroll 1
    for (int r = 0; r < RS; ++r) {
        const int line = r * LPR + grp;
        const int b = line / G, j = line - b * G;
        const int row = u * B + b + j * a.m;
        const RowLayout<PADS> lay{line * LINE};
        C x[E];
        if (via_smem_in) {
#pragma unroll
            for (int e = 0; e < E; ++e) x[e] = sm[lay(t + e * TL)];
        } else {
            const C *ir = in + (size_t)row * NY + t;
#pragma unroll
            for (int e = 0; e < E; ++e) x[e] = ld_stream(ir + e * TL);
        }
        // [row iFFT] -> V -> [row FFT], the iFFT as conj(FFT(conj(x)))
        const int npass = (in_split ? 1 : 0) + (out_split ? 1 : 0);
        const int vpos = in_split ? 1 : 0;
        if (in_split) {
#pragma unroll
            for (int e = 0; e < E; ++e) x[e] = cconj(x[e]);
        }
#pragma unroll 1
        for (int p = 0; p <= npass; ++p) {
            if (p == vpos) {
                if (in_split) {
#pragma unroll
                    for (int e = 0; e < E; ++e) x[e] = cconj(x[e]);
                }
                if (vt) {
                    const C *vr = opaque(vt) + (size_t)row * NY + t;
                    // all loads first, then the multiplies: interleaved, the
                    // schedule exposed the load latency (152 vs 168 us at 4096^2);
                    // with 1024 threads in chunks of 8 (registers)
                    constexpr int VC = NT > 512 && E > 8 ? 8 : E;
#pragma unroll
                    for (int e0 = 0; e0 < E; e0 += VC) {
                        C mv[VC];
#pragma unroll
                        for (int e = 0; e < VC; ++e) mv[e] = ld_stream(vr + (e0 + e) * TL);
                        if (sizeof(C) == 8 && a.vdiff) {
#pragma unroll
                            for (int e = 0; e < VC; ++e) x[e0 + e] = PhaseOps<C>::increment(x[e0 + e], mv[e], a.vtwice);
                        } else if (a.vtwice) {
#pragma unroll
                            for (int e = 0; e < VC; ++e)
                                x[e0 + e] = PhaseOps<C>::apply(PhaseOps<C>::apply(x[e0 + e], mv[e]), mv[e]);
                        } else {
#pragma unroll
                            for (int e = 0; e < VC; ++e) x[e0 + e] = PhaseOps<C>::apply(x[e0 + e], mv[e]);
                        }
                    }
                }
            }
            if (p < npass) line_fft<C, NY, E, false>(x, sm, lay, lbar, t, tw);
        }
        if (!out_split) {
            C *orow = const_cast<C *>(opaque(out)) + (size_t)row * NY + t;
#pragma unroll
            for (int e = 0; e < E; ++e) {
                st_stream(orow + e * TL, x[e]);
                nsum += abs2d(x[e]);
            }
        } else if (via_smem_out) {
            lbar();  // this line's readers of the last exchange are done
#pragma unroll
            for (int e = 0; e < E; ++e) sm[lay(t + e * TL)] = x[e];
        } else {
            C *orow = const_cast<C *>(opaque(out)) + (size_t)row * NY + t;
#pragma unroll
            for (int e = 0; e < E; ++e) st_stream(orow + e * TL, x[e]);
        }
    }

    // the next unit's split-k input is in flight while this unit's results go out
    if (via_smem_out) cbar();
    if constexpr (XPF) xs_load(unext, unext < a.units);
    if constexpr (via_smem_in && !XPF && NT > 512) {
        // 1024 threads hold no next-unit input in registers: its rows go to L2 instead
        if (tid < G && unext < a.units) {
            for (int bb = 0; bb < B; ++bb)
                prefetch_l2_bulk(in + (size_t)(tid * a.m + unext * B + bb) * NY, NY * (unsigned)sizeof(C));
        }
    }
    if (via_smem_out) {
        if constexpr (G > 1) {
#pragma unroll 2
            for (int v = 0; v < B * NY / NT; ++v) {
                const int gc = tid + v * NT;
                const int bb = gc / NY, c = gc - bb * NY;
                const int nn1 = u * B + bb;
                C y[G];
#pragma unroll
                for (int q = 0; q < G; ++q) y[q] = sm[(bb * G + q) * LINE + c + (c >> PADS)];
                dftg<G, false>(y);
#pragma unroll
                for (int q = 0; q < G; ++q) {
                    if (q > 0) y[q] = twmul<false>(y[q], __ldg(twx + nn1 * q));
                    st_stream(out + (size_t)(q * a.m + nn1) * NY + c, y[q]);
                }
            }
        }
    }
    if (!out_split && a.partials) {
        nsum = block_sum<NT>(nsum, red);
        if (tid == 0) a.partials[u] = nsum;
    }
    }  // units
}

// One kernel serves the three pass kinds of a step (runtime flags); the body
// is specialised on in_split so that the registers holding the next unit's
// input exist only where that input is split-k.
template <class T, int NY, int E, int G, int B, int RS, bool PL = false>
__global__ void __launch_bounds__(B *G *(NY / E) / RS) k_row_pass(RowPassArgs a)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[32];
    if (a.in_split)
        row_pass_units<T, NY, E, G, B, RS, true, PL>(a, smraw, red);
    else
        row_pass_units<T, NY, E, G, B, RS, false, PL>(a, smraw, red);
}

struct ColPassArgs {
    void *psi;              // in/out, Nx*Ny in split-k layout (momentum form: the state)
    void *work;             // momentum form (complex64): the potential increment in, the next
                            // step's split-k input out; null in the direct form
    int first;              // momentum form: no stored state yet (the input is the state)
    int invonly;            // momentum form: only the column iFFT of the stored state, to work
    int *err;               // counter a pass whose bounded waits ran out adds 1 to (TMA pass), or null
    int no_copies;          // TMA pass, failure-path test only: issue no copies, so the first wait runs out
    int plain;              // complex64: tw_col is a float2 table (plain twiddles)
    const void *kx;         // complex64: x kinetic factor - 1, Nx entries
    const void *ky;         // complex64: y kinetic factor - 1, Ny entries
    const void *k2d;        // complex128: full table Nx*Ny with 1/(Nx Ny) folded in
    const void *tw_col;     // stage-major twiddles for (M, E)
    int nx, ny, g;
    float inv_n;            // 1/(Nx Ny) (complex64 path)
    int tiles;              // (Ny / W) * G tiles; CTAs loop over them
    double *partials;       // or null: per CTA, sum |psi|^2 of the output (split-k scale)
};

// A tile is block q, columns [xt*W, +W), tile index u = q * (Ny/W) + xt;
// CTA u handles tile u.
// Radix-32 variants are held to 128 registers so that 512 threads (two CTAs
// of 256) share an SM.  (Four CTAs of 128 threads, W = 4, measured slower at
// 4096^2: 168 against 119 us.)
template <class T, int M, int E, int W, bool PL = false>
__global__ void __launch_bounds__(W *(M / E), E == 32 ? 512 / (W * (M / E)) : 1) k_col_pass(ColPassArgs a)
{
    using C = cplx_t<T>;
    using TW = pass_tw_t<C, PL>;
    using P = Plan<M, E>;
    constexpr int TM = P::TL;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[32];
    C *sm = reinterpret_cast<C *>(smraw);
    const int tid = threadIdx.x;
    const int c = tid % W, t = tid / W;
    const int ny = a.ny;
    const int ntx = ny / W;
    C *psi = static_cast<C *>(a.psi);
    const TW *tw = static_cast<const TW *>(a.tw_col);
    constexpr ColPad CP = col_pad(sizeof(C), M, W, E);
    const ColLayout<W, CP.sh, CP.p> lay{c};
    const CtaBarrier bar{};
    const int stride = TM * ny;  // between a thread's elements

    auto tile = [&](int u) {
    const int q = u / ntx;
    const int col = (u - q * ntx) * W + c;
    const size_t base = ((size_t)q * M + t) * ny + col;

    // momentum form: the input is the potential increment (or, first, the
    // state), the stored state is read, updated and written at the transform's
    // output positions, and the output is the next step's split-k input
    C *work = static_cast<C *>(a.work);
    const bool mom = sizeof(C) == 8 && work != nullptr;
    float nf = 0;  // momentum form: sum |state|^2 of this thread

    // inverse only: the stored state, conjugated for the conj(FFT(conj)) iFFT
    const bool inv_only = mom && a.invonly;
    C x[E];
    {
        const C *p = (mom && !inv_only ? work : psi) + base;
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = ld_stream(p + (size_t)e * stride);
        if (inv_only) {
#pragma unroll
            for (int e = 0; e < E; ++e) x[e] = cconj(x[e]);
        }
    }
    if (mom && !a.first && !inv_only) {
        // the stored state is read after the forward transform: pull it into
        // L2 now so that those reads do not wait on HBM (no registers held).
        // (Prefetching the tile one wave ahead as well was slower: 136 against
        // 124 us at 4096^2.)
        const C *p = psi + base;
#pragma unroll
        for (int e = 0; e < E; ++e) prefetch_l2(p + (size_t)e * stride);
    }

    // FFT -> K -> iFFT, the iFFT as conj(FFT(conj(x)))
#pragma unroll 1
    for (int p = inv_only ? 1 : 0; p < 2; ++p) {
        line_fft<C, M, E, false>(x, sm, lay, bar, t, tw);
        if (p == 1) continue;  // (a break here makes the compiler duplicate the body)
        if constexpr (sizeof(C) == 8) {
            const C *kx = opaque(static_cast<const C *>(a.kx));
            const C ky = ld_c(static_cast<const C *>(a.ky) + col);
            if (mom) {
                // state += increment / (Nx Ny); state *= K; the K factor is
                // applied to the state itself, never to a transform of it
                C *ps = const_cast<C *>(opaque(psi)) + base;
                const bool add = !a.first;
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    const int kxi = a.g * (t + e * TM) + q;
                    C v = cscale(x[e], a.inv_n);
                    if (add) v = cadd(ld_stream(ps + (size_t)e * stride), v);
                    v = cmul1p(v, ld_c(kx + kxi));
                    v = cmul1p(v, ky);
                    st_stream(ps + (size_t)e * stride, v);
                    nf = fmaf(v.x, v.x, fmaf(v.y, v.y, nf));
                    x[e] = cconj(v);
                }
            } else {
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    const int kxi = a.g * (t + e * TM) + q;
                    C v = cscale(x[e], a.inv_n);
                    v = cmul1p(v, ld_c(kx + kxi));
                    x[e] = cconj(cmul1p(v, ky));
                }
            }
        } else {
            const C *k2 = static_cast<const C *>(a.k2d) + col;
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const int kxi = a.g * (t + e * TM) + q;
                x[e] = cconj(cmul(x[e], ld_stream(k2 + (size_t)kxi * ny)));
            }
        }
    }
#pragma unroll
    for (int e = 0; e < E; ++e) x[e] = cconj(x[e]);

    {
        // recomputed rather than kept live across both transforms
        C *p = const_cast<C *>(opaque(mom ? work : psi)) + base;
#pragma unroll
        for (int e = 0; e < E; ++e) st_stream(p + (size_t)e * stride, x[e]);
    }
    if (a.partials) {
        // the norm of the step's state without a pass of its own: in split-k
        // space sum |psi|^2 is 1 / (G Ny) of the real-space one (the row FFT and
        // the radix-G stage are unnormalised, the column pass carries 1/(Nx Ny));
        // the momentum-form state holds F psi / (Nx Ny), 1 / (Nx Ny) of it.
        // complex64 sums a thread's elements in FP32 (FP64 runs at 1/64 rate:
        // per-element FP64 doubled this pass), the CTA sum in FP64.
        double s;
        if constexpr (sizeof(C) == 8) {
            float f = nf;
            if (!mom) {
#pragma unroll
                for (int e = 0; e < E; ++e) f = fmaf(x[e].x, x[e].x, fmaf(x[e].y, x[e].y, f));
            }
            s = f;
        } else {
            s = 0;
#pragma unroll
            for (int e = 0; e < E; ++e) s += abs2d(x[e]);
        }
        s = block_sum<W *(M / E)>(s, red);
        if (tid == 0) a.partials[blockIdx.x] = s;
    }
    };
    // one tile per CTA (persistent CTAs measured slower here)
    tile(blockIdx.x);
}

// ---------------------------------------------------------------------------
// kinetic energy: forward transform + reductions
// ---------------------------------------------------------------------------

// 1D: sums[0] = sum |X_i|^2 fold(i)^2 * dtk, sums[1] = sum |X_i|^2
// (SplittingMethod1D::CalKinEn, src/SplittingMethod1D.cpp:93-107)
template <class T, int L, int E>
__global__ void __launch_bounds__(L / E) k_kinetic1d(const void *psi_, const void *tw_, double dtk,
                                                     double *sums)
{
    using C = cplx_t<T>;
    constexpr int TL = Plan<L, E>::TL;
    constexpr int PADS = sizeof(C) == 8 ? 4 : 3;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C *>(smraw);
    __shared__ double red[32];
    const int t = threadIdx.x;
    const C *psi = static_cast<const C *>(psi_);
    C x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) x[e] = psi[t + e * TL];
    line_fft<C, L, E, false>(x, sm, RowLayout<PADS>{0}, CtaBarrier{}, t, static_cast<const tw_t<C> *>(tw_));
    double k = 0, nn = 0;
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int i = t + e * TL;
        const double f = double(i > L / 2 ? L - i : i);
        const double a2 = abs2d(x[e]);
        k += a2 * (f * f) * dtk;
        nn += a2;
    }
    k = block_sum<L / E>(k, red);
    nn = block_sum<L / E>(nn, red);
    if (t == 0) {
        sums[0] = k;
        sums[1] = nn;
    }
}

// 2D column transform of one split block + kinetic reductions; partials[2*cta]
// = sum |X|^2 (fold(kx)^2 DTx + fold(ky)^2 DTy), partials[2*cta+1] = sum |X|^2
// (SplittingMethod2D::CalKinEn, src/SplittingMethod2D.cpp:123-138)
template <class T, int M, int E, int W>
__global__ void __launch_bounds__(W *(M / E)) k_col_kinetic(ColPassArgs a, double dtx, double dty,
                                                            double *partials)
{
    using C = cplx_t<T>;
    constexpr int TM = Plan<M, E>::TL;
    constexpr int NT = W * TM;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C *>(smraw);
    __shared__ double red[32];
    const int tid = threadIdx.x;
    const int c = tid % W, t = tid / W;
    const int q = blockIdx.y;
    const int col = blockIdx.x * W + c;
    const int ny = a.ny, nx = a.nx;
    const C *psi = static_cast<const C *>(a.psi);
    const size_t base = (size_t)q * M * ny + col;
    C x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) x[e] = psi[base + (size_t)(t + e * TM) * ny];
    constexpr ColPad CP = col_pad(sizeof(C), M, W);
    line_fft<C, M, E, false>(x, sm, ColLayout<W, CP.sh, CP.p>{c}, CtaBarrier{}, t,
                             static_cast<const tw_t<C> *>(a.tw_col));
    const double fy = double(col > ny / 2 ? ny - col : col);
    double k = 0, nn = 0;
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int kxi = a.g * (t + e * TM) + q;
        const double fx = double(kxi > nx / 2 ? nx - kxi : kxi);
        const double a2 = abs2d(x[e]);
        k += a2 * ((fx * fx) * dtx + (fy * fy) * dty);
        nn += a2;
    }
    k = block_sum<NT>(k, red);
    nn = block_sum<NT>(nn, red);
    if (tid == 0) {
        const int cta = blockIdx.y * gridDim.x + blockIdx.x;
        partials[2 * cta] = k;
        partials[2 * cta + 1] = nn;
    }
}

// ---------------------------------------------------------------------------
// 1D four-step passes (N = N1 * N2 too large for one CTA)
//
// psi[n], n = n1 + N1*n2, is viewed as an N2 x N1 row-major array (row n2,
// column n1).  Forward transform: column FFTs (length N2) -> twiddle
// exp(-2 pi i n1 k2 / N) -> row FFTs (length N1); frequency k = k2 + N2*k1
// sits at row k2, column k1.  A step is then
//   column pass (real space): [conj twiddle, column iFFT] -> V -> [column FFT, twiddle]
//   row pass    (k space):    row FFT -> K(k)/N -> row iFFT
// so an O2 step costs two HBM round trips, an O4 step six (as in 2D).
// Instances of one size are batched: blockIdx.y selects the instance.
// ---------------------------------------------------------------------------

struct FsInst {
    void *psi;
    const void *vtab[2];    // V phase tables, natural layout
    const void *ktab[2];    // kinetic tables in row layout: entry k2*N1 + k1 for k = k2 + N2*k1
    double *partials;       // per-CTA norm partials of natural-output passes (or null)
};

struct FsColArgs {
    const FsInst *inst;
    const void *tw_col;     // stage twiddles for (N2, E)
    const void *tw_n;       // exp(-2 pi i r c / N) at r * n1 + c (row r < n2, column c < n1)
    int n1;
    int vsel, vtwice;       // V table index; apply it twice
    int in_k, out_k;        // input in k layout / output to k layout
    const void *maps;       // tensor-copy pass: 3 tensor maps per instance (state, V 0, V 1), or null
    int tiles;              // tensor-copy pass: column blocks x instances
    int *err;               // tensor-copy pass: counter it adds 1 to when a bounded wait ran out
    int wall;               // the state is a wall's 2n odd extension: sites 0 and n (rows 0 and
                            // n2 / 2 of column 0) are zeroed before the forward transform, as the
                            // reference's wall KinEn discards them (src/SplittingMethod1D.cpp:
                            // 112-114); set by KinEn's transform only
};

// three 256-thread CTAs per SM (registers capped at 85) for the strided
// column pass: it waits on its scattered loads more than it issues
template <class T, int N2, int E, int W>
__global__ void __launch_bounds__(W *(N2 / E), (W * (N2 / E) <= 256 && sizeof(T) == 4) ? 3 : 1) k_fs_col(FsColArgs a)
{
    using C = cplx_t<T>;
    constexpr int TM = Plan<N2, E>::TL;
    constexpr int NT = W * TM;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C *>(smraw);
    __shared__ double red[32];
    const FsInst in = a.inst[blockIdx.y];
    const bool in_k = a.in_k != 0, out_k = a.out_k != 0;
    const int tid = threadIdx.x;
    const int c = tid % W, t = tid / W;
    const int col = blockIdx.x * W + c;
    const int n1 = a.n1;
    C *psi = static_cast<C *>(in.psi);
    const tw_t<C> *tw = static_cast<const tw_t<C> *>(a.tw_col);
    const tw_t<C> *twn = static_cast<const tw_t<C> *>(a.tw_n);
    constexpr ColPad CP = col_pad(sizeof(C), N2, W);
    const ColLayout<W, CP.sh, CP.p> lay{c};
    const CtaBarrier bar{};
    const size_t base = (size_t)t * n1 + col;
    const size_t stride = (size_t)TM * n1;

    C x[E];
    {
        const C *p = psi + base;
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = ld_stream(p + e * stride);
    }
    if (in_k) {
        // iFFT(y * conj(w)) = conj(FFT(conj(y) * w))
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = twmul<false>(cconj(x[e]), __ldg(twn + base + e * stride));
    }
    const int npass = (in_k ? 1 : 0) + (out_k ? 1 : 0);
    const int vpos = in_k ? 1 : 0;
#pragma unroll 1
    for (int p = 0; p <= npass; ++p) {
        if (p == vpos) {
            if (in_k) {
#pragma unroll
                for (int e = 0; e < E; ++e) x[e] = cconj(x[e]);
            }
            const C *vt = static_cast<const C *>(in.vtab[a.vsel]);
            if (vt) {
                const C *vr = opaque(vt) + base;
                C mv[E];
#pragma unroll
                for (int e = 0; e < E; ++e) mv[e] = ld_stream(vr + e * stride);
                if (a.vtwice) {
#pragma unroll
                    for (int e = 0; e < E; ++e) x[e] = PhaseOps<C>::apply(PhaseOps<C>::apply(x[e], mv[e]), mv[e]);
                } else {
#pragma unroll
                    for (int e = 0; e < E; ++e) x[e] = PhaseOps<C>::apply(x[e], mv[e]);
                }
            }
            // row t + e * TM of column col: site 0 is (t, e) = (0, 0), site n (row n2 / 2) is (0, E / 2)
            if (a.wall && out_k && col == 0 && t == 0) {
                x[0] = cmk<C>(0, 0);
                x[E / 2] = cmk<C>(0, 0);
            }
        }
        if (p < npass) line_fft<C, N2, E, false>(x, sm, lay, bar, t, tw);
    }
    double nsum = 0;
    if (out_k) {
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = twmul<false>(x[e], __ldg(opaque(twn) + base + e * stride));
    } else {
#pragma unroll
        for (int e = 0; e < E; ++e) nsum += abs2d(x[e]);
    }
    {
        C *p = const_cast<C *>(opaque(psi)) + base;
#pragma unroll
        for (int e = 0; e < E; ++e) st_stream(p + e * stride, x[e]);
    }
    if (!out_k && in.partials) {
        nsum = block_sum<NT>(nsum, red);
        if (tid == 0) in.partials[blockIdx.x] = nsum;
    }
}

struct FsRowArgs {
    const FsInst *inst;
    const void *tw_row;     // stage twiddles for (N1, E)
    int ksel;
    float inv_n;            // 1/N (complex64 path; complex128 tables carry it)
    int plain;              // the table holds plain complex factors (any modulus, scale included):
                            // a plain product, no 1/N (Bluestein's convolution kernels)
};

// B rows of N1 per CTA (B * N1/E threads)
template <class T, int N1, int E, int B>
__global__ void __launch_bounds__(B *(N1 / E)) k_fs_row(FsRowArgs a)
{
    using C = cplx_t<T>;
    constexpr int TL = Plan<N1, E>::TL;
    constexpr int PADS = sizeof(C) == 8 ? 4 : 3;
    constexpr int LINE = padded<N1, PADS>(N1);
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C *>(smraw);
    const FsInst in = a.inst[blockIdx.y];
    const int tid = threadIdx.x;
    const int line = tid / TL, t = tid - line * TL;
    const int row = blockIdx.x * B + line;
    const RowLayout<PADS> lay{line * LINE};
    const auto lbar = LineBarrierOf<TL, B>::make(line);
    C *psi = static_cast<C *>(in.psi);
    const tw_t<C> *tw = static_cast<const tw_t<C> *>(a.tw_row);
    const size_t base = (size_t)row * N1 + t;

    C x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) x[e] = ld_stream(psi + base + e * TL);
    // FFT -> K -> iFFT, the iFFT as conj(FFT(conj(x)))
#pragma unroll 1
    for (int p = 0; p < 2; ++p) {
        line_fft<C, N1, E, false>(x, sm, lay, lbar, t, tw);
        if (p == 1) continue;
        const C *kt = opaque(static_cast<const C *>(in.ktab[a.ksel])) + base;
        if (a.plain) {
#pragma unroll
            for (int e = 0; e < E; ++e) x[e] = cconj(cmul(x[e], ld_stream(kt + e * TL)));
        } else {
#pragma unroll
            for (int e = 0; e < E; ++e) {
                C v = x[e];
                if constexpr (sizeof(C) == 8) v = cscale(v, a.inv_n);
                x[e] = cconj(PhaseOps<C>::apply(v, ld_stream(kt + e * TL)));
            }
        }
    }
    C *p = const_cast<C *>(opaque(psi)) + base;
#pragma unroll
    for (int e = 0; e < E; ++e) st_stream(p + e * TL, cconj(x[e]));
}


// Four-step kinetic energy: the row FFT of a k-layout array (after a column
// pass) with partials[2*cta] = sum |X|^2 fold(k)^2 dtk, [2*cta+1] = sum |X|^2.
template <class T, int N1, int E, int B>
__global__ void __launch_bounds__(B *(N1 / E)) k_fs_row_kinetic(FsRowArgs a, int n2, double dtk, double *partials)
{
    using C = cplx_t<T>;
    constexpr int TL = Plan<N1, E>::TL;
    constexpr int NT = B * TL;
    constexpr int PADS = sizeof(C) == 8 ? 4 : 3;
    constexpr int LINE = padded<N1, PADS>(N1);
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C *>(smraw);
    __shared__ double red[32];
    const FsInst in = a.inst[0];
    const int tid = threadIdx.x;
    const int line = tid / TL, t = tid - line * TL;
    const int row = blockIdx.x * B + line;
    const C *psi = static_cast<const C *>(in.psi);
    C x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) x[e] = psi[(size_t)row * N1 + t + e * TL];
    line_fft<C, N1, E, false>(x, sm, RowLayout<PADS>{line * LINE}, CtaBarrier{}, t,
                              static_cast<const tw_t<C> *>(a.tw_row));
    const long n = (long)N1 * n2;
    double k = 0, nn = 0;
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const long kk = row + (long)n2 * (t + e * TL);
        const double f = double(kk > n / 2 ? n - kk : kk);
        const double a2 = abs2d(x[e]);
        k += a2 * (f * f) * dtk;
        nn += a2;
    }
    k = block_sum<NT>(k, red);
    nn = block_sum<NT>(nn, red);
    if (tid == 0) {
        partials[2 * blockIdx.x] = k;
        partials[2 * blockIdx.x + 1] = nn;
    }
}

// Batched 1D resident evolution: one CTA per instance (blockIdx.x), all
// instances of the same N and order.
struct Evolve1DBatchArgs {
    const FsInst *inst;     // psi, vtab[0..1], ktab[0..1] (natural layout)
    const void *tw;
    double *norm_out;       // per-instance sum |psi|^2 (before renormalisation) or null
    const double *dv;       // per-instance volume element (renormalisation)
    uint64_t nsteps;
    int order, renormalize;
    int count;              // instances in the launch
};

// The lines of NI instances of length L, held by the NI * (L / E) threads of
// the CTA: instance `first + line` for line < count (the other lines run on
// instance `first` without storing), for all a.nsteps steps.
template <class T, int L, int E, int NI>
__device__ __forceinline__ void evolve1d_lines(const Evolve1DBatchArgs &a, int first, int count, const void *twp,
                                               unsigned char *smraw)
{
    using C = cplx_t<T>;
    using P = Plan<L, E>;
    constexpr int TL = P::TL;
    constexpr int PADS = sizeof(C) == 8 ? 4 : 3;
    C *sm = reinterpret_cast<C *>(smraw);
    const int line = threadIdx.x / TL;
    const int t = threadIdx.x - line * TL;
    const int idx = first + line;
    const bool active = line < count;
    const FsInst in = a.inst[active ? idx : first];
    C *psi = static_cast<C *>(in.psi);
    const tw_t<C> *tw = static_cast<const tw_t<C> *>(twp);
    const C *v0 = static_cast<const C *>(in.vtab[0]);
    const C *v1 = static_cast<const C *>(in.vtab[1]);
    const C *k0 = static_cast<const C *>(in.ktab[0]);
    const C *k1 = static_cast<const C *>(in.ktab[1]);
    const RowLayout<PADS> lay{line * padded<L, PADS>(L)};
    // instances are independent: lines of whole warps synchronise on their own
    const auto bar = LineBarrierOf<TL, NI>::make(line);
    constexpr T inv_n = T(1) / T(L);

    C x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) x[e] = psi[t + e * TL];

    // substep schedule: V(v[0]) T(k[0]) V(v[1]) T(k[1]) ... V(v[nsub])
    // O2: V1/2 T1 V1/2;  O4: VC1 TD1 VC2 TD2 VC2 TD1 VC1
    // T(k) = iFFT(k * FFT(x)) = conj(FFT(conj(k * FFT(x)))): each half-substep
    // is one forward transform followed by a conjugating multiply.
    const int nsub = a.order == 2 ? 1 : 3;
    // one count for the whole launch: instances that share a CTA synchronise
    // with CTA-wide barriers, so every line must run the same number of steps
    const uint64_t nsteps = a.nsteps;
#pragma unroll
    for (int e = 0; e < E; ++e) x[e] = PhaseOps<C>::apply(x[e], ld_c(v0 + t + e * TL));
    for (uint64_t s = 0; s < nsteps; ++s) {
#pragma unroll 1
        for (int h = 0; h < 2 * nsub; ++h) {
            line_fft<C, L, E, false>(x, sm, lay, bar, t, tw);
            const int u = h >> 1;
            if ((h & 1) == 0) {
                const C *kt = (a.order == 4 && u == 1) ? k1 : k0;
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    if constexpr (sizeof(C) == 8) x[e] = cscale(x[e], inv_n);
                    x[e] = cconj(PhaseOps<C>::apply(x[e], ld_c(kt + t + e * TL)));
                }
            } else {
                // the next V: the step's own closing factor, then (if more
                // steps follow) the next step's opening factor
                const bool last = u == nsub - 1;
                const C *vt = (a.order == 4 && !last) ? v1 : v0;
                const bool twice = last && s + 1 < nsteps;
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    const C m = ld_c(vt + t + e * TL);
                    x[e] = PhaseOps<C>::apply(cconj(x[e]), m);
                    if (twice) x[e] = PhaseOps<C>::apply(x[e], m);
                }
            }
        }
    }

    if (a.norm_out || a.renormalize) {
        // per-instance sum |psi|^2: shuffles within the line's lanes, then
        // (lines of whole warps) across the line's warps via shared memory
        double s = 0;
#pragma unroll
        for (int e = 0; e < E; ++e) s += abs2d(x[e]);
        double tot = 0;
        if constexpr (TL < 32) {
#pragma unroll
            for (int o = TL / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            tot = s;
        } else {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            __shared__ double wsum[32];
            __syncthreads();
            if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = s;
            __syncthreads();
            constexpr int WPL = TL / 32;  // warps per line
            for (int w = 0; w < WPL; ++w) tot += wsum[line * WPL + w];
        }
        if (t == 0 && a.norm_out && active) a.norm_out[idx] = tot;
        if (a.renormalize && active) {
            const T sc = T(1.0 / sqrt(tot * a.dv[idx]));
#pragma unroll
            for (int e = 0; e < E; ++e) x[e] = cscale(x[e], sc);
        }
    }
    if (active) {
#pragma unroll
        for (int e = 0; e < E; ++e) psi[t + e * TL] = x[e];
    }
}

template <class T, int L, int E, int NI>
__global__ void __launch_bounds__(NI *(L / E)) k_evolve1d_resident(Evolve1DBatchArgs a)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    const int first = blockIdx.x * NI;
    evolve1d_lines<T, L, E, NI>(a, first, a.count - first, a.tw, smraw);
}

// One persistent launch over the resident-size classes of a batch with
// lengths 1024 .. QT (smaller lengths, whose bodies would push the shared
// register allocation into spills, keep their own launches): a work queue of
// tiles of QT sites (QT / L instances of one length L, every tile filling the
// CTA's QT / E threads); each CTA takes the next tile from a
// device counter until the queue is empty.  Tiles are independent (a tile
// holds its instances for all the steps of the call), so no CTA ever waits on
// another.  The last CTA to finish resets the counter for the next launch.
struct QueueTile {
    const void *tw;  // stage-major twiddles of the tile's length
    int L;           // line length
    int first;       // first instance (index into the launch's descriptors)
    int count;       // instances in the tile (<= QT / L)
    int pad;
};
struct Evolve1DQueueArgs {
    Evolve1DBatchArgs b;    // descriptors, dv, norm_out, nsteps, order, renormalize
    const QueueTile *tiles;
    int ntiles;
    unsigned *counter;      // [0]: next tile, [1]: CTAs finished
};

template <class T, int QT, int E>
__global__ void __launch_bounds__(QT / E) k_evolve1d_queue(Evolve1DQueueArgs a)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ int tile_s;
#pragma unroll 1
    for (;;) {
        __syncthreads();  // every thread is done with the previous tile (and tile_s)
        if (threadIdx.x == 0) tile_s = (int)atomicAdd(a.counter, 1u);
        __syncthreads();
        const int k = tile_s;
        if (k >= a.ntiles) break;
        const QueueTile tl = a.tiles[k];
        switch (tl.L) {
#define QSG_QUEUE_CASE(LL) \
    case LL: \
        if constexpr (LL <= QT) evolve1d_lines<T, LL, E, QT / LL>(a.b, tl.first, tl.count, tl.tw, smraw); \
        break;
            QSG_QUEUE_CASE(1024) QSG_QUEUE_CASE(2048) QSG_QUEUE_CASE(4096) QSG_QUEUE_CASE(8192)
#undef QSG_QUEUE_CASE
        default:
            break;
        }
    }
    if (threadIdx.x == 0) {
        // the last CTA out resets the queue (every CTA has taken its final,
        // out-of-range ticket by now)
        __threadfence();
        if (atomicAdd(a.counter + 1, 1u) == gridDim.x - 1) {
            a.counter[0] = 0u;
            a.counter[1] = 0u;
        }
    }
}

// ---------------------------------------------------------------------------
// 1D infinite wall (SplittingMethod1D::ExpT, src/SplittingMethod1D.cpp:61-81):
// psi on [0, N) with psi_0 = psi_N = 0, odd extension to 2N, inverse 2N-point
// transform, K_i = exp(f i^2) on the first N outputs, odd extension again,
// inverse transform, first N values times -1/(2N).  One CTA holds the 2N line
// (slot e of thread t is element t + e*L2/E; slots e < E/2 are psi itself).
// ---------------------------------------------------------------------------

// odd extension of the first half into the second: x_0 = x_N = 0,
// x_{2N-k} = -x_k (k = 1 .. N-1)
template <class C, int L2, int E, class Lay>
__device__ __forceinline__ void odd_extend(C (&x)[E], C *sm, const Lay &lay, int t)
{
    constexpr int TL = L2 / E;
    __syncthreads();  // the buffer is free
#pragma unroll
    for (int e = 0; e < E / 2; ++e) sm[lay(t + e * TL)] = x[e];
    __syncthreads();
#pragma unroll
    for (int e = E / 2; e < E; ++e) {
        const int idx = t + e * TL;
        x[e] = idx == L2 / 2 ? cmk<C>(0, 0) : csub(cmk<C>(0, 0), sm[lay(L2 - idx)]);
    }
    if (t == 0) x[0] = cmk<C>(0, 0);
}

template <class T, int L2, int E>
__global__ void __launch_bounds__(L2 / E) k_evolve1d_wall(Evolve1DBatchArgs a)
{
    using C = cplx_t<T>;
    constexpr int TL = L2 / E;
    constexpr int H = E / 2;  // slots holding psi
    constexpr int PADS = sizeof(C) == 8 ? 4 : 3;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C *>(smraw);
    __shared__ double red[32];
    const int t = threadIdx.x;
    const FsInst in = a.inst[blockIdx.x];
    C *psi = static_cast<C *>(in.psi);
    const tw_t<C> *tw = static_cast<const tw_t<C> *>(a.tw);
    const C *v0 = static_cast<const C *>(in.vtab[0]);
    const C *v1 = static_cast<const C *>(in.vtab[1]);
    const C *k0 = static_cast<const C *>(in.ktab[0]);
    const C *k1 = static_cast<const C *>(in.ktab[1]);
    const RowLayout<PADS> lay{0};
    const CtaBarrier bar{};
    constexpr T neg_inv_2n = T(-1) / T(L2);

    C x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) x[e] = e < H ? psi[t + e * TL] : cmk<C>(0, 0);

    const int nsub = a.order == 2 ? 1 : 3;
    const uint64_t nsteps = a.nsteps;
#pragma unroll
    for (int e = 0; e < H; ++e) x[e] = PhaseOps<C>::apply(x[e], ld_c(v0 + t + e * TL));
    for (uint64_t s = 0; s < nsteps; ++s) {
        for (int u = 0; u < nsub; ++u) {
            const C *kt = (a.order == 4 && u == 1) ? k1 : k0;
            // two inverse transforms of odd extensions, K between them
#pragma unroll 1
            for (int h = 0; h < 2; ++h) {
                odd_extend<C, L2, E>(x, sm, lay, t);
#pragma unroll
                for (int e = 0; e < E; ++e) x[e] = cconj(x[e]);
                line_fft<C, L2, E, false>(x, sm, lay, bar, t, tw);
#pragma unroll
                for (int e = 0; e < E; ++e) x[e] = cconj(x[e]);
                if (h == 0) {
#pragma unroll
                    for (int e = 0; e < H; ++e) {
                        if constexpr (sizeof(C) == 8) x[e] = cscale(x[e], neg_inv_2n);
                        x[e] = PhaseOps<C>::apply(x[e], ld_c(kt + t + e * TL));
                    }
                }
            }
            const bool last = u == nsub - 1;
            const C *vt = (a.order == 4 && !last) ? v1 : v0;
            const bool twice = last && s + 1 < nsteps;
#pragma unroll
            for (int e = 0; e < H; ++e) {
                const C m = ld_c(vt + t + e * TL);
                x[e] = PhaseOps<C>::apply(x[e], m);
                if (twice) x[e] = PhaseOps<C>::apply(x[e], m);
            }
        }
    }
    if (a.norm_out || a.renormalize) {
        double sum = 0;
#pragma unroll
        for (int e = 0; e < H; ++e) sum += abs2d(x[e]);
        sum = block_sum<L2 / E>(sum, red);
        if (t == 0 && a.norm_out) a.norm_out[blockIdx.x] = sum;
        if (a.renormalize) {
            const T sc = T(1.0 / sqrt(sum * a.dv[blockIdx.x]));
#pragma unroll
            for (int e = 0; e < H; ++e) x[e] = cscale(x[e], sc);
        }
    }
#pragma unroll
    for (int e = 0; e < H; ++e) psi[t + e * TL] = x[e];
}

// <T> with the wall (SplittingMethod1D::CalKinEn, :110-124): odd extension,
// inverse 2N transform, sums[0] = sum_{i<N} |X_i|^2 i^2 dtk, sums[1] = sum_{i<N} |X_i|^2
template <class T, int L2, int E>
__global__ void __launch_bounds__(L2 / E) k_kinetic1d_wall(const void *psi_, const void *tw_, double dtk, double *sums)
{
    using C = cplx_t<T>;
    constexpr int TL = L2 / E;
    constexpr int H = E / 2;
    constexpr int PADS = sizeof(C) == 8 ? 4 : 3;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C *>(smraw);
    __shared__ double red[32];
    const int t = threadIdx.x;
    const C *psi = static_cast<const C *>(psi_);
    const RowLayout<PADS> lay{0};
    C x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) x[e] = e < H ? psi[t + e * TL] : cmk<C>(0, 0);
    odd_extend<C, L2, E>(x, sm, lay, t);
#pragma unroll
    for (int e = 0; e < E; ++e) x[e] = cconj(x[e]);
    line_fft<C, L2, E, false>(x, sm, lay, CtaBarrier{}, t, static_cast<const tw_t<C> *>(tw_));
    double k = 0, nn = 0;
#pragma unroll
    for (int e = 0; e < H; ++e) {
        const double i = double(t + e * TL);
        const double a2 = abs2d(x[e]);
        k += a2 * (i * i);
        nn += a2;
    }
    k = block_sum<L2 / E>(k, red);
    nn = block_sum<L2 / E>(nn, red);
    if (t == 0) {
        sums[0] = k * dtk;
        sums[1] = nn;
    }
}

}  // namespace qsg
