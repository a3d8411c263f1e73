// qsg_row_tm.cuh -- 2D row pass with the waiting lines parked in tensor memory.
//
// Same pass as k_row_pass (inverse x-split stage, row iFFT, V, row FFT,
// forward x-split stage; SplittingMethod2D ExpV / the row half of ExpT,
// src/SplittingMethod2D.cpp:81-121), organised around the Blackwell tensor
// memory (TMEM, 256 KB per SM beside shared memory):
//
//   - NT = NY/16 threads transform one line at a time; thread t owns columns
//     t + e*NT (e < 16) of every line of the unit, so the radix-G x-split
//     stages across the G lines are thread-local register arithmetic;
//   - the lines of a unit that are not being transformed wait in the thread's
//     own TMEM lane (tcgen05.st / tcgen05.ld, 32 floats per line);
//   - shared memory holds only the exchange buffer of the line in flight
//     (35 KB at NY = 4096), so one 512-thread CTA runs 512/NT independent
//     groups, each with its own buffer, named barrier and sequence of units;
//     the groups drift apart and overlap each other's memory phases.
//
// The runtime schedules one CTA per SM for a kernel that allocates TMEM, so
// the CTA takes all 512 columns: each thread owns 128 columns of its lane
// (G = 4 slots of 32 floats), 4 threads per lane.
#pragma once
#include <cstdint>
#include "qsg_kernels.cuh"

namespace qsg {

namespace tm {

// 32x32b shape: thread i of a warp reads / writes TMEM lane (lane field of
// taddr) + i, columns [col, col + 8) of 32-bit words.
__device__ __forceinline__ void st8(uint32_t taddr, const float2 (&v)[4])
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
                 "f"(v[0].x), "f"(v[0].y), "f"(v[1].x), "f"(v[1].y), "f"(v[2].x), "f"(v[2].y), "f"(v[3].x),
                 "f"(v[3].y)
                 : "memory");
}
__device__ __forceinline__ void ld8(uint32_t taddr, float2 (&v)[4])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=f"(v[0].x), "=f"(v[0].y), "=f"(v[1].x), "=f"(v[1].y), "=f"(v[2].x), "=f"(v[2].y),
                   "=f"(v[3].x), "=f"(v[3].y)
                 : "r"(taddr)
                 : "memory");
}
__device__ __forceinline__ void wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// park / fetch a whole line slot (16 complex = 4 chunks of 8 words)
__device__ __forceinline__ void st_line(uint32_t taddr, const float2 (&x)[16])
{
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const float2 v[4] = {x[4 * c], x[4 * c + 1], x[4 * c + 2], x[4 * c + 3]};
        st8(taddr + 8 * c, v);
    }
}
__device__ __forceinline__ void ld_line(uint32_t taddr, float2 (&x)[16])
{
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        float2 v[4];
        ld8(taddr + 8 * c, v);
#pragma unroll
        for (int i = 0; i < 4; ++i) x[4 * c + i] = v[i];
    }
}

}  // namespace tm

// sum of v over the NT threads of group grp (named barrier 1 + grp); thread 0
// of the group gets the result
template <int NT>
__device__ __forceinline__ double group_sum(double v, double *red, int grp, int gt)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const NamedBarrier gb{1 + grp, NT};
    gb();
    if ((gt & 31) == 0) red[gt >> 5] = v;
    gb();
    double s = 0;
    if (gt == 0)
        for (int i = 0; i < NT / 32; ++i) s += red[i];
    gb();
    return s;
}

// One unit = the G = 4 lines n1 + j*M (j < 4) of row group n1 = u.  Group grp
// of NG takes units grp + NG*blockIdx.x, then every NG*gridDim.x-th.
template <int NY, bool IN, bool PL>
__device__ __forceinline__ void row_tm_units(const RowPassArgs &a, float2 *sm, double *red, uint32_t tbase,
                                             int grp, int gt)
{
    using C = float2;
    using TW = pass_tw_t<C, PL>;
    constexpr int E = 16, G = 4;
    constexpr int NT = NY / E;
    constexpr int NG = 512 / NT;
    constexpr int PADS = 4;
    const int tid = gt;  // thread within the group: owns columns tid + e*NT
    const int w = threadIdx.x >> 5;
    // this thread's TMEM words: lane quadrant of its warp, 128 columns per thread
    const uint32_t taddr = tbase + ((uint32_t)(32 * (w & 3)) << 16) + (uint32_t)((w >> 2) * 128);
    const C *in = static_cast<const C *>(a.in);
    C *out = static_cast<C *>(a.out);
    const TW *tw = static_cast<const TW *>(a.tw_row);
    const TW *twx = static_cast<const TW *>(a.tw_nx);
    const C *vt = static_cast<const C *>(a.vtab);
    const bool out_split = a.out_split != 0;
    const RowLayout<PADS> lay{0};
    const NamedBarrier bar{1 + grp, NT};
    const int u0 = grp + NG * blockIdx.x, ustep = NG * gridDim.x;

    // split-k input chunk c of unit uu: rows q*M + uu, columns t + (4c + i)*NT.
    // Every path defines pf (zeros when !live), so consumed values are dead
    // during the transforms.
    C pf[G][4];
    auto xs_load = [&](int uu, int c, bool live) {
#pragma unroll
        for (int q = 0; q < G; ++q)
#pragma unroll
            for (int i = 0; i < 4; ++i)
                pf[q][i] = live ? ld_stream(in + (size_t)(q * a.m + uu) * NY + tid + (4 * c + i) * NT)
                                : cmk<C>(0, 0);
    };
    if constexpr (IN) xs_load(u0 < a.units ? u0 : 0, 0, u0 < a.units);

#pragma unroll 1
    for (int u = u0; u < a.units; u += ustep) {
        const int unext = u + ustep;
        C x[E];
        if constexpr (IN) {
            // inverse x-split stage, thread-local: line 0 stays in registers,
            // lines 1..3 go to TMEM slots 1..3
            TW tq[G];
#pragma unroll
            for (int q = 1; q < G; ++q) tq[q] = __ldg(twx + u * q);
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                C y[G][4];
#pragma unroll
                for (int q = 0; q < G; ++q)
#pragma unroll
                    for (int i = 0; i < 4; ++i) y[q][i] = pf[q][i];
                if (c < 3) xs_load(u, c + 1, true);
                C z[G][4];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    C v[G];
#pragma unroll
                    for (int q = 0; q < G; ++q) v[q] = q > 0 ? twmul<true>(y[q][i], tq[q]) : y[q][i];
                    dftg<G, true>(v);
#pragma unroll
                    for (int q = 0; q < G; ++q) z[q][i] = v[q];
                }
#pragma unroll
                for (int i = 0; i < 4; ++i) x[4 * c + i] = z[0][i];
#pragma unroll
                for (int j = 1; j < G; ++j) tm::st8(taddr + 32 * j + 8 * c, z[j]);
            }
        }

        double nsum = 0;
#pragma unroll 1
        for (int r = 0; r < G; ++r) {
            const int row = u + r * a.m;
            if constexpr (IN) {
                if (r > 0) {
                    tm::wait_st();
                    tm::ld_line(taddr + 32 * r, x);
                    tm::wait_ld();
                }
            } else {
                const C *ir = in + (size_t)row * NY + tid;
#pragma unroll
                for (int e = 0; e < E; ++e) x[e] = ld_stream(ir + e * NT);
            }
            // [row iFFT] -> V -> [row FFT], the iFFT as conj(FFT(conj(x)))
            const int npass = (IN ? 1 : 0) + (out_split ? 1 : 0);
            constexpr int vpos = IN ? 1 : 0;
            if constexpr (IN) {
#pragma unroll
                for (int e = 0; e < E; ++e) x[e] = cconj(x[e]);
            }
#pragma unroll 1
            for (int p = 0; p <= npass; ++p) {
                if (p == vpos) {
                    if constexpr (IN) {
#pragma unroll
                        for (int e = 0; e < E; ++e) x[e] = cconj(x[e]);
                    }
                    if (vt) {
                        const C *vr = opaque(vt) + (size_t)row * NY + tid;
                        C mv[E];
#pragma unroll
                        for (int e = 0; e < E; ++e) mv[e] = ld_stream(vr + e * NT);
                        if (a.vdiff) {
#pragma unroll
                            for (int e = 0; e < E; ++e) x[e] = PhaseOps<C>::increment(x[e], mv[e], a.vtwice);
                        } else if (a.vtwice) {
#pragma unroll
                            for (int e = 0; e < E; ++e) x[e] = cmul1p(cmul1p(x[e], mv[e]), mv[e]);
                        } else {
#pragma unroll
                            for (int e = 0; e < E; ++e) x[e] = cmul1p(x[e], mv[e]);
                        }
                    }
                }
                if (p < npass) line_fft<C, NY, E, false>(x, sm, lay, bar, tid, tw);
            }
            if (!out_split) {
                C *orow = const_cast<C *>(opaque(out)) + (size_t)row * NY + tid;
#pragma unroll
                for (int e = 0; e < E; ++e) {
                    st_stream(orow + e * NT, x[e]);
                    nsum += abs2d(x[e]);
                }
            } else if (r < G - 1) {
                tm::st_line(taddr + 32 * r, x);  // line 3 stays in registers
            }
        }

        // the next unit's first input chunk is in flight while this unit's
        // results go out
        if constexpr (IN) xs_load(unext < a.units ? unext : u, 0, unext < a.units);
        if (out_split) {
            // forward x-split stage, thread-local, straight to the output rows
            TW tq[G];
#pragma unroll
            for (int q = 1; q < G; ++q) tq[q] = __ldg(twx + u * q);
            tm::wait_st();
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                C l[G - 1][4];
#pragma unroll
                for (int j = 0; j < G - 1; ++j) tm::ld8(taddr + 32 * j + 8 * c, l[j]);
                tm::wait_ld();
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    C v[G];
#pragma unroll
                    for (int j = 0; j < G - 1; ++j) v[j] = l[j][i];
                    v[G - 1] = x[4 * c + i];
                    dftg<G, false>(v);
#pragma unroll
                    for (int q = 0; q < G; ++q) {
                        if (q > 0) v[q] = twmul<false>(v[q], tq[q]);
                        st_stream(out + (size_t)(q * a.m + u) * NY + tid + (4 * c + i) * NT, v[q]);
                    }
                }
            }
        } else if (a.partials) {
            nsum = group_sum<NT>(nsum, red + 32 * grp, grp, gt);
            if (gt == 0) a.partials[u] = nsum;
        }
    }
}

template <int NY, bool PL = false>
__global__ void __launch_bounds__(512, 1) k_row_pass_tm(RowPassArgs a)
{
    constexpr int NT = NY / 16;
    constexpr int LINE = padded<NY, 4>(NY);
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[4 * 32];
    __shared__ uint32_t tbase_s;
    const int w = threadIdx.x >> 5;
    if (w == 0) {
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&tbase_s);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(dst) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tbase = tbase_s;
    const int grp = threadIdx.x / NT, gt = threadIdx.x - grp * NT;
    float2 *sm = reinterpret_cast<float2 *>(smraw) + grp * LINE;
    if (a.in_split)
        row_tm_units<NY, true, PL>(a, sm, red, tbase, grp, gt);
    else
        row_tm_units<NY, false, PL>(a, sm, red, tbase, grp, gt);
    tm::wait_st();
    tm::wait_ld();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (w == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tbase) : "memory");
    }
}

}  // namespace qsg
