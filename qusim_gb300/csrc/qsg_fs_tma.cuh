// qsg_fs_tma.cuh -- 1D four-step column pass fed by tensor copies (complex64).
//
// Same arithmetic as k_fs_col (conjugate twiddle, column iFFT, V phase, column
// FFT, twiddle; SplittingMethod1D's ExpV between the two halves of the
// four-step transform), so the results are bitwise those of k_fs_col.  The
// instance's state and V-table blocks of a tile (N2 rows x W columns, 32 KB
// each) arrive in shared memory by 2D tensor copies, one mbarrier per buffer,
// each buffer's next copy issued as soon as every thread has read it.  Two
// 256-thread CTAs per SM walk the tiles u = (instance, column block) of the
// launch, u = blockIdx.x, + gridDim.x, ...  The tensor maps are per instance
// (state, V table 0, V table 1), in device memory.  Waits are bounded as in
// k_col_pass_tma.
#pragma once
#include "qsg_col_tma.cuh"

namespace qsg {

__host__ __device__ constexpr size_t fs_tma_ex_bytes(int n2, int w)
{
    return ((size_t)8 * col_tile_elems(8, n2, w) + 1023) / 1024 * 1024;
}
__host__ __device__ constexpr size_t fs_tma_smem(int n2, int w) { return fs_tma_ex_bytes(n2, w) + 2 * (size_t)8 * n2 * w; }

template <int N2, int W>
__global__ void __launch_bounds__(W *(N2 / 16), 2) k_fs_col_tma(FsColArgs a)
{
    using C = float2;
    constexpr int E = 16;
    constexpr int TM = Plan<N2, E>::TL;
    constexpr int NT = W * TM;
    constexpr int TILE = N2 * W;
    constexpr int BOXR = N2 < 256 ? N2 : 256;  // rows per box
    constexpr int BOXES = N2 / BOXR;
    extern __shared__ __align__(128) unsigned char smraw[];
    __shared__ double red[32];
    __shared__ __align__(8) uint64_t mbar[2];
    C *sm = reinterpret_cast<C *>(smraw);
    const uint32_t sb = tma::smem_u32(smraw + fs_tma_ex_bytes(N2, W));
    C *xb = reinterpret_cast<C *>(smraw + fs_tma_ex_bytes(N2, W) + ((128 - (sb & 127)) & 127));
    C *vb = xb + TILE;
    const CUtensorMap *maps = static_cast<const CUtensorMap *>(a.maps);
    const bool in_k = a.in_k != 0, out_k = a.out_k != 0;
    const int tid = threadIdx.x;
    const int c = tid % W, t = tid / W;
    const int n1 = a.n1;
    const int cb = n1 / W;  // column blocks per instance
    const tw_t<C> *tw = static_cast<const tw_t<C> *>(a.tw_col);
    const tw_t<C> *twn = static_cast<const tw_t<C> *>(a.tw_n);
    constexpr ColPad CP = col_pad(sizeof(C), N2, W);
    const ColLayout<W, CP.sh, CP.p> lay{c};
    const CtaBarrier bar{};
    const size_t stride = (size_t)TM * n1;
    const uint32_t mb_x = tma::smem_u32(&mbar[0]), mb_v = tma::smem_u32(&mbar[1]);

    if (tid == 0) {
        tma::mbar_init(mb_x, 1);
        tma::mbar_init(mb_v, 1);
        tma::fence_mbar_init();
    }
    __syncthreads();

    // thread 0: column block b of a map into dst, completing on mb
    auto issue = [&](uint32_t mb, const CUtensorMap *map, C *dst, int b) {
        tma::mbar_expect_tx(mb, (uint32_t)(TILE * sizeof(C)));
#pragma unroll
        for (int r = 0; r < BOXES; ++r) tma::load_2d(tma::smem_u32(dst + r * BOXR * W), map, b * W, r * BOXR, mb);
    };
    auto issue_tile = [&](int uu, bool x, bool v) {
        const int i = uu / cb, b = uu - i * cb;
        if (x) issue(mb_x, maps + 3 * i, xb, b);
        if (v) issue(mb_v, maps + 3 * i + 1 + a.vsel, vb, b);
    };

    int u = blockIdx.x;
    uint32_t ph_x = 0, ph_v = 0;
    int in_flight_x = 0, in_flight_v = 0;
    if (tid == 0 && u < a.tiles) {
        issue_tile(u, true, true);
        in_flight_x = in_flight_v = 1;
    }
    bool ok = true;

#pragma unroll 1
    for (; u < a.tiles; u += gridDim.x) {
        const int i = u / cb, b = u - i * cb;
        const FsInst in = a.inst[i];
        const int col = b * W + c;
        const size_t base = (size_t)t * n1 + col;
        const int unext = u + gridDim.x;
        C *psi = static_cast<C *>(in.psi);

        ok = __syncthreads_and(tma::mbar_wait(mb_x, ph_x, kTmaWaitNs));
        if (!ok) break;
        ph_x ^= 1;
        if (tid == 0) in_flight_x = 0;
        C x[E];
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = xb[(t + e * TM) * W + c];
        __syncthreads();  // every thread has read xb
        if (tid == 0 && unext < a.tiles) {
            tma::fence_proxy_async();
            issue_tile(unext, true, false);
            in_flight_x = 1;
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
                ok = __syncthreads_and(tma::mbar_wait(mb_v, ph_v, kTmaWaitNs));
                if (!ok) break;
                ph_v ^= 1;
                if (tid == 0) in_flight_v = 0;
                C mv[E];
#pragma unroll
                for (int e = 0; e < E; ++e) mv[e] = vb[(t + e * TM) * W + c];
                __syncthreads();  // every thread has read vb
                if (tid == 0 && unext < a.tiles) {
                    tma::fence_proxy_async();
                    issue_tile(unext, false, true);
                    in_flight_v = 1;
                }
                if (a.vtwice) {
#pragma unroll
                    for (int e = 0; e < E; ++e) x[e] = PhaseOps<C>::apply(PhaseOps<C>::apply(x[e], mv[e]), mv[e]);
                } else {
#pragma unroll
                    for (int e = 0; e < E; ++e) x[e] = PhaseOps<C>::apply(x[e], mv[e]);
                }
            }
            if (p < npass) line_fft<C, N2, E, false>(x, sm, lay, bar, t, tw);
        }
        if (!ok) break;
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
            if (tid == 0) in.partials[b] = nsum;
        }
    }
    if (!ok && tid == 0) {
        if (a.err) atomicAdd(a.err, 1);  // a count: each failure is seen by every instance it touched
        if (in_flight_x) tma::mbar_wait(mb_x, ph_x, kTmaDrainNs);
        if (in_flight_v) tma::mbar_wait(mb_v, ph_v, kTmaDrainNs);
    }
}

}  // namespace qsg
