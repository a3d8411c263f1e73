// qsg_col_tma.cuh -- momentum-form column pass fed by the tensor memory
// accelerator (TMA).
//
// Same arithmetic as k_col_pass's momentum path (column FFT of the potential
// increment, + the stored state P, x Kx Ky, store P, column iFFT of P to the
// work buffer), so the results are bitwise those of k_col_pass.  What changes
// is the data movement: one persistent 256-thread CTA per SM walks tiles
// u = blockIdx.x, + gridDim.x, ...; a tile's increment and stored-state
// blocks (M rows x W columns, 64 KB each) arrive in shared memory by 2D tensor
// copies (cp.async.bulk.tensor, M/256 boxes of 256 rows x W columns each),
// completing on one mbarrier per buffer.  A buffer's next copy is issued as
// soon as every thread has read it, so the next tile's loads run under this
// tile's transforms:
//
//   wait W(u)  -> read -> [issue W(u+grid)] -> FFT -> wait P(u) -> P += ...
//   -> read / store P -> [issue P(u+grid)] -> iFFT -> store W
//
// Every wait is bounded (1 s on %globaltimer); a CTA that runs out sets the
// error flag, waits (bounded again) for its copies in flight and returns, and
// the host reports QSG_ERR_TIMEOUT at its next synchronisation.
#pragma once
#include <cuda.h>
#include "qsg_kernels.cuh"

namespace qsg {

namespace tma {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t mb, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mb), "r"(count) : "memory");
}
// the barrier inits visible to the async (TMA) proxy
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// generic-proxy accesses of shared memory ordered before later async-proxy ones
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint32_t mb, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(bytes) : "memory");
}

// box at (x = column, y = row) of a 2D tensor map into shared memory
__device__ __forceinline__ void load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t mb)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"(map), "r"(x), "r"(y), "r"(mb)
        : "memory");
}

__device__ __forceinline__ uint64_t now_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// wait for phase `parity` of the barrier to complete, for at most limit_ns
__device__ __forceinline__ bool mbar_wait(uint32_t mb, uint32_t parity, uint64_t limit_ns)
{
    const uint64_t t0 = now_ns();
    while (true) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(mb), "r"(parity)
            : "memory");
        if (done) return true;
        if (now_ns() - t0 > limit_ns) return false;
    }
}

}  // namespace tma

constexpr uint64_t kTmaWaitNs = 1000000000ull;  // 1 s
// After a wait ran out, the issuing thread gives the copies it still has in
// flight this much longer to land before the CTA exits; a copy that lands
// later would write into shared memory the CTA no longer owns, so this limit is
// the longer one (the first wait can also run out on a time-sliced GPU).
constexpr uint64_t kTmaDrainNs = 4 * kTmaWaitNs;

// shared-memory bytes of the exchange buffer, rounded up so that the staging
// buffers after it start on a 1024-byte boundary
__host__ __device__ constexpr size_t col_tma_ex_bytes(int m, int w, int e)
{
    return ((size_t)8 * col_tile_elems(8, m, w, e) + 1023) / 1024 * 1024;
}
__host__ __device__ constexpr size_t col_tma_smem(int m, int w, int e) { return col_tma_ex_bytes(m, w, e) + 2 * (size_t)8 * m * w; }

template <int M, int E, int W, bool PL>
__global__ void __launch_bounds__(W *(M / E), 1)
    k_col_pass_tma(ColPassArgs a, const __grid_constant__ CUtensorMap map_w, const __grid_constant__ CUtensorMap map_p)
{
    using C = float2;
    using TW = pass_tw_t<C, PL>;
    using P = Plan<M, E>;
    constexpr int TM = P::TL;
    constexpr int NT = W * TM;
    constexpr int TILE = M * W;  // complex elements of one staging buffer
    constexpr int BOXES = M / 256;
    static_assert(M % 256 == 0, "boxes of 256 rows");
    extern __shared__ __align__(128) unsigned char smraw[];
    __shared__ double red[32];
    __shared__ __align__(8) uint64_t mbar[2];
    C *sm = reinterpret_cast<C *>(smraw);
    // staging buffers on a 128-byte boundary (the launch adds 128 bytes of slack)
    const uint32_t sb = tma::smem_u32(smraw + col_tma_ex_bytes(M, W, E));
    C *wb = reinterpret_cast<C *>(smraw + col_tma_ex_bytes(M, W, E) + ((128 - (sb & 127)) & 127));
    C *pb = wb + TILE;
    const int tid = threadIdx.x;
    const int c = tid % W, t = tid / W;
    const int ny = a.ny;
    const int ntx = ny / W;
    C *psi = static_cast<C *>(a.psi);
    C *work = static_cast<C *>(a.work);
    const TW *tw = static_cast<const TW *>(a.tw_col);
    constexpr ColPad CP = col_pad(sizeof(C), M, W, E);
    const ColLayout<W, CP.sh, CP.p> lay{c};
    const CtaBarrier bar{};
    const int stride = TM * ny;
    const uint32_t mb_w = tma::smem_u32(&mbar[0]), mb_p = tma::smem_u32(&mbar[1]);

    if (tid == 0) {
        tma::mbar_init(mb_w, 1);
        tma::mbar_init(mb_p, 1);
        tma::fence_mbar_init();
    }
    __syncthreads();

    // thread 0: the copies of tile u's block of `map` into dst, completing on mb
    auto issue = [&](uint32_t mb, const CUtensorMap *map, C *dst, int u) {
        const int q = u / ntx;
        const int x = (u - q * ntx) * W;
        tma::mbar_expect_tx(mb, (uint32_t)(TILE * sizeof(C)));
#pragma unroll
        for (int b = 0; b < BOXES; ++b) tma::load_2d(tma::smem_u32(dst + b * 256 * W), map, x, q * M + b * 256, mb);
    };

    int u = blockIdx.x;
    uint32_t ph_w = 0, ph_p = 0;
    int in_flight_w = 0, in_flight_p = 0;  // (thread 0's view, for the error path)
    if (tid == 0 && u < a.tiles && !a.no_copies) {
        issue(mb_w, &map_w, wb, u);
        issue(mb_p, &map_p, pb, u);
        in_flight_w = in_flight_p = 1;
    }
    bool ok = true;

#pragma unroll 1
    for (; u < a.tiles; u += gridDim.x) {
        const int q = u / ntx;
        const int col = (u - q * ntx) * W + c;
        const size_t base = ((size_t)q * M + t) * ny + col;
        const int unext = u + gridDim.x;

        // the increment
        ok = __syncthreads_and(tma::mbar_wait(mb_w, ph_w, kTmaWaitNs));
        if (!ok) break;
        ph_w ^= 1;
        if (tid == 0) in_flight_w = 0;
        C x[E];
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = wb[(t + e * TM) * W + c];
        __syncthreads();  // every thread has read wb
        if (tid == 0 && unext < a.tiles) {
            tma::fence_proxy_async();
            issue(mb_w, &map_w, wb, unext);
            in_flight_w = 1;
        }

        float nf = 0;
#pragma unroll 1
        for (int p = 0; p < 2; ++p) {
            line_fft<C, M, E, false>(x, sm, lay, bar, t, tw);
            if (p == 1) continue;
            const C *kx = opaque(static_cast<const C *>(a.kx));
            const C ky = ld_c(static_cast<const C *>(a.ky) + col);
            ok = __syncthreads_and(tma::mbar_wait(mb_p, ph_p, kTmaWaitNs));
            if (!ok) break;
            ph_p ^= 1;
            if (tid == 0) in_flight_p = 0;
            C *ps = const_cast<C *>(opaque(psi)) + base;
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const int kxi = a.g * (t + e * TM) + q;
                C v = cscale(x[e], a.inv_n);
                v = cadd(pb[(t + e * TM) * W + c], v);
                v = cmul1p(v, ld_c(kx + kxi));
                v = cmul1p(v, ky);
                st_stream(ps + (size_t)e * stride, v);
                nf = fmaf(v.x, v.x, fmaf(v.y, v.y, nf));
                x[e] = cconj(v);
            }
            __syncthreads();  // every thread has read pb
            if (tid == 0 && unext < a.tiles) {
                tma::fence_proxy_async();
                issue(mb_p, &map_p, pb, unext);
                in_flight_p = 1;
            }
        }
        if (!ok) break;
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = cconj(x[e]);
        {
            C *o = const_cast<C *>(opaque(work)) + base;
#pragma unroll
            for (int e = 0; e < E; ++e) st_stream(o + (size_t)e * stride, x[e]);
        }
        if (a.partials) {
            const double s = block_sum<NT>((double)nf, red);
            if (tid == 0) a.partials[u] = s;
        }
    }
    if (!ok && tid == 0) {
        // record the timeout, then give the copies still in flight a bounded
        // chance to land before the CTA (and its shared memory) goes away
        if (a.err) atomicAdd(a.err, 1);  // a count: each failure is seen by every instance it touched
        if (in_flight_w) tma::mbar_wait(mb_w, ph_w, kTmaDrainNs);
        if (in_flight_p) tma::mbar_wait(mb_p, ph_p, kTmaDrainNs);
    }
}

}  // namespace qsg
