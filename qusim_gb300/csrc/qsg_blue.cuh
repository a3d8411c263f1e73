// qsg_blue.cuh -- split-operator steps on grids whose sizes are not powers of
// two, through Bluestein's algorithm on the power-of-two transforms.
//
// The reference transforms any length with KISS's mixed radix (factors 4, 2,
// 3, 5, then any prime; src/kissfft.hh:26-45, 185-345), so SplittingMethod1D/2D
// run on any n (its own FFT test uses 1234 and 123 x 234,
// applications/QuSimTest/TestFFT.cpp:89-99).  Here an n-point DFT is computed
// as a circular convolution of length M (a power of two, M >= 2n - 1):
//
//   X_k = w_k sum_j (x_j w_j) h_{k-j},   w_j = exp(-i pi j^2 / n),  h = conj(w)
//       = w_k [ iFFT_M( FFT_M(x w) . FFT_M(h) ) ]_k
//
// with h laid out circularly (h_j and h_{M-j} for j < n, zeros between).
// FFT_M(h) / M is a table (hs), so one n-point DFT is two M-point transforms
// and three pointwise products; the inverse DFT is conj(DFT(conj(.))).  The
// kinetic multiply sits between a forward and an inverse DFT, where the
// output chirp of the first and the input chirp of the second cancel
// (conj(w_k b_k K_k) w_k = conj(b_k K_k) for |w_k| = 1 in exact arithmetic), so
// a kinetic substep is four M-point transforms: FFT, x hs, iFFT, x K/n, conj,
// FFT, x hs, iFFT, x w, conj.  The result equals the reference's DFTs to
// rounding (complex128 <= 1e-12 after the full runs of the tests).
//
// Tables (per instance, device): w (M entries: the chirp for j < n, 0 above,
// so a product with it also zero-pads), hs (M entries), K / n per kinetic
// coefficient (M entries, 0 for k >= n), and the usual V phase tables (n
// entries).  All of them are plain complex factors multiplied with cmul.
#pragma once
#include "qsg_kernels.cuh"

namespace qsg {

struct BlueArgs {
    void *psi;              // n complex, natural order (1D) / one line per CTA (2D passes)
    const void *tw;         // stage-major twiddles of (M, E)
    const void *w;          // chirp, M entries (0 for j >= n)
    const void *hs;         // FFT_M(conj chirp) / M, M entries
    const void *vtab[2];    // V phase tables (PhaseOps form), n entries
    const void *ktab[2];    // K_k / n for k < n (0 above), M entries
    double *norm_out;       // sum |psi|^2 of the final state, or null
    double dv;              // renormalisation volume element
    uint64_t nsteps;
    int n;                  // line length
    int order, renormalize;
    int wall_n;             // InfiniteWall as the 2 wall_n odd extension (n = 2 wall_n), 0 for a
                            // periodic line: KinEn zeroes sites 0 and wall_n as the reference's
                            // wall KinEn discards them (src/SplittingMethod1D.cpp:112-114).  The
                            // steps keep the extension as it evolves (odd to rounding; the host
                            // zeroes the caller's site 0 once per uploaded state)
    int norm_n;             // sites the norm sums (the wall's n), 0: all n
};

// 1D resident evolution of one instance of any length n (2n - 1 <= M)
template <class T, int M, int E>
__global__ void __launch_bounds__(M / E) k_evolve1d_blue(BlueArgs a)
{
    using C = cplx_t<T>;
    constexpr int TL = M / E;
    constexpr int PADS = sizeof(C) == 8 ? 4 : 3;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C *>(smraw);
    const int t = threadIdx.x;
    const int n = a.n;
    C *psi = static_cast<C *>(a.psi);
    const tw_t<C> *tw = static_cast<const tw_t<C> *>(a.tw);
    const C *w = static_cast<const C *>(a.w);
    const C *hs = static_cast<const C *>(a.hs);
    const C *v0 = static_cast<const C *>(a.vtab[0]);
    const C *v1 = static_cast<const C *>(a.vtab[1]);
    const C *k0 = static_cast<const C *>(a.ktab[0]);
    const C *k1 = static_cast<const C *>(a.ktab[1]);
    const RowLayout<PADS> lay{0};
    const CtaBarrier bar{};

    C x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int j = t + e * TL;
        x[e] = j < n ? psi[j] : cmk<C>(0, 0);
    }
    // V on the n sites of the line (the slots above n are zeroed by the next chirp)
    auto apply_v = [&](const C *vt, bool twice) {
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int j = t + e * TL;
            if (j < n) {
                const C m = ld_c(vt + j);
                x[e] = PhaseOps<C>::apply(x[e], m);
                if (twice) x[e] = PhaseOps<C>::apply(x[e], m);
            }
        }
    };
    // T: forward DFT, K / n, inverse DFT (see the file comment), as four passes
    // of one transform body (a loop, not four inlined bodies: register demand):
    //   x w -> FFT -> conj(. hs) -> FFT -> . conj(K / n) -> FFT -> conj(. hs) -> FFT -> . conj(w)
    // (conj(FFT(conj z)) is the unnormalised inverse; the conjugations around the
    // kinetic product cancel into one conjugated factor)
    auto apply_t = [&](const C *kt) {
#pragma unroll 1
        for (int ph = 0; ph < 4; ++ph) {
            if (ph == 0) {
#pragma unroll
                for (int e = 0; e < E; ++e) x[e] = cmul(x[e], ld_c(w + t + e * TL));
            } else if (ph == 2) {
#pragma unroll
                for (int e = 0; e < E; ++e) x[e] = cmulc(x[e], ld_c(kt + t + e * TL));
            } else {
#pragma unroll
                for (int e = 0; e < E; ++e) x[e] = cconj(cmul(x[e], ld_c(hs + t + e * TL)));
            }
            line_fft<C, M, E, false>(x, sm, lay, bar, t, tw);
        }
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = cmulc(x[e], ld_c(w + t + e * TL));
    };
    const int nsub = a.order == 2 ? 1 : 3;
    apply_v(v0, false);
#pragma unroll 1
    for (uint64_t s = 0; s < a.nsteps; ++s) {
#pragma unroll 1
        for (int u = 0; u < nsub; ++u) {
            // O2: V1/2 T V1/2;  O4: VC1 TD1 VC2 TD2 VC2 TD1 VC1 (tables 0: C1 / D1, 1: C2 / D2)
            apply_t((a.order == 4 && u == 1) ? k1 : k0);
            const bool last = u == nsub - 1;
            apply_v((a.order == 4 && !last) ? v1 : v0, last && s + 1 < a.nsteps);
        }
    }
    double nsum = 0;
    const int nn = a.norm_n ? a.norm_n : n;
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int j = t + e * TL;
        if (j < nn) nsum += abs2d(x[e]);
    }
    if (a.norm_out || a.renormalize) {
        __shared__ double red[32];
        nsum = block_sum<TL>(nsum, red);
        if (t == 0 && a.norm_out) *a.norm_out = nsum;
        if (a.renormalize) {
            const typename RealOf<C>::type sc = (typename RealOf<C>::type)(1.0 / sqrt(nsum * a.dv));
#pragma unroll
            for (int e = 0; e < E; ++e) x[e] = cscale(x[e], sc);
        }
    }
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int j = t + e * TL;
        if (j < n) psi[j] = x[e];
    }
}

// 1D kinetic energy of any length n: one forward DFT of psi, then
// sums[0] = sum |X_k|^2 fold(k)^2 DT, sums[1] = sum |X_k|^2 over k < n
template <class T, int M, int E>
__global__ void __launch_bounds__(M / E) k_kinetic1d_blue(BlueArgs a, double dtk, double *sums)
{
    using C = cplx_t<T>;
    constexpr int TL = M / E;
    constexpr int PADS = sizeof(C) == 8 ? 4 : 3;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C *>(smraw);
    __shared__ double red[32];
    const int t = threadIdx.x;
    const int n = a.n;
    const C *psi = static_cast<const C *>(a.psi);
    const C *w = static_cast<const C *>(a.w);
    const RowLayout<PADS> lay{0};
    C x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int j = t + e * TL;
        const bool zero = j >= n || (a.wall_n && (j == 0 || j == a.wall_n));
        x[e] = zero ? cmk<C>(0, 0) : cmul(psi[j], ld_c(w + j));
    }
    // FFT -> conj(. hs) -> FFT: X_k = w_k conj(result_k), |X_k| = |result_k|
    const tw_t<C> *tw = static_cast<const tw_t<C> *>(a.tw);
    const C *hs = static_cast<const C *>(a.hs);
#pragma unroll 1
    for (int ph = 0; ph < 2; ++ph) {
        if (ph == 1) {
#pragma unroll
            for (int e = 0; e < E; ++e) x[e] = cconj(cmul(x[e], ld_c(hs + t + e * TL)));
        }
        line_fft<C, M, E, false>(x, sm, lay, CtaBarrier{}, t, tw);
    }
    double kin = 0, nn = 0;
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int k = t + e * TL;
        if (k < n) {
            const double a2 = abs2d(cmul(cconj(x[e]), ld_c(w + k)));
            const double f = (double)(k > n / 2 ? n - k : k);
            kin += a2 * f * f * dtk;
            nn += a2;
        }
    }
    kin = block_sum<TL>(kin, red);
    nn = block_sum<TL>(nn, red);
    if (t == 0) {
        sums[0] = kin;
        sums[1] = nn;
    }
}

}  // namespace qsg

namespace qsg {

// ---------------------------------------------------------------------------
// 2D grids with a side that is not a power of two (SplittingMethod2D on any
// nx x ny, src/SplittingMethod2D.cpp:81-121): the state stays in natural
// layout (index iy + ix ny); a step alternates
//   row pass:    [inverse row DFT] -> V (once, or twice at a step boundary) -> [forward row DFT]
//   column pass: forward column DFT -> K_x(kx) K_y(ky) / (nx ny) -> inverse column DFT
// so between passes the rows hold their y-spectra.  Each DFT of a side that is
// not a power of two runs through Bluestein (w / hs tables of that side); a
// power-of-two side uses the same kernels with the chirp 1 and hs the
// transform of a delta (the transform length is then twice the side).
// ---------------------------------------------------------------------------

struct Blue2DArgs {
    void *psi;
    const void *vtab;       // V phase table (PhaseOps form), nx ny entries, or null
    int vtwice;
    int in_k, out_k;        // row pass: input / output in row-spectrum form
    const void *tw;         // twiddles of (M, E) of this pass's side
    const void *w, *hs;     // Bluestein tables of this pass's side (M entries)
    const void *kx, *ky;    // column pass: kinetic factors along x (nx entries, 1/(nx ny) folded) and y
    int nx, ny;
};

// one DFT of the M-slot line x (zero above the side length): forward when
// INV is false, the unnormalised inverse otherwise (both through
// conj(FFT(conj .)) and the one forward transform body)
template <bool INV, class C, int M, int E, class Lay, class Bar, class TW>
__device__ __forceinline__ void blue_dft(C (&x)[E], C *sm, const Lay &lay, const Bar &bar, int t, const TW *tw,
                                         const C *w, const C *hs)
{
    constexpr int TL = M / E;
#pragma unroll 1
    for (int ph = 0; ph < 2; ++ph) {
        if (ph == 0) {
            // forward: x w; inverse: conj(x) w (the inverse is conj(DFT(conj x)))
#pragma unroll
            for (int e = 0; e < E; ++e) x[e] = cmul(INV ? cconj(x[e]) : x[e], ld_c(w + t + e * TL));
        } else {
#pragma unroll
            for (int e = 0; e < E; ++e) x[e] = cconj(cmul(x[e], ld_c(hs + t + e * TL)));
        }
        line_fft<C, M, E, false>(x, sm, lay, bar, t, tw);
    }
    // forward: X = w conj(y); inverse: conj(w conj(y)) = conj(w) y
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const C wk = ld_c(w + t + e * TL);
        x[e] = INV ? cmulc(x[e], wk) : cmul(cconj(x[e]), wk);
    }
}

// Row pass: RPC rows per CTA, TL = M / E threads per row.
template <class T, int M, int E, int RPC>
__global__ void __launch_bounds__(RPC *(M / E)) k_row_blue(Blue2DArgs a)
{
    using C = cplx_t<T>;
    constexpr int TL = M / E;
    constexpr int PADS = sizeof(C) == 8 ? 4 : 3;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C *>(smraw);
    const int line = threadIdx.x / TL, t = threadIdx.x - line * TL;
    const int row = blockIdx.x * RPC + line;
    const bool active = row < a.nx;
    const int ny = a.ny;
    C *psi = static_cast<C *>(a.psi) + (size_t)(active ? row : 0) * ny;
    const tw_t<C> *tw = static_cast<const tw_t<C> *>(a.tw);
    const C *w = static_cast<const C *>(a.w);
    const C *hs = static_cast<const C *>(a.hs);
    const RowLayout<PADS> lay{line * padded<M, PADS>(M)};
    const auto bar = LineBarrierOf<TL, RPC>::make(line);
    C x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int j = t + e * TL;
        x[e] = j < ny ? psi[j] : cmk<C>(0, 0);
    }
    if (a.in_k) {
        blue_dft<true, C, M, E>(x, sm, lay, bar, t, tw, w, hs);
    }
    if (a.vtab) {
        const C *vt = static_cast<const C *>(a.vtab) + (size_t)(active ? row : 0) * ny;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int j = t + e * TL;
            if (j < ny) {
                const C m = ld_c(vt + j);
                x[e] = PhaseOps<C>::apply(x[e], m);
                if (a.vtwice) x[e] = PhaseOps<C>::apply(x[e], m);
            }
        }
    }
    if (a.out_k) {
#pragma unroll
        for (int e = 0; e < E; ++e)
            if (t + e * TL >= ny) x[e] = cmk<C>(0, 0);
        blue_dft<false, C, M, E>(x, sm, lay, bar, t, tw, w, hs);
    }
    if (active) {
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int j = t + e * TL;
            if (j < ny) psi[j] = x[e];
        }
    }
}

// Column pass: W adjacent columns per CTA, TM = M / E threads per column.
template <class T, int M, int E, int W>
__global__ void __launch_bounds__(W *(M / E)) k_col_blue(Blue2DArgs a)
{
    using C = cplx_t<T>;
    constexpr int TM = M / E;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C *>(smraw);
    const int tid = threadIdx.x;
    const int c = tid % W, t = tid / W;
    const int col = blockIdx.x * W + c;
    const bool active = col < a.ny;
    const int nx = a.nx, ny = a.ny;
    C *psi = static_cast<C *>(a.psi) + (active ? col : 0);
    const tw_t<C> *tw = static_cast<const tw_t<C> *>(a.tw);
    const C *w = static_cast<const C *>(a.w);
    const C *hs = static_cast<const C *>(a.hs);
    constexpr ColPad CP = col_pad(sizeof(C), M, W);
    const ColLayout<W, CP.sh, CP.p> lay{c};
    const CtaBarrier bar{};
    C x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int i = t + e * TM;
        x[e] = i < nx ? psi[(size_t)i * ny] : cmk<C>(0, 0);
    }
    blue_dft<false, C, M, E>(x, sm, lay, bar, t, tw, w, hs);
    const C ky = ld_c(static_cast<const C *>(a.ky) + (active ? col : 0));
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int i = t + e * TM;
        x[e] = i < nx ? cmul(cmul(x[e], ld_c(static_cast<const C *>(a.kx) + i)), ky) : cmk<C>(0, 0);
    }
    blue_dft<true, C, M, E>(x, sm, lay, bar, t, tw, w, hs);
    if (active) {
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int i = t + e * TM;
            if (i < nx) psi[(size_t)i * ny] = x[e];
        }
    }
}

// Kinetic energy of a 2D grid of any sides: the rows already hold their
// y-spectra (a forward row pass); forward column DFT, then per CTA
// partials[2 cta] = sum |X|^2 (fold(kx)^2 DTx + fold(ky)^2 DTy), partials[2 cta + 1] = sum |X|^2
template <class T, int M, int E, int W>
__global__ void __launch_bounds__(W *(M / E)) k_col_blue_kinetic(Blue2DArgs a, double dtx, double dty,
                                                                  double *partials)
{
    using C = cplx_t<T>;
    constexpr int TM = M / E;
    constexpr int NT = W * TM;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C *>(smraw);
    __shared__ double red[32];
    const int tid = threadIdx.x;
    const int c = tid % W, t = tid / W;
    const int col = blockIdx.x * W + c;
    const bool active = col < a.ny;
    const int nx = a.nx, ny = a.ny;
    const C *psi = static_cast<const C *>(a.psi) + (active ? col : 0);
    constexpr ColPad CP = col_pad(sizeof(C), M, W);
    const ColLayout<W, CP.sh, CP.p> lay{c};
    C x[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int i = t + e * TM;
        x[e] = i < nx ? psi[(size_t)i * ny] : cmk<C>(0, 0);
    }
    blue_dft<false, C, M, E>(x, sm, lay, CtaBarrier{}, t, static_cast<const tw_t<C> *>(a.tw),
                             static_cast<const C *>(a.w), static_cast<const C *>(a.hs));
    double kin = 0, nn = 0;
    const double fy = (double)(col > ny / 2 ? ny - col : col);
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int i = t + e * TM;
        if (active && i < nx) {
            const double a2 = abs2d(x[e]);
            const double fx = (double)(i > nx / 2 ? nx - i : i);
            kin += a2 * ((fx * fx) * dtx + (fy * fy) * dty);
            nn += a2;
        }
    }
    kin = block_sum<NT>(kin, red);
    nn = block_sum<NT>(nn, red);
    if (tid == 0) {
        partials[2 * blockIdx.x] = kin;
        partials[2 * blockIdx.x + 1] = nn;
    }
}

}  // namespace qsg
