// qsg_fft.cuh -- register/shared-memory Stockham FFT building blocks for sm_103a.
//
// A "line" is one 1D transform of length L (a power of two).  Each thread of a
// line owns E elements (E a power of two, E <= L): at entry and exit of a
// transform, register slot e of thread t holds element t + e*(L/E) of the line
// (natural order), so an FFT, a pointwise multiply and an inverse FFT chain in
// registers with no reordering.  Between radix stages the data goes through
// shared memory once (Stockham autosort: every stage reads element t + e*L/E
// and writes a permuted position, so no bit reversal pass is ever needed).
//
// Transform definitions follow the reference (src/FourierTransform.h:16-20):
// forward X_k = sum_n x_n exp(-2 pi i k n / L), inverse unnormalised with the
// + sign.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace qsg {

template <class T> struct CplxOf;
template <> struct CplxOf<float> { using type = float2; };
template <> struct CplxOf<double> { using type = double2; };
template <class T> using cplx_t = typename CplxOf<T>::type;

template <class C> struct RealOf;
template <> struct RealOf<float2> { using type = float; };
template <> struct RealOf<double2> { using type = double; };

template <class C>
__device__ __forceinline__ C cmk(typename RealOf<C>::type x, typename RealOf<C>::type y)
{
    C r;
    r.x = x;
    r.y = y;
    return r;
}

// Packed FP32 pairs (the f32x2 arithmetic of sm_100 and later): one
// instruction computes both lanes, each lane rounded exactly as the scalar
// operation, so a complex64 add or a pair of FMAs issues once instead of twice.
// Every packed helper below rounds exactly as the scalar code it replaces (same
// products rounded, same FMAs), so results do not depend on the choice.  The
// pairs must sit in aligned register pairs, which raises register demand: a
// translation unit opts in with QSG_PACKED_F32 (defined before this header)
// where its kernels have the registers to spare (measured per kernel).
#ifdef QSG_PACKED_F32
inline constexpr bool kPackedF32 = true;
#else
inline constexpr bool kPackedF32 = false;
#endif
namespace pk {
__device__ __forceinline__ unsigned long long b64(float2 a)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
    return r;
}
__device__ __forceinline__ float2 f2(unsigned long long v)
{
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}
__device__ __forceinline__ float2 add(float2 a, float2 b)
{
    unsigned long long r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(b64(a)), "l"(b64(b)));
    return f2(r);
}
__device__ __forceinline__ float2 sub(float2 a, float2 b)
{
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(b64(a)), "l"(b64(b)));
    return f2(r);
}
__device__ __forceinline__ float2 mul(float2 a, float2 b)
{
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(b64(a)), "l"(b64(b)));
    return f2(r);
}
// a * b + c, one rounding per lane
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c)
{
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(b64(a)), "l"(b64(b)), "l"(b64(c)));
    return f2(r);
}
__device__ __forceinline__ float2 swap(float2 a) { return float2{a.y, a.x}; }
__device__ __forceinline__ float2 bc(float v) { return float2{v, v}; }
}  // namespace pk

template <class C> __device__ __forceinline__ C cadd(C a, C b) { return cmk<C>(a.x + b.x, a.y + b.y); }
template <class C> __device__ __forceinline__ C csub(C a, C b) { return cmk<C>(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cadd(float2 a, float2 b)
{
    if constexpr (kPackedF32) return pk::add(a, b);
    return float2{a.x + b.x, a.y + b.y};
}
__device__ __forceinline__ float2 csub(float2 a, float2 b)
{
    if constexpr (kPackedF32) return pk::sub(a, b);
    return float2{a.x - b.x, a.y - b.y};
}
template <class C> __device__ __forceinline__ C cmul(C a, C b)
{
    return cmk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <class C> __device__ __forceinline__ C cmulc(C a, C b)  // a * conj(b)
{
    return cmk<C>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <class C> __device__ __forceinline__ C cscale(C a, typename RealOf<C>::type s)
{
    return cmk<C>(a.x * s, a.y * s);
}
// multiply by w or conj(w): forward transforms use the table value w = exp(-i th),
// inverse transforms its conjugate
template <bool INV, class C> __device__ __forceinline__ C cmulw(C a, C w)
{
    return INV ? cmulc(a, w) : cmul(a, w);
}
// a * (1 + m) for m stored as (cos th - 1, sin th): the "phase minus one"
// representation used by the complex64 tables, which keeps the systematic
// rounding of a unit-modulus factor proportional to |th| instead of to 1.
// The correction a*m is formed completely before it is added to a, so the one
// rounding of the sum is unbiased.  Chaining a + a.x*m.x after a - a.y*m.y
// instead drops a.x*m.x (~ -a.x th^2/2) whenever it is below half an ulp of
// a.x, i.e. for |th| below ~2e-4: every such multiply then grows |a|^2 by
// th^2, coherently, step after step (measured: 2.5e-5 norm drift over 1000 O4
// steps at 1024^2, 3.0e-5 with the packet at k = 0).
template <class C> __device__ __forceinline__ C cmul1p(C a, C m)
{
    const auto cx = fma(a.x, m.x, -(a.y * m.y));
    const auto cy = fma(a.y, m.x, a.x * m.y);
    return cmk<C>(a.x + cx, a.y + cy);
}
// packed: (-(a.y m.y), a.x m.y), then the FMAs with m.x, then a + c
__device__ __forceinline__ float2 cmul1p(float2 a, float2 m)
{
    if constexpr (!kPackedF32) {
        const float cx = fmaf(a.x, m.x, -(a.y * m.y)), cy = fmaf(a.y, m.x, a.x * m.y);
        return float2{a.x + cx, a.y + cy};
    }
    const float2 t = pk::mul(pk::swap(a), float2{-m.y, m.y});
    return pk::add(a, pk::fma(a, pk::bc(m.x), t));
}
// multiply by -i (forward) or +i (inverse)
template <bool INV, class C> __device__ __forceinline__ C crot(C a)
{
    return INV ? cmk<C>(-a.y, a.x) : cmk<C>(a.y, -a.x);
}

// ---------------------------------------------------------------------------
// Small DFTs on register arrays (natural order in, natural order out).
// ---------------------------------------------------------------------------

template <bool INV, class C> __device__ __forceinline__ void dft2(C &a0, C &a1)
{
    C t = a0;
    a0 = cadd(t, a1);
    a1 = csub(t, a1);
}

template <bool INV, class C> __device__ __forceinline__ void dft4(C &a0, C &a1, C &a2, C &a3)
{
    C s02 = cadd(a0, a2), d02 = csub(a0, a2);
    C s13 = cadd(a1, a3);
    if constexpr (std::is_same<C, float2>::value && kPackedF32) {
        // d02 -+ i (a1 - a3): the difference's lanes swapped, its signs applied by
        // FMAs with +-1 (exact, so the sums round as the scalar adds do)
        const float2 d13s = pk::swap(csub(a1, a3));
        const float2 k = INV ? float2{-1.f, 1.f} : float2{1.f, -1.f};
        a0 = cadd(s02, s13);
        a2 = csub(s02, s13);
        a1 = pk::fma(d13s, k, d02);
        a3 = pk::fma(d13s, float2{-k.x, -k.y}, d02);
    } else {
        C d13 = crot<INV>(csub(a1, a3));
        a0 = cadd(s02, s13);
        a2 = csub(s02, s13);
        a1 = cadd(d02, d13);
        a3 = csub(d02, d13);
    }
}

// ---------------------------------------------------------------------------
// Multiplication by the fixed roots of unity inside the radix-8/16 butterflies.
//
// complex128 uses the constants rounded once.  In complex64 the same constant
// is applied in every transform of every step, so any error of the constant
// itself compounds coherently; the complex64 rotations below use hi + lo
// constants (see Roots<float2>), leaving rounding of the data.
// ---------------------------------------------------------------------------

template <class C> struct Roots;
template <> struct Roots<double2> {
    // a * exp(-+ i th), (c, s) = (cos th, sin th)
    template <bool INV> static __device__ __forceinline__ double2 cs(double2 a, double c, double s)
    {
        return INV ? cmk<double2>(a.x * c - a.y * s, a.y * c + a.x * s)
                   : cmk<double2>(a.x * c + a.y * s, a.y * c - a.x * s);
    }
    static constexpr double C1 = 0.92387953251128675613, S1 = 0.38268343236508977173;
    static constexpr double H = 0.70710678118654752440;
    template <bool INV> static __device__ __forceinline__ double2 w16_1(double2 a) { return cs<INV>(a, C1, S1); }
    template <bool INV> static __device__ __forceinline__ double2 w16_3(double2 a) { return cs<INV>(a, S1, C1); }
    template <bool INV> static __device__ __forceinline__ double2 w16_9(double2 a) { return cs<INV>(a, -C1, -S1); }
    // exp(-+ i pi/4), exp(-+ 3 i pi/4)
    template <bool INV> static __device__ __forceinline__ double2 w8_1(double2 a)
    {
        return INV ? cmk<double2>((a.x - a.y) * H, (a.x + a.y) * H) : cmk<double2>((a.x + a.y) * H, (a.y - a.x) * H);
    }
    template <bool INV> static __device__ __forceinline__ double2 w8_3(double2 a)
    {
        return INV ? cmk<double2>(-(a.x + a.y) * H, (a.x - a.y) * H) : cmk<double2>((a.y - a.x) * H, -(a.x + a.y) * H);
    }
    // exp(-+ i r pi/16), r = 1, 3, 5, 7 (radix 32)
    static constexpr double C16 = 0.98078528040323044913, S16 = 0.19509032201612826785;
    static constexpr double C316 = 0.83146961230254523708, S316 = 0.55557023301960222474;
    template <bool INV> static __device__ __forceinline__ double2 w32_1(double2 a) { return cs<INV>(a, C16, S16); }
    template <bool INV> static __device__ __forceinline__ double2 w32_3(double2 a) { return cs<INV>(a, C316, S316); }
    template <bool INV> static __device__ __forceinline__ double2 w32_5(double2 a) { return cs<INV>(a, S316, C316); }
    template <bool INV> static __device__ __forceinline__ double2 w32_7(double2 a) { return cs<INV>(a, S16, C16); }
};
template <> struct Roots<float2> {
    // complex64: every fixed rotation multiplies by (cos th, sin th) given as
    // hi + lo float pairs (lo = float(c - hi)), as the table twiddles are.  The
    // rotation is then unitary to ~1e-14, so the inverse transform (conjugate
    // constants) undoes the forward one to rounding.  Both cheaper forms leave
    // a fixed operator error that every step repeats, so it adds up linearly:
    // - plain float constants are off the unit circle by ~3e-8;
    // - three-shear rotations (determinant exactly 1) are not orthogonal, so
    //   conj(FFT(conj(FFT x))) != N x by ~1e-8.
    // Measured at 1024^2 with dt = 0 over 1000 O4 steps (pure round trips):
    // shears gave relative L2 6.3e-5, hi + lo pairs 1.2e-5.
    static constexpr float C1H = 0x1.d906bcp-1f, C1L = 0x1.e651a8p-26f;  // cos(pi/8)
    static constexpr float S1H = 0x1.87de2ap-2f, S1L = 0x1.abaa58p-28f;  // sin(pi/8)
    static constexpr float HH = 0x1.6a09e6p-1f, HL = 0x1.9fcef4p-27f;    // 1/sqrt(2)
    // a * exp(-+ i th), th given by (cos th, sin th) = (ch + cl, sh + sl)
    // (scalar: the constants are instruction immediates; packed pairs of them
    // would each take a register pair, and the radix-32 passes then spill)
    template <bool INV>
    static __device__ __forceinline__ float2 cs(float2 a, float ch, float cl, float sh, float sl)
    {
        if (INV) {
            const float lx = fmaf(a.x, cl, -a.y * sl), ly = fmaf(a.y, cl, a.x * sl);
            return cmk<float2>(fmaf(a.x, ch, fmaf(-a.y, sh, lx)), fmaf(a.y, ch, fmaf(a.x, sh, ly)));
        }
        const float lx = fmaf(a.x, cl, a.y * sl), ly = fmaf(a.y, cl, -a.x * sl);
        return cmk<float2>(fmaf(a.x, ch, fmaf(a.y, sh, lx)), fmaf(a.y, ch, fmaf(-a.x, sh, ly)));
    }
    template <bool INV> static __device__ __forceinline__ float2 w16_1(float2 a)
    {
        return cs<INV>(a, C1H, C1L, S1H, S1L);
    }
    template <bool INV> static __device__ __forceinline__ float2 w16_3(float2 a)
    {
        return cs<INV>(a, S1H, S1L, C1H, C1L);
    }
    template <bool INV> static __device__ __forceinline__ float2 w16_9(float2 a)
    {
        return cs<INV>(cmk<float2>(-a.x, -a.y), C1H, C1L, S1H, S1L);
    }
    // exp(-+ i pi/4) = (1 -+ i) / sqrt(2)
    template <bool INV> static __device__ __forceinline__ float2 w8_1(float2 a)
    {
        if constexpr (!kPackedF32) {
            const float u = INV ? a.x - a.y : a.x + a.y, v = INV ? a.x + a.y : a.y - a.x;
            return cmk<float2>(fmaf(u, HH, u * HL), fmaf(v, HH, v * HL));
        }
        // (u, v) = forward (a.x + a.y, a.y - a.x), inverse (a.x - a.y, a.x + a.y)
        const float2 uv = pk::fma(pk::swap(a), INV ? float2{-1.f, 1.f} : float2{1.f, -1.f}, a);
        return pk::fma(uv, pk::bc(HH), pk::mul(uv, pk::bc(HL)));
    }
    // exp(-+ 3 i pi/4) = exp(-+ i pi/4) * (-+ i)
    template <bool INV> static __device__ __forceinline__ float2 w8_3(float2 a) { return w8_1<INV>(crot<INV>(a)); }
    // exp(-+ i r pi/16), r = 1, 3, 5, 7 (radix 32)
    static constexpr float C16H = 0x1.f6297cp-1f, C16L = 0x1.feeb96p-26f;    // cos(pi/16)
    static constexpr float S16H = 0x1.8f8b84p-3f, S16L = -0x1.cb2cfcp-30f;   // sin(pi/16)
    static constexpr float C316H = 0x1.a9b662p-1f, C316L = 0x1.21d434p-26f;  // cos(3pi/16)
    static constexpr float S316H = 0x1.1c73b4p-1f, S316L = -0x1.9465cep-27f; // sin(3pi/16)
    template <bool INV> static __device__ __forceinline__ float2 w32_1(float2 a)
    {
        return cs<INV>(a, C16H, C16L, S16H, S16L);
    }
    template <bool INV> static __device__ __forceinline__ float2 w32_3(float2 a)
    {
        return cs<INV>(a, C316H, C316L, S316H, S316L);
    }
    template <bool INV> static __device__ __forceinline__ float2 w32_5(float2 a)
    {
        return cs<INV>(a, S316H, S316L, C316H, C316L);
    }
    template <bool INV> static __device__ __forceinline__ float2 w32_7(float2 a)
    {
        return cs<INV>(a, S16H, S16L, C16H, C16L);
    }
};

// complex64 with plain float constants (each root rounded once).  Used by
// the transforms of the complex64 2D momentum form only: there the transforms
// carry increments (V - 1) psi or feed only such increments, so the fixed
// operator error of plain constants is scaled by |V - 1| as their rounding is
// (a CPU emulation of the FP32 arithmetic: plain constants raise the direct
// form's error 5.7x and leave the momentum form's unchanged).
struct RootsPlain32 {
    // scalar, as Roots<float2>::cs: its constants stay instruction immediates
    template <bool INV> static __device__ __forceinline__ float2 cs(float2 a, float c, float s)
    {
        return INV ? cmk<float2>(fmaf(a.x, c, -a.y * s), fmaf(a.y, c, a.x * s))
                   : cmk<float2>(fmaf(a.x, c, a.y * s), fmaf(a.y, c, -a.x * s));
    }
    static constexpr float C1 = 0x1.d906bcp-1f, S1 = 0x1.87de2ap-2f;      // cos, sin (pi/8)
    static constexpr float H = 0x1.6a09e6p-1f;                             // 1/sqrt(2)
    static constexpr float C16 = 0x1.f6297cp-1f, S16 = 0x1.8f8b84p-3f;    // cos, sin (pi/16)
    static constexpr float C316 = 0x1.a9b662p-1f, S316 = 0x1.1c73b4p-1f;  // cos, sin (3pi/16)
    template <bool INV> static __device__ __forceinline__ float2 w16_1(float2 a) { return cs<INV>(a, C1, S1); }
    template <bool INV> static __device__ __forceinline__ float2 w16_3(float2 a) { return cs<INV>(a, S1, C1); }
    template <bool INV> static __device__ __forceinline__ float2 w16_9(float2 a)
    {
        return cs<INV>(cmk<float2>(-a.x, -a.y), C1, S1);
    }
    template <bool INV> static __device__ __forceinline__ float2 w8_1(float2 a)
    {
        if constexpr (!kPackedF32) {
            const float u = INV ? a.x - a.y : a.x + a.y, v = INV ? a.x + a.y : a.y - a.x;
            return cmk<float2>(u * H, v * H);
        }
        const float2 uv = pk::fma(pk::swap(a), INV ? float2{-1.f, 1.f} : float2{1.f, -1.f}, a);
        return pk::mul(uv, pk::bc(H));
    }
    template <bool INV> static __device__ __forceinline__ float2 w8_3(float2 a) { return w8_1<INV>(crot<INV>(a)); }
    template <bool INV> static __device__ __forceinline__ float2 w32_1(float2 a) { return cs<INV>(a, C16, S16); }
    template <bool INV> static __device__ __forceinline__ float2 w32_3(float2 a) { return cs<INV>(a, C316, S316); }
    template <bool INV> static __device__ __forceinline__ float2 w32_5(float2 a) { return cs<INV>(a, S316, C316); }
    template <bool INV> static __device__ __forceinline__ float2 w32_7(float2 a) { return cs<INV>(a, S16, C16); }
};

// Table twiddles: complex128 tables hold the factor; complex64 tables hold
// float4 {hi.x, hi.y, lo.x, lo.y}, the factor as an unevaluated sum of two
// float pairs (lo = float(w - hi)), multiplied in by both so the product is
// as accurate as with an exact twiddle (same coherent-modulus reason as above).
// A complex64 transform given a float2 table (the factor rounded once) runs
// with plain twiddles and plain constants (RootsPlain32).
template <class C> struct TwOf;
template <> struct TwOf<double2> { using type = double2; };
template <> struct TwOf<float2> { using type = float4; };
template <class C> using tw_t = typename TwOf<C>::type;

// the fixed roots that go with a twiddle table type
template <class C, class TW> struct RootsOf { using type = Roots<C>; };
template <> struct RootsOf<float2, float2> { using type = RootsPlain32; };

// a * exp(-+ 2 pi i M / 32) for a compile-time M: the r pi/16 rotation of
// M mod 8, then (M / 8) quarter turns
template <int M, bool INV, class C, class TW = tw_t<C>> __device__ __forceinline__ C rot32(C a)
{
    using RT = typename RootsOf<C, TW>::type;
    constexpr int r = M % 8, q = (M / 8) % 4;
    if constexpr (r == 1) a = RT::template w32_1<INV>(a);
    if constexpr (r == 2) a = RT::template w16_1<INV>(a);
    if constexpr (r == 3) a = RT::template w32_3<INV>(a);
    if constexpr (r == 4) a = RT::template w8_1<INV>(a);
    if constexpr (r == 5) a = RT::template w32_5<INV>(a);
    if constexpr (r == 6) a = RT::template w16_3<INV>(a);
    if constexpr (r == 7) a = RT::template w32_7<INV>(a);
    if constexpr (q >= 1) a = crot<INV>(a);
    if constexpr (q >= 2) a = crot<INV>(a);
    if constexpr (q >= 3) a = crot<INV>(a);
    return a;
}

template <bool INV> __device__ __forceinline__ double2 twmul(double2 a, double2 w) { return cmulw<INV>(a, w); }
// plain complex64 product with its FMAs spelt out, so that every kernel rounds
// it the same way (left to contraction, the fused product can differ between
// instantiations)
template <bool INV> __device__ __forceinline__ float2 cmulw_f(float2 a, float2 w)
{
    if constexpr (!kPackedF32) {
        if (INV) return cmk<float2>(fmaf(a.x, w.x, a.y * w.y), fmaf(a.y, w.x, -(a.x * w.y)));
        return cmk<float2>(fmaf(a.x, w.x, -(a.y * w.y)), fmaf(a.x, w.y, a.y * w.x));
    }
    // forward (fma(a.x, w.x, -(a.y w.y)), fma(a.x, w.y, a.y w.x)),
    // inverse (fma(a.x, w.x, a.y w.y), fma(a.y, w.x, -(a.x w.y)))
    if (INV) return pk::fma(a, pk::bc(w.x), pk::mul(pk::swap(a), float2{w.y, -w.y}));
    return pk::fma(pk::bc(a.x), w, pk::mul(pk::bc(a.y), float2{-w.y, w.x}));
}
template <bool INV> __device__ __forceinline__ float2 twmul(float2 a, float2 w) { return cmulw_f<INV>(a, w); }
template <bool INV> __device__ __forceinline__ float2 twmul(float2 a, float4 w)
{
    if constexpr (!kPackedF32) {
        if (INV) {  // a * conj(w)
            const float lx = fmaf(a.x, w.z, a.y * w.w), ly = fmaf(a.y, w.z, -a.x * w.w);
            return cmk<float2>(fmaf(a.x, w.x, fmaf(a.y, w.y, lx)), fmaf(a.y, w.x, fmaf(-a.x, w.y, ly)));
        }
        const float lx = fmaf(a.x, w.z, -a.y * w.w), ly = fmaf(a.x, w.w, a.y * w.z);
        return cmk<float2>(fmaf(a.x, w.x, fmaf(-a.y, w.y, lx)), fmaf(a.x, w.y, fmaf(a.y, w.x, ly)));
    }
    if (INV) {  // a * conj(w): lanes (a.x wx + a.y wy, a.y wx - a.x wy), lo parts (z, w) first
        const float2 sa = pk::swap(a);
        const float2 l = pk::fma(a, pk::bc(w.z), pk::mul(sa, float2{w.w, -w.w}));
        return pk::fma(a, pk::bc(w.x), pk::fma(sa, float2{w.y, -w.y}, l));
    }
    // lanes (a.x wx - a.y wy, a.x wy + a.y wx)
    const float2 ax = pk::bc(a.x), ay = pk::bc(a.y);
    const float2 l = pk::fma(ax, float2{w.z, w.w}, pk::mul(ay, float2{-w.w, w.z}));
    return pk::fma(ax, float2{w.x, w.y}, pk::fma(ay, float2{-w.y, w.x}, l));
}

template <bool INV, class C, class TW = tw_t<C>> __device__ __forceinline__ void dft8(C (&v)[8])
{
    using RT = typename RootsOf<C, TW>::type;
    // even / odd halves, then combine with w8^k
    dft4<INV>(v[0], v[2], v[4], v[6]);
    dft4<INV>(v[1], v[3], v[5], v[7]);
    C o1 = RT::template w8_1<INV>(v[3]), o2 = crot<INV>(v[5]), o3 = RT::template w8_3<INV>(v[7]);
    C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    v[0] = cadd(e0, v[1]);
    v[4] = csub(e0, v[1]);
    v[1] = cadd(e1, o1);
    v[5] = csub(e1, o1);
    v[2] = cadd(e2, o2);
    v[6] = csub(e2, o2);
    v[3] = cadd(e3, o3);
    v[7] = csub(e3, o3);
}

template <bool INV, class C, class TW = tw_t<C>> __device__ __forceinline__ void dft16(C (&v)[16])
{
    using RT = typename RootsOf<C, TW>::type;
    // n = 4 n1 + n2; first DFT4 over n1 for each n2
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) dft4<INV>(v[n2], v[4 + n2], v[8 + n2], v[12 + n2]);
    // v[4 k1 + n2] now holds z[n2][k1]; twiddle w16^(n2 k1)
    v[5] = RT::template w16_1<INV>(v[5]);    // n2=1,k1=1: w^1
    v[6] = RT::template w8_1<INV>(v[6]);     // n2=2,k1=1: w^2
    v[7] = RT::template w16_3<INV>(v[7]);    // n2=3,k1=1: w^3
    v[9] = RT::template w8_1<INV>(v[9]);     // n2=1,k1=2: w^2
    v[10] = crot<INV>(v[10]);                // n2=2,k1=2: w^4
    v[11] = RT::template w8_3<INV>(v[11]);   // n2=3,k1=2: w^6
    v[13] = RT::template w16_3<INV>(v[13]);  // n2=1,k1=3: w^3
    v[14] = RT::template w8_3<INV>(v[14]);   // n2=2,k1=3: w^6
    v[15] = RT::template w16_9<INV>(v[15]);  // n2=3,k1=3: w^9 = -w^1
    // second DFT4 over n2 for each k1: output k = k1 + 4 k2
    C r[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
        C a0 = v[4 * k1], a1 = v[4 * k1 + 1], a2 = v[4 * k1 + 2], a3 = v[4 * k1 + 3];
        dft4<INV>(a0, a1, a2, a3);
        r[k1] = a0;
        r[k1 + 4] = a1;
        r[k1 + 8] = a2;
        r[k1 + 12] = a3;
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = r[i];
}

// n = 8 n1 + n2: DFT4 over n1, twiddle w32^(n2 k1), DFT8 over n2; output k = k1 + 4 k2
template <bool INV, class C, class TW = tw_t<C>> __device__ __forceinline__ void dft32(C (&v)[32])
{
#pragma unroll
    for (int n2 = 0; n2 < 8; ++n2) dft4<INV>(v[n2], v[8 + n2], v[16 + n2], v[24 + n2]);
    // v[8 k1 + n2] = z[n2][k1]
    v[9] = rot32<1, INV, C, TW>(v[9]);
    v[10] = rot32<2, INV, C, TW>(v[10]);
    v[11] = rot32<3, INV, C, TW>(v[11]);
    v[12] = rot32<4, INV, C, TW>(v[12]);
    v[13] = rot32<5, INV, C, TW>(v[13]);
    v[14] = rot32<6, INV, C, TW>(v[14]);
    v[15] = rot32<7, INV, C, TW>(v[15]);
    v[17] = rot32<2, INV, C, TW>(v[17]);
    v[18] = rot32<4, INV, C, TW>(v[18]);
    v[19] = rot32<6, INV, C, TW>(v[19]);
    v[20] = rot32<8, INV, C, TW>(v[20]);
    v[21] = rot32<10, INV, C, TW>(v[21]);
    v[22] = rot32<12, INV, C, TW>(v[22]);
    v[23] = rot32<14, INV, C, TW>(v[23]);
    v[25] = rot32<3, INV, C, TW>(v[25]);
    v[26] = rot32<6, INV, C, TW>(v[26]);
    v[27] = rot32<9, INV, C, TW>(v[27]);
    v[28] = rot32<12, INV, C, TW>(v[28]);
    v[29] = rot32<15, INV, C, TW>(v[29]);
    v[30] = rot32<18, INV, C, TW>(v[30]);
    v[31] = rot32<21, INV, C, TW>(v[31]);
    C r[32];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
        C u[8];
#pragma unroll
        for (int n2 = 0; n2 < 8; ++n2) u[n2] = v[8 * k1 + n2];
        dft8<INV, C, TW>(u);
#pragma unroll
        for (int k2 = 0; k2 < 8; ++k2) r[k1 + 4 * k2] = u[k2];
    }
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = r[i];
}

template <int R, bool INV, class C, class TW = tw_t<C>> __device__ __forceinline__ void dft(C (&v)[R])
{
    if constexpr (R == 2) {
        dft2<INV>(v[0], v[1]);
    } else if constexpr (R == 4) {
        dft4<INV>(v[0], v[1], v[2], v[3]);
    } else if constexpr (R == 8) {
        dft8<INV, C, TW>(v);
    } else if constexpr (R == 16) {
        dft16<INV, C, TW>(v);
    } else if constexpr (R == 32) {
        dft32<INV, C, TW>(v);
    } else {
        static_assert(R == 1, "radix must be 1, 2, 4, 8, 16 or 32");
    }
}

// ---------------------------------------------------------------------------
// Radix plan for a line of length L with E elements per thread.
// Stage 0 has radix 2^(log L - (S-1) log E) (the remainder), every later stage
// radix E.  p_s = product of the radices before stage s.
// ---------------------------------------------------------------------------

__host__ __device__ constexpr int ilog2(int v) { return v <= 1 ? 0 : 1 + ilog2(v >> 1); }

template <int L, int E> struct Plan {
    static_assert((L & (L - 1)) == 0 && (E & (E - 1)) == 0, "powers of two only");
    static_assert(E >= 2 && E <= 32 && E <= L, "2 <= E <= 32, E <= L");
    static constexpr int LOGL = ilog2(L);
    static constexpr int LOGE = ilog2(E);
    static constexpr int NST = (LOGL + LOGE - 1) / LOGE;
    static constexpr int LOGR0 = LOGL - (NST - 1) * LOGE;
    static constexpr int TL = L / E;  // threads per line
    __host__ __device__ static constexpr int radix_log(int s) { return s == 0 ? LOGR0 : LOGE; }
    __host__ __device__ static constexpr int p_log(int s) { return s == 0 ? 0 : LOGR0 + (s - 1) * LOGE; }
    // offset of stage s in the stage-major twiddle table; stage s holds
    // (R_s - 1) * p_s entries tw[(q-1)*p_s + k] = exp(-2 pi i q k / (p_s R_s))
    __host__ __device__ static constexpr int tw_offset(int s)
    {
        return s <= 1 ? 0 : tw_offset(s - 1) + ((1 << radix_log(s - 1)) - 1) * (1 << p_log(s - 1));
    }
    static constexpr int TW_SIZE = tw_offset(NST);
};

// One Stockham stage: butterflies on the register slots, twiddles from the
// stage-major table, then (unless this is the last stage) scatter to shared
// memory and gather the next stage's inputs.
//
//   lay(n)  -> shared-memory element index of line element n (this line)
//   bar()   -> barrier over every thread that shares the buffer
template <class C, int L, int E, bool INV, int S, class Lay, class Bar, class TW>
__device__ __forceinline__ void fft_stage(C (&x)[E], C *sm, const Lay &lay, const Bar &bar, int t,
                                          const TW *__restrict__ tw)
{
    using P = Plan<L, E>;
    constexpr int RL = P::radix_log(S);
    constexpr int R = 1 << RL;
    constexpr int PL = P::p_log(S);
    constexpr int PP = 1 << PL;
    constexpr int J = E / R;  // butterflies per thread in this stage
    constexpr int TL = P::TL;
    constexpr int TWO = P::tw_offset(S);
#pragma unroll
    for (int j = 0; j < J; ++j) {
        C v[R];
#pragma unroll
        for (int q = 0; q < R; ++q) v[q] = x[j + q * J];
        if constexpr (PP > 1) {
            const int k = (t + j * TL) & (PP - 1);
#pragma unroll
            for (int q = 1; q < R; ++q) v[q] = twmul<INV>(v[q], __ldg(&tw[TWO + (q - 1) * PP + k]));
        }
        dft<R, INV, C, TW>(v);
#pragma unroll
        for (int q = 0; q < R; ++q) x[j + q * J] = v[q];
    }
    if constexpr (S + 1 < P::NST) {
        bar();  // every reader of the previous stage is done with the buffer
#pragma unroll
        for (int j = 0; j < J; ++j) {
            const int b = t + j * TL;
            const int k = b & (PP - 1);
            const int o = ((b - k) << RL) + k;
#pragma unroll
            for (int q = 0; q < R; ++q) sm[lay(o + q * PP)] = x[j + q * J];
        }
        bar();
#pragma unroll
        for (int e = 0; e < E; ++e) x[e] = sm[lay(t + e * TL)];
    }
}

template <class C, int L, int E, bool INV, int S, class Lay, class Bar, class TW>
__device__ __forceinline__ void fft_stages(C (&x)[E], C *sm, const Lay &lay, const Bar &bar, int t,
                                           const TW *__restrict__ tw)
{
    if constexpr (S < Plan<L, E>::NST) {
        fft_stage<C, L, E, INV, S>(x, sm, lay, bar, t, tw);
        fft_stages<C, L, E, INV, S + 1>(x, sm, lay, bar, t, tw);
    }
}

// A copy of p the compiler cannot prove equal to p.  A forward and an inverse
// transform read the same twiddle entries; without this the compiler keeps the
// first transform's twiddles live in registers for the second (dozens of
// registers, spills), where reloading them from L1 is nearly free.
template <class P> __device__ __forceinline__ const P *opaque(const P *p)
{
    const P *r;
    asm volatile("mov.b64 %0, %1;" : "=l"(r) : "l"(p));
    return r;
}

// Full transform of one line held in registers (natural order in and out).
// The table's type picks the twiddle arithmetic (tw_t<C>, or float2: plain).
template <class C, int L, int E, bool INV, class Lay, class Bar, class TW>
__device__ __forceinline__ void line_fft(C (&x)[E], C *sm, const Lay &lay, const Bar &bar, int t,
                                         const TW *__restrict__ tw)
{
    fft_stages<C, L, E, INV, 0>(x, sm, lay, bar, t, opaque(tw));
}

// Shared-memory index maps.  PADSHIFT adds one element of padding every
// 2^PADSHIFT elements, which breaks the power-of-two strides of the Stockham
// scatter across banks.
template <int PADSHIFT> struct RowLayout {
    int base;
    __device__ __forceinline__ int operator()(int n) const { return base + n + (n >> PADSHIFT); }
};
// column tile: element n of column c at n*W + c + (n >> SH)*P.  The pad is a
// function of the row index only, so every address of a thread is a base plus
// compile-time offsets (no per-element index arithmetic held in registers).
// (SH, P) per shape come from col_pad(), chosen by a bank-conflict model of
// the Stockham gather / scatter patterns.
template <int W, int SH, int P> struct ColLayout {
    int c;
    __device__ __forceinline__ int operator()(int n) const { return n * W + c + (n >> SH) * P; }
};
struct ColPad {
    int sh, p;
};
__host__ __device__ constexpr ColPad col_pad(int esize, int m, int w, int e = 16)
{
    // radix 32 (one exchange): thread t writes rows 32t + q, so rows 32 apart
    // must land in different halves of the banks
    if (e == 32) return ColPad{5, 8};
    if (esize == 8) {
        if (w >= 16) return ColPad{0, 1};
        if (m <= 128) return ColPad{1, 2};
        if (m >= 1024) return ColPad{1, 4};
        return ColPad{1, 1};
    }
    if (w >= 8) return ColPad{0, 1};
    if (w == 4) return m <= 128 ? ColPad{1, 4} : m == 256 ? ColPad{1, 2} : m == 512 ? ColPad{1, 1} : ColPad{1, 4};
    return (m == 256 || m >= 2048) ? ColPad{2, 2} : ColPad{2, 1};
}
// elements of shared memory a column tile needs
__host__ __device__ constexpr int col_tile_elems(int esize, int m, int w, int e = 16)
{
    return m * w + (m >> col_pad(esize, m, w, e).sh) * col_pad(esize, m, w, e).p;
}

template <int L, int PADSHIFT> __host__ __device__ constexpr int padded(int n) { return n + (n >> PADSHIFT); }

struct CtaBarrier {
    __device__ __forceinline__ void operator()() const { __syncthreads(); }
};
// named barrier over the NT threads [id*NT, (id+1)*NT) of one line group
struct NamedBarrier {
    int id, nthreads;
    __device__ __forceinline__ void operator()() const
    {
        asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
    }
};
// a line held by the lanes of one warp (2..32 consecutive lanes): __syncwarp
// on those lanes orders their shared-memory accesses
struct WarpLineBarrier {
    unsigned mask;
    __device__ __forceinline__ void operator()() const { __syncwarp(mask); }
};

// The barrier of one line of TL threads in a CTA of NL lines (line l holds
// threads [l*TL, (l+1)*TL)): __syncwarp when lines are parts of one warp, a
// named barrier per line when lines are whole warps (at most 15 of them),
// otherwise the CTA barrier.
template <int TL, int NL> struct LineBarrierOf {
    static constexpr bool WARP = TL > 1 && TL <= 32 && NL > 1;
    static constexpr bool NAMED = !WARP && (TL % 32 == 0) && NL <= 15 && NL > 1;
    using type = typename std::conditional<
        WARP, WarpLineBarrier, typename std::conditional<NAMED, NamedBarrier, CtaBarrier>::type>::type;
    static __device__ __forceinline__ type make(int line)
    {
        type b;
        if constexpr (WARP) b = WarpLineBarrier{(TL == 32 ? 0xffffffffu : ((1u << TL) - 1u)) << ((line * TL) & 31)};
        if constexpr (NAMED) b = NamedBarrier{1 + line, TL};
        return b;
    }
};

}  // namespace qsg
