/*
 * qusim_oracle.c -- CPU restatement of QuSim's split-operator time evolution
 * and of its Born-series scattering solvers.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle for the GB300
 * engine: only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
 * reference legs load it, and only as the checker or as the timed CPU
 * baseline.  The product path (libqsg.so) never links, loads or calls it.
 *
 * Parity pinning: the outputs of this restatement are checked against the
 * reference's own SplittingMethod1D/2D compiled from its sources (the
 * oracle/_ref build, fixtures under tests/golden/) and against the
 * reference's published known answers (tunnelling transmission
 * 0.15937744085 of applications/QuEvol1DPrecision/QuSimPrecision.cpp:82, group
 * velocity 1 of :206-218, FFT ramp round trip of
 * applications/QuSimTest/TestFFT.cpp:27-81).
 *
 * Everything is complex128 (interleaved re,im doubles), single threaded.
 *
 * What is restated (reference file:line, paths inside lhprojects/QuSim):
 *   - mixed-radix recursive decimation-in-time FFT: src/kissfft.hh:15-45
 *     (twiddles exp(+-2 pi i k/N), factor order 4,2,3,5,7,...), :82-115
 *     (recursion), :185-350 (radix 2/3/4/5/generic butterflies)
 *   - 2D transform = row transforms along contiguous y, then column
 *     transforms along x: src/FourierTransform.cpp:148-291
 *   - step sequences O2 / O4 and their constants: src/SplittingUtils.h:14-64,
 *     src/SplittingUtils.cpp:3-8
 *   - 1D ExpV / ExpT (periodic and infinite wall), CalKinEn:
 *     src/SplittingMethod1D.cpp:40-127
 *   - 2D phase tables, ExpV / ExpT, CalKinEn: src/SplittingMethod2D.cpp:38-138
 *   - Norm2 / PotEn / Xavg / Norm2(x0,x1) / Step renormalisation:
 *     src/EvolverImpl.cpp:45-68, src/EvolverImpl1D.cpp:83-102
 *   - k index fold i > N/2 ? N - i : i: src/DeviceTemplate.h:544-547
 *   - Born-series scattering solvers QuPerturbation1D/2D (naive and
 *     preconditioned series, absorbing layer, epsilon, R/T, delta-psi norm,
 *     cross sections): src/Perturbation1DImpl.cpp, src/Perturbation2DImpl.cpp,
 *     src/Perburbation.h, src/ScatteringSolverImpl.cpp (cited per function
 *     in the last section of this file)
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef double _Complex cplx;

static const double kPi = 3.141592653589793238462643383279502884197169399375;

/* ------------------------------------------------------------------------ */
/* Mixed-radix FFT plan (kissfft.hh:15-45)                                   */
/* ------------------------------------------------------------------------ */

typedef struct {
    size_t n;
    int inverse;
    cplx *tw;            /* tw[i] = exp(sign * 2 pi i / n), sign = -1 forward */
    int nstages;
    size_t radix[64];
    size_t remain[64];
} fft_plan;

static int plan_init(fft_plan *p, size_t n, int inverse)
{
    memset(p, 0, sizeof(*p));
    if (n == 0) return -1;
    p->n = n;
    p->inverse = inverse;
    p->tw = (cplx *)malloc(sizeof(cplx) * n);
    if (!p->tw) return -1;
    /* phase increment (inverse ? +2 : -2) * acos(-1) / n, kissfft.hh:22 */
    const double phinc = (inverse ? 2.0 : -2.0) * acos(-1.0) / (double)n;
    for (size_t i = 0; i < n; ++i) p->tw[i] = cexp(I * ((double)i * phinc));
    /* factor out 4s, then 2s, then odd numbers 3,5,7,...; kissfft.hh:26-43 */
    size_t m = n, f = 4;
    do {
        while (m % f) {
            if (f == 4) f = 2;
            else if (f == 2) f = 3;
            else f += 2;
            if (f * f > m) f = m;
        }
        m /= f;
        p->radix[p->nstages] = f;
        p->remain[p->nstages] = m;
        p->nstages++;
    } while (m > 1);
    return 0;
}

static void plan_free(fft_plan *p)
{
    free(p->tw);
    p->tw = NULL;
}

static void bfly2(const fft_plan *p, cplx *out, size_t fs, size_t m)
{
    for (size_t k = 0; k < m; ++k) {
        cplx t = out[m + k] * p->tw[k * fs];
        out[m + k] = out[k] - t;
        out[k] += t;
    }
}

static void bfly3(const fft_plan *p, cplx *out, size_t fs, size_t m)
{
    const double e3 = cimag(p->tw[fs * m]);
    for (size_t k = 0; k < m; ++k) {
        cplx a1 = out[k + m] * p->tw[k * fs];
        cplx a2 = out[k + 2 * m] * p->tw[2 * k * fs];
        cplx s = a1 + a2, d = (a1 - a2) * e3;
        cplx mid = out[k] - s * 0.5;
        out[k] += s;
        out[k + 2 * m] = creal(mid) + cimag(d) + I * (cimag(mid) - creal(d));
        out[k + m] = creal(mid) - cimag(d) + I * (cimag(mid) + creal(d));
    }
}

static void bfly4(const fft_plan *p, cplx *out, size_t fs, size_t m)
{
    const double sg = p->inverse ? -1.0 : 1.0;
    for (size_t k = 0; k < m; ++k) {
        cplx a1 = out[k + m] * p->tw[k * fs];
        cplx a2 = out[k + 2 * m] * p->tw[2 * k * fs];
        cplx a3 = out[k + 3 * m] * p->tw[3 * k * fs];
        cplx d02 = out[k] - a2;
        cplx s02 = out[k] + a2;
        cplx s13 = a1 + a3;
        cplx d13 = a1 - a3;
        /* multiply d13 by -i (forward) or +i (inverse) */
        cplx r = cimag(d13) * sg - I * (creal(d13) * sg);
        out[k + 2 * m] = s02 - s13;
        out[k] = s02 + s13;
        out[k + m] = d02 + r;
        out[k + 3 * m] = d02 - r;
    }
}

static void bfly5(const fft_plan *p, cplx *out, size_t fs, size_t m)
{
    const cplx ya = p->tw[fs * m], yb = p->tw[fs * 2 * m];
    for (size_t u = 0; u < m; ++u) {
        cplx x0 = out[u];
        cplx x1 = out[u + m] * p->tw[u * fs];
        cplx x2 = out[u + 2 * m] * p->tw[2 * u * fs];
        cplx x3 = out[u + 3 * m] * p->tw[3 * u * fs];
        cplx x4 = out[u + 4 * m] * p->tw[4 * u * fs];
        cplx s14 = x1 + x4, d14 = x1 - x4, s23 = x2 + x3, d23 = x2 - x3;
        out[u] = x0 + s14 + s23;
        cplx a = x0 + (creal(s14) * creal(ya) + creal(s23) * creal(yb))
                    + I * (cimag(s14) * creal(ya) + cimag(s23) * creal(yb));
        cplx b = (cimag(d14) * cimag(ya) + cimag(d23) * cimag(yb))
                    - I * (creal(d14) * cimag(ya) + creal(d23) * cimag(yb));
        out[u + m] = a - b;
        out[u + 4 * m] = a + b;
        cplx c = x0 + (creal(s14) * creal(yb) + creal(s23) * creal(ya))
                    + I * (cimag(s14) * creal(yb) + cimag(s23) * creal(ya));
        cplx d = (-cimag(d14) * cimag(yb) + cimag(d23) * cimag(ya))
                    + I * (creal(d14) * cimag(yb) - creal(d23) * cimag(ya));
        out[u + 2 * m] = c + d;
        out[u + 3 * m] = c - d;
    }
}

static void bfly_generic(const fft_plan *p, cplx *out, size_t fs, size_t m, size_t r)
{
    cplx scratch_s[32];
    cplx *scratch = r > 32 ? (cplx *)malloc(sizeof(cplx) * r) : scratch_s;
    for (size_t u = 0; u < m; ++u) {
        for (size_t q = 0; q < r; ++q) scratch[q] = out[u + q * m];
        for (size_t q1 = 0; q1 < r; ++q1) {
            size_t k = u + q1 * m, ti = 0;
            cplx acc = scratch[0];
            for (size_t q = 1; q < r; ++q) {
                ti += fs * k;
                if (ti >= p->n) ti -= p->n;
                acc += scratch[q] * p->tw[ti];
            }
            out[k] = acc;
        }
    }
    if (scratch != scratch_s) free(scratch);
}

/* kissfft.hh:82-115: DFT of size r*m = r DFTs of size m over decimated input,
 * recombined by a radix-r butterfly. */
static void fft_rec(const fft_plan *p, const cplx *in, cplx *out, int stage,
                    size_t fstride, size_t istride)
{
    const size_t r = p->radix[stage], m = p->remain[stage];
    cplx *const beg = out, *const end = out + r * m;
    if (m == 1) {
        do {
            *out = *in;
            in += fstride * istride;
        } while (++out != end);
    } else {
        do {
            fft_rec(p, in, out, stage + 1, fstride * r, istride);
            in += fstride * istride;
        } while ((out += m) != end);
    }
    out = beg;
    switch (r) {
    case 2: bfly2(p, out, fstride, m); break;
    case 3: bfly3(p, out, fstride, m); break;
    case 4: bfly4(p, out, fstride, m); break;
    case 5: bfly5(p, out, fstride, m); break;
    default: bfly_generic(p, out, fstride, m, r); break;
    }
}

static void plan_exec(const fft_plan *p, const cplx *in, cplx *out)
{
    fft_rec(p, in, out, 0, 1, 1);
}

/* Row transforms along contiguous y (length ny), then column transforms
 * along x (length nx); FourierTransform.cpp:243-285.  Index iy + ix*ny. */
static void fft2d_exec(const fft_plan *px, const fft_plan *py, size_t nx, size_t ny,
                       const cplx *in, cplx *out, cplx *col_in, cplx *col_out)
{
    for (size_t i = 0; i < nx; ++i) plan_exec(py, in + i * ny, out + i * ny);
    for (size_t j = 0; j < ny; ++j) {
        for (size_t i = 0; i < nx; ++i) col_in[i] = out[i * ny + j];
        plan_exec(px, col_in, col_out);
        for (size_t i = 0; i < nx; ++i) out[i * ny + j] = col_out[i];
    }
}

/* ------------------------------------------------------------------------ */
/* Public FFT entry points                                                   */
/* ------------------------------------------------------------------------ */

int orc_fft1d(size_t n, int inverse, const double *in, double *out)
{
    fft_plan p;
    if (plan_init(&p, n, inverse)) return -1;
    plan_exec(&p, (const cplx *)in, (cplx *)out);
    plan_free(&p);
    return 0;
}

int orc_fft2d(size_t nx, size_t ny, int inverse, const double *in, double *out)
{
    fft_plan px, py;
    if (plan_init(&px, nx, inverse)) return -1;
    if (plan_init(&py, ny, inverse)) { plan_free(&px); return -1; }
    cplx *ci = (cplx *)malloc(sizeof(cplx) * nx), *co = (cplx *)malloc(sizeof(cplx) * nx);
    fft2d_exec(&px, &py, nx, ny, (const cplx *)in, (cplx *)out, ci, co);
    free(ci); free(co);
    plan_free(&px); plan_free(&py);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Splitting constants (SplittingUtils.cpp:3-8)                              */
/* ------------------------------------------------------------------------ */

void orc_splitting_constants(double *c1, double *c2, double *d1, double *d2)
{
    const double t = pow(2.0, 1.0 / 3.0);
    *c1 = 1.0 / (2.0 * (2.0 - t));
    *c2 = (1.0 - t) / (2.0 * (2.0 - t));
    *d1 = 1.0 / (2.0 - t);
    *d2 = -t / (2.0 - t);
}

static size_t fold_half(size_t i, size_t n) { return i > n / 2 ? n - i : i; }

/* The reference's CPU reductions are std::transform_reduce with the sequential
 * policy (src/DeviceTemplate.h:404-407), which libstdc++ evaluates four
 * elements at a time: init + ((f0 + f1) + (f2 + f3)), then the tail one by
 * one.  Restated with that pairing so the sums agree to the last bit. */
#define TR_SUM(n, F)                                                           \
    ({                                                                         \
        double acc_ = 0;                                                       \
        size_t i_ = 0;                                                         \
        for (; (n) - i_ >= 4; i_ += 4) {                                       \
            size_t i = i_;                                                     \
            const double f0_ = (F);                                            \
            i = i_ + 1;                                                        \
            const double f1_ = (F);                                            \
            i = i_ + 2;                                                        \
            const double f2_ = (F);                                            \
            i = i_ + 3;                                                        \
            const double f3_ = (F);                                            \
            acc_ = acc_ + ((f0_ + f1_) + (f2_ + f3_));                         \
        }                                                                      \
        for (; i_ < (n); ++i_) {                                               \
            size_t i = i_;                                                     \
            acc_ = acc_ + (F);                                                 \
        }                                                                      \
        acc_;                                                                  \
    })

/* The two-range reductions (Abs2Mul, Abs2K1D/2D, Abs2Idx: a data range zipped
 * with V or an index range) go through the sequential policy's inner_product
 * brick instead: init = init + f(i), one element at a time. */
#define SEQ_SUM(n, F)                                                          \
    ({                                                                         \
        double acc_ = 0;                                                       \
        for (size_t i = 0; i < (n); ++i) acc_ = acc_ + (F);                    \
        acc_;                                                                  \
    })

static double abs2c(cplx z) { return cimag(z) * cimag(z) + creal(z) * creal(z); }  /* op_Abs2 */

/* Device::Norm2 without dv (DeviceTemplate.h:1222-1229) */
static double norm2_raw(const cplx *p, size_t n) { return TR_SUM(n, abs2c(p[i])); }

/* the complex coefficient -i * dt * t / hbar of ExpV, SplittingMethod1D.cpp:87 */
static cplx expv_coef(cplx dt, double t, double hbar) { return (-I / hbar) * dt * t; }

/* ------------------------------------------------------------------------ */
/* 1D evolver (SplittingMethod1D.cpp)                                        */
/* ------------------------------------------------------------------------ */

typedef struct {
    size_t n;
    double dx, mass, hbar;
    cplx dt;
    int order, wall;
    fft_plan fwd, inv, inv2n;
    cplx *ft, *iw, *iwk;
} ev1d;

static void ev1d_expv(ev1d *e, cplx *psi, const double *V, double t)
{
    const cplx f = expv_coef(e->dt, t, e->hbar);
    for (size_t i = 0; i < e->n; ++i) psi[i] = psi[i] * cexp(f * V[i]);
}

static void ev1d_expt(ev1d *e, cplx *psi, double tt)
{
    const size_t n = e->n;
    if (!e->wall) {
        plan_exec(&e->fwd, psi, e->ft);
        const double dk = 2 * kPi / (e->dx * n);
        const double DT = (dk * e->hbar) * (dk * e->hbar) / (2 * e->mass);
        const cplx f = -I * DT * e->dt * tt / e->hbar;
        for (size_t i = 0; i < n; ++i) {
            const double fi = (double)fold_half(i, n);
            e->ft[i] = e->ft[i] * cexp(f * (fi * fi));
        }
        plan_exec(&e->inv, e->ft, psi);
        const double s = 1.0 / (double)n;
        for (size_t i = 0; i < n; ++i) psi[i] = psi[i] * s;
    } else {
        /* odd extension to 2N, sine transform through a 2N inverse FFT,
         * SplittingMethod1D.cpp:61-81 */
        cplx *iw = e->iw, *iwk = e->iwk;
        memcpy(iw, psi, sizeof(cplx) * n);
        iw[0] = 0; iw[n] = 0;
        for (size_t k = 0; k + 1 < n; ++k) iw[2 * n - 1 - k] = -iw[1 + k];
        plan_exec(&e->inv2n, iw, iwk);
        const double dp = e->hbar * kPi / (e->dx * n);
        const double DT = dp * dp / (2 * e->mass);
        const cplx f = -I * DT * e->dt * tt / e->hbar;
        for (size_t i = 0; i < n; ++i) iwk[i] = iwk[i] * cexp(((double)i * (double)i) * f);
        iwk[0] = 0; iwk[n] = 0;
        for (size_t k = 0; k + 1 < n; ++k) iwk[2 * n - 1 - k] = -iwk[1 + k];
        plan_exec(&e->inv2n, iwk, iw);
        const double s = -1.0 / (2.0 * n);
        for (size_t i = 0; i < n; ++i) psi[i] = iw[i] * s;
    }
}

static int ev1d_init(ev1d *e, size_t n, double dx, double mass, double hbar,
                     double dt_re, double dt_im, int order, int wall)
{
    memset(e, 0, sizeof(*e));
    if (n < 2 || (order != 2 && order != 4)) return -1;
    e->n = n; e->dx = dx; e->mass = mass; e->hbar = hbar;
    e->dt = dt_re + I * dt_im; e->order = order; e->wall = wall;
    if (!wall) {
        if (plan_init(&e->fwd, n, 0) || plan_init(&e->inv, n, 1)) return -1;
        e->ft = (cplx *)malloc(sizeof(cplx) * n);
    } else {
        if (plan_init(&e->inv2n, 2 * n, 1)) return -1;
        e->iw = (cplx *)malloc(sizeof(cplx) * 2 * n);
        e->iwk = (cplx *)malloc(sizeof(cplx) * 2 * n);
    }
    return 0;
}

static void ev1d_free(ev1d *e)
{
    plan_free(&e->fwd); plan_free(&e->inv); plan_free(&e->inv2n);
    free(e->ft); free(e->iw); free(e->iwk);
}

/* QuUpdatePsi, SplittingUtils.h:14-64 (fold_head_tail == false) */
static void ev1d_step(ev1d *e, cplx *psi, const double *V)
{
    if (e->order == 2) {
        ev1d_expv(e, psi, V, 0.5);
        ev1d_expt(e, psi, 1.0);
        ev1d_expv(e, psi, V, 0.5);
    } else {
        double c1, c2, d1, d2;
        orc_splitting_constants(&c1, &c2, &d1, &d2);
        ev1d_expv(e, psi, V, c1);
        ev1d_expt(e, psi, d1);
        ev1d_expv(e, psi, V, c2);
        ev1d_expt(e, psi, d2);
        ev1d_expv(e, psi, V, c2);
        ev1d_expt(e, psi, d1);
        ev1d_expv(e, psi, V, c1);
    }
}

/* Evolve psi (n complex, in place) by nsteps steps.  fnes = renormalise to
 * Norm2 == 1 after each step (EvolverImpl.cpp:60-63).  Returns 0 on success. */
int orc_evolve1d(size_t n, double dx, double mass, double hbar, double dt_re, double dt_im,
                 int order, int wall, int fnes, double *psi_io, const double *V, uint64_t nsteps)
{
    ev1d e;
    if (ev1d_init(&e, n, dx, mass, hbar, dt_re, dt_im, order, wall)) { ev1d_free(&e); return -1; }
    cplx *psi = (cplx *)psi_io;
    for (uint64_t s = 0; s < nsteps; ++s) {
        ev1d_step(&e, psi, V);
        if (fnes) {
            const double sc = 1.0 / sqrt(norm2_raw(psi, n) * dx);
            for (size_t i = 0; i < n; ++i) psi[i] = psi[i] * sc;
        }
    }
    ev1d_free(&e);
    return 0;
}

/* <T> of SplittingMethod1D::CalKinEn (:91-127).  The periodic branch omits
 * hbar^2 (:102); the wall branch includes it (:119). */
double orc_kinen1d(size_t n, double dx, double mass, double hbar, int wall, const double *psi_in)
{
    const cplx *psi = (const cplx *)psi_in;
    double kin = 0, nn = 0;
    if (!wall) {
        fft_plan p;
        if (plan_init(&p, n, 0)) return NAN;
        cplx *ft = (cplx *)malloc(sizeof(cplx) * n);
        plan_exec(&p, psi, ft);
        const double dk = 2 * kPi / (dx * n);
        const double DT = dk * dk / (2 * mass);
        /* Abs2K1D (DeviceTemplate.h:1527-1536, op :738-752) */
        kin = SEQ_SUM(n, abs2c(ft[i]) * ((double)fold_half(i, n) * (double)fold_half(i, n)) * DT);
        nn = norm2_raw(ft, n);
        free(ft);
        plan_free(&p);
    } else {
        fft_plan p;
        if (plan_init(&p, 2 * n, 1)) return NAN;
        cplx *iw = (cplx *)malloc(sizeof(cplx) * 2 * n), *iwk = (cplx *)malloc(sizeof(cplx) * 2 * n);
        memcpy(iw, psi, sizeof(cplx) * n);
        iw[0] = 0; iw[n] = 0;
        for (size_t k = 0; k + 1 < n; ++k) iw[2 * n - 1 - k] = -iw[1 + k];
        plan_exec(&p, iw, iwk);
        const double dk = kPi / (dx * n);
        const double DT = (dk * hbar) * (dk * hbar) / (2 * mass);
        /* Abs2Idx2 (op_Abs2MulSquare) */
        kin = SEQ_SUM(n, abs2c(iwk[i]) * ((double)i * (double)i)) * DT;
        nn = norm2_raw(iwk, n);
        free(iw); free(iwk);
        plan_free(&p);
    }
    return kin / nn;
}

/* ------------------------------------------------------------------------ */
/* 2D evolver (SplittingMethod2D.cpp), periodic only                         */
/* ------------------------------------------------------------------------ */

typedef struct {
    size_t nx, ny, n;
    int order;
    fft_plan fx, fy, ix, iy;
    cplx *ft, *ci, *co;
    cplx *ev[2];   /* V tables: O2 {1/2}; O4 {C1, C2}  (SplittingMethod2D.cpp:38-54) */
    cplx *et[2];   /* T tables: O2 {1};   O4 {D1, D2}  (:56-79) */
} ev2d;

static void ev2d_free(ev2d *e)
{
    plan_free(&e->fx); plan_free(&e->fy); plan_free(&e->ix); plan_free(&e->iy);
    free(e->ft); free(e->ci); free(e->co);
    for (int k = 0; k < 2; ++k) { free(e->ev[k]); free(e->et[k]); }
}

static int ev2d_init(ev2d *e, size_t nx, size_t ny, double dx, double dy, double mass,
                     double hbar, double dt_re, double dt_im, int order, const double *V)
{
    memset(e, 0, sizeof(*e));
    if (nx < 2 || ny < 2 || (order != 2 && order != 4)) return -1;
    e->nx = nx; e->ny = ny; e->n = nx * ny; e->order = order;
    if (plan_init(&e->fx, nx, 0) || plan_init(&e->fy, ny, 0) ||
        plan_init(&e->ix, nx, 1) || plan_init(&e->iy, ny, 1)) return -1;
    e->ft = (cplx *)malloc(sizeof(cplx) * e->n);
    e->ci = (cplx *)malloc(sizeof(cplx) * nx);
    e->co = (cplx *)malloc(sizeof(cplx) * nx);
    const cplx dt = dt_re + I * dt_im;
    double c1, c2, d1, d2;
    orc_splitting_constants(&c1, &c2, &d1, &d2);
    const double vc[2] = {order == 2 ? 0.5 : c1, c2};
    const double tc[2] = {order == 2 ? 1.0 : d1, d2};
    const int ntab = order == 2 ? 1 : 2;
    const double dkx = 2 * kPi / (dx * nx), dky = 2 * kPi / (dy * ny);
    const double DTx = (dkx * hbar) * (dkx * hbar) / (2 * mass);
    const double DTy = (dky * hbar) * (dky * hbar) / (2 * mass);
    const cplx alpha = -I * dt / hbar;
    for (int k = 0; k < ntab; ++k) {
        e->ev[k] = (cplx *)malloc(sizeof(cplx) * e->n);
        e->et[k] = (cplx *)malloc(sizeof(cplx) * e->n);
        const cplx f = expv_coef(dt, vc[k], hbar);
        for (size_t i = 0; i < e->n; ++i) e->ev[k][i] = cexp(f * V[i]);
        const cplx a = alpha * tc[k];
        for (size_t i = 0; i < nx; ++i) {
            const double fi = (double)fold_half(i, nx);
            for (size_t j = 0; j < ny; ++j) {
                const double fj = (double)fold_half(j, ny);
                e->et[k][i * ny + j] = 1.0 * cexp(a * ((fi * fi) * DTx + (fj * fj) * DTy));
            }
        }
    }
    return 0;
}

static void ev2d_mul(cplx *p, const cplx *t, size_t n)
{
    for (size_t i = 0; i < n; ++i) p[i] = t[i] * p[i];
}

static void ev2d_expt(ev2d *e, cplx *psi, const cplx *tab)
{
    fft2d_exec(&e->fx, &e->fy, e->nx, e->ny, psi, e->ft, e->ci, e->co);
    ev2d_mul(e->ft, tab, e->n);
    fft2d_exec(&e->ix, &e->iy, e->nx, e->ny, e->ft, psi, e->ci, e->co);
    const double s = 1.0 / (double)e->n;
    for (size_t i = 0; i < e->n; ++i) psi[i] = psi[i] * s;
}

static void ev2d_step(ev2d *e, cplx *psi)
{
    if (e->order == 2) {
        ev2d_mul(psi, e->ev[0], e->n);
        ev2d_expt(e, psi, e->et[0]);
        ev2d_mul(psi, e->ev[0], e->n);
    } else {
        ev2d_mul(psi, e->ev[0], e->n);
        ev2d_expt(e, psi, e->et[0]);
        ev2d_mul(psi, e->ev[1], e->n);
        ev2d_expt(e, psi, e->et[1]);
        ev2d_mul(psi, e->ev[1], e->n);
        ev2d_expt(e, psi, e->et[0]);
        ev2d_mul(psi, e->ev[0], e->n);
    }
}

int orc_evolve2d(size_t nx, size_t ny, double dx, double dy, double mass, double hbar,
                 double dt_re, double dt_im, int order, int fnes, double *psi_io,
                 const double *V, uint64_t nsteps)
{
    ev2d e;
    if (ev2d_init(&e, nx, ny, dx, dy, mass, hbar, dt_re, dt_im, order, V)) { ev2d_free(&e); return -1; }
    cplx *psi = (cplx *)psi_io;
    for (uint64_t s = 0; s < nsteps; ++s) {
        ev2d_step(&e, psi);
        if (fnes) {
            const double sc = 1.0 / sqrt(norm2_raw(psi, e.n) * dx * dy);
            for (size_t i = 0; i < e.n; ++i) psi[i] = psi[i] * sc;
        }
    }
    ev2d_free(&e);
    return 0;
}

/* SplittingMethod2D::CalKinEn (:123-138) */
double orc_kinen2d(size_t nx, size_t ny, double dx, double dy, double mass, double hbar,
                   const double *psi_in)
{
    fft_plan px, py;
    if (plan_init(&px, nx, 0) || plan_init(&py, ny, 0)) return NAN;
    const size_t n = nx * ny;
    cplx *ft = (cplx *)malloc(sizeof(cplx) * n);
    cplx *ci = (cplx *)malloc(sizeof(cplx) * nx), *co = (cplx *)malloc(sizeof(cplx) * nx);
    fft2d_exec(&px, &py, nx, ny, (const cplx *)psi_in, ft, ci, co);
    const double dkx = 2 * kPi / (dx * nx), dky = 2 * kPi / (dy * ny);
    const double DTx = (dkx * hbar) * (dkx * hbar) / (2 * mass);
    const double DTy = (dky * hbar) * (dky * hbar) / (2 * mass);
    /* Abs2K2D (DeviceTemplate.h:1539-1548, op :772-792), element index i*ny + j */
#define KIN2D_TERM(k)                                                                   \
    (abs2c(ft[k]) * (((double)fold_half((k) / ny, nx) * (double)fold_half((k) / ny, nx)) * DTx + \
                     ((double)fold_half((k) % ny, ny) * (double)fold_half((k) % ny, ny)) * DTy))
    const double kin = SEQ_SUM(n, KIN2D_TERM(i));
#undef KIN2D_TERM
    const double nn = norm2_raw(ft, n);
    free(ft); free(ci); free(co);
    plan_free(&px); plan_free(&py);
    return kin / nn;
}

/* ------------------------------------------------------------------------ */
/* Observables (EvolverImpl.cpp:45-54, EvolverImpl1D.cpp:83-102)            */
/* ------------------------------------------------------------------------ */

double orc_norm2(size_t n, double dv, const double *psi)
{
    return norm2_raw((const cplx *)psi, n) * dv;
}

/* The renormalisation that ends QuEvolverImpl::Step when
 * force_normalization_each_step is set (EvolverImpl.cpp:60-63):
 * scale = 1 / sqrt(Norm2()), psi_i = scale * psi_i (Device::Scale). */
void orc_renormalize(size_t n, double dv, double *psi_io)
{
    cplx *psi = (cplx *)psi_io;
    const double sc = 1.0 / sqrt(norm2_raw(psi, n) * dv);
    for (size_t i = 0; i < n; ++i) psi[i] = sc * psi[i];
}

/* Sum |psi|^2 V dv / Norm2 */
double orc_poten(size_t n, double dv, const double *psi_in, const double *V)
{
    const cplx *psi = (const cplx *)psi_in;
    const double s = SEQ_SUM(n, abs2c(psi[i]) * V[i]);  /* Abs2Mul (DeviceTemplate.h:1601-1609) */
    return (s * dv) / orc_norm2(n, dv, psi_in);
}

double orc_xavg(size_t n, double x0, double dx, const double *psi_in)
{
    const cplx *psi = (const cplx *)psi_in;
    const double s = SEQ_SUM(n, abs2c(psi[i]) * (double)i);  /* Abs2Idx (DeviceTemplate.h:1200-1209) */
    return x0 + dx * (s / norm2_raw(psi, n));
}

/* Norm2 over [xa, xb) of a 1D grid starting at x0; EvolverImpl1D.cpp:90-102 */
double orc_norm2_range(size_t n, double x0, double dx, double xa, double xb, const double *psi)
{
    int64_t i1 = (int64_t)((xa - x0) / dx), i2 = (int64_t)((xb - x0) / dx);
    if (i1 <= 0) i1 = 0;
    if (i2 >= (int64_t)n) i2 = (int64_t)n;
    if (i1 >= i2) return 0;
    return norm2_raw((const cplx *)psi + i1, (size_t)(i2 - i1)) * dx;
}

/* ------------------------------------------------------------------------ */
/* Persistent evolvers: set up once (plans, tables), step many times.  Used */
/* to time the CPU path per step, as the reference's Evolver::step() runs.  */
/* ------------------------------------------------------------------------ */

void *orc_ev1d_new(size_t n, double dx, double mass, double hbar, double dt_re, double dt_im,
                   int order, int wall)
{
    ev1d *e = (ev1d *)malloc(sizeof(ev1d));
    if (!e) return NULL;
    if (ev1d_init(e, n, dx, mass, hbar, dt_re, dt_im, order, wall)) {
        ev1d_free(e);
        free(e);
        return NULL;
    }
    return e;
}

void orc_ev1d_step(void *h, double *psi, const double *V, uint64_t nsteps)
{
    for (uint64_t s = 0; s < nsteps; ++s) ev1d_step((ev1d *)h, (cplx *)psi, V);
}

void orc_ev1d_free(void *h)
{
    if (!h) return;
    ev1d_free((ev1d *)h);
    free(h);
}

void *orc_ev2d_new(size_t nx, size_t ny, double dx, double dy, double mass, double hbar,
                   double dt_re, double dt_im, int order, const double *V)
{
    ev2d *e = (ev2d *)malloc(sizeof(ev2d));
    if (!e) return NULL;
    if (ev2d_init(e, nx, ny, dx, dy, mass, hbar, dt_re, dt_im, order, V)) {
        ev2d_free(e);
        free(e);
        return NULL;
    }
    return e;
}

void orc_ev2d_step(void *h, double *psi, uint64_t nsteps)
{
    for (uint64_t s = 0; s < nsteps; ++s) ev2d_step((ev2d *)h, (cplx *)psi);
}

void orc_ev2d_free(void *h)
{
    if (!h) return;
    ev2d_free((ev2d *)h);
    free(h);
}

/* ------------------------------------------------------------------------ */
/* Born-series scattering solvers (QuPerturbation1D / QuPerturbation2D)      */
/*                                                                          */
/*   init:   src/Perturbation1DImpl.cpp:7-42, src/Perturbation2DImpl.cpp:4-47, */
/*           src/ScatteringSolverImpl.cpp:20-38, 68-83, 87-172               */
/*   layer:  GaussMAsbLayer1D/2D and cal_v15, src/Perburbation.h:47-57,      */
/*           80-95, 131-148                                                  */
/*   eps:    PreconditionalBornSeries::GetEpsilon, src/Perburbation.h:326-341 */
/*   naive:  BornSeries::Update1D/2D, src/Perburbation.h:238-287             */
/*   precon: PreconditionalBornSeries::Update, src/Perburbation.h:349-417,   */
/*           ops src/DeviceTemplate.h:1004-1093 (AddMul, Vellekoop, Hao1,    */
/*           Hao2, Add3), G01D/G02D :881-931, LinearUpdate :532-541          */
/*   R, T:   ScatteringSolver1DImpl::ComputeRT, ScatteringSolverImpl.cpp:40-55 */
/*   2D:     Compute's delta-psi norm, src/Perturbation2DImpl.cpp:49-83;     */
/*           ComputeXSection / ComputeTotalXSection,                         */
/*           src/ScatteringSolverImpl.cpp:218-266                            */
/* preconditioner: 0 identity ("BornIndentity"), 1 Vellekoop, 2 Hao1, 3 Hao2 */
/* ------------------------------------------------------------------------ */

static size_t fold_half_pb(size_t i, size_t n) { return i < n / 2 ? i : n - i; }  /* Perburbation.h:30-33 */

static double cal_v15(double x, double k0, double e0)  /* Perburbation.h:47-57 */
{
    x *= k0;
    const double u = 1 - x * x / (15. * 15);
    return (-0.8 * e0) * (u > 0 ? exp(-0.015 * x * x * 1. / sqrt(1 - x * x / (15. * 15))) : 0);
}


/* epsilon actually used by the preconditioned series (GetEpsilon) */
static double born_min_epsilon(const cplx *v, size_t n, int precer)
{
    if (precer == 0) {
        const double a = TR_SUM(n, cimag(v[i]));
        const double a2 = TR_SUM(n, abs2c(v[i]));
        return 0.5 * a2 / (-a);
    }
    double m = 0;
    for (size_t i = 0; i < n; ++i) {
        const double s = abs2c(v[i]);
        m = m >= s ? m : s;
    }
    return sqrt(m);
}

/* 1D set-up: psi0 = exp(i dir k0 x_i), absorbing layer and epsilon when
 * preconditioned.  v_io: n complex in (the sampled potential), out (with the
 * layer).  Returns 0, or -1 for a world too small for the layer. */
int orc_born_init1d(size_t n, double x0, double dx, double en, double direction, double mass,
                    double hbar, int preconditional, int precer, double *eps_io, double *v_io,
                    double *psi0_out)
{
    cplx *v = (cplx *)v_io, *psi0 = (cplx *)psi0_out;
    const double k0 = sqrt(2 * en * mass) / hbar;
    const double dir = direction > 0 ? 1 : -1;
    for (size_t i = 0; i < n; ++i) psi0[i] = cexp(dir * k0 * (x0 + dx * i) * I);
    if (preconditional) {
        const double lambda = 2 * kPi / (sqrt(2 * mass * en) / hbar);
        if (n * dx < 24 * lambda) return -1;
        const double kk = sqrt(2 * mass * en) / hbar;
        if (kk * dx * n < 30) return -1;
        for (size_t i = 0; i < n; ++i)
            v[i] = CMPLX(creal(v[i]), cimag(v[i]) + cal_v15(fold_half_pb(i, n) * dx, kk, en));
        const double me = born_min_epsilon(v, n, precer);
        if (*eps_io < me) *eps_io = me;
    }
    return 0;
}

int orc_born_init2d(size_t nx, size_t ny, double x0, double dx, double y0, double dy, double en,
                    double dirx, double diry, double mass, double hbar, int preconditional,
                    int precer, double *eps_io, double *v_io, double *psi0_out)
{
    cplx *v = (cplx *)v_io, *psi0 = (cplx *)psi0_out;
    const double k0 = sqrt(2 * en * mass) / hbar;
    const double nm = 1 / sqrt(dirx * dirx + diry * diry);
    const double kx = k0 * (dirx * nm), ky = k0 * (diry * nm);
    for (size_t i = 0; i < nx; ++i)
        for (size_t j = 0; j < ny; ++j)
            psi0[i * ny + j] = cexp((kx * (x0 + dx * i) + ky * (y0 + dy * j)) * I);
    if (preconditional) {
        const double lambda = 2 * kPi / (sqrt(2 * mass * en) / hbar);
        if (nx * dx < 24 * lambda || ny * dy < 24 * lambda) return -1;
        const double kk = sqrt(2 * mass * en) / hbar;
        for (size_t i = 0; i < nx; ++i)
            for (size_t j = 0; j < ny; ++j) {
                const size_t k = i * ny + j;
                v[k] = CMPLX(creal(v[k]), cimag(v[k]) + (cal_v15(fold_half_pb(i, nx) * dx, kk, en) +
                                                         cal_v15(fold_half_pb(j, ny) * dy, kk, en)));
            }
        const double me = born_min_epsilon(v, nx * ny, precer);
        if (*eps_io < me) *eps_io = me;
    }
    return 0;
}

/* tmp <- (Re v + i (Im v + eps)) dpsi + Re v psi0 (op_Add3) or
 * dpsi <- (dpsi + psi0) v (op_AddMul) */
static void born_pre(size_t n, int preconditional, double eps, const cplx *psi0, const cplx *v,
                     const cplx *dpsi, cplx *out)
{
    for (size_t i = 0; i < n; ++i) {
        if (preconditional)
            out[i] = CMPLX(creal(v[i]), cimag(v[i]) + eps) * dpsi[i] + creal(v[i]) * psi0[i];
        else
            out[i] = (dpsi[i] + psi0[i]) * v[i];
    }
}

/* the update after the transform pair; tmp already carries 1/N */
static void born_post(size_t n, int precer, double slow, double eps, const cplx *v, const cplx *tmp,
                      cplx *dpsi)
{
    for (size_t i = 0; i < n; ++i) {
        if (precer == 0) {
            dpsi[i] = slow == 1. ? tmp[i] : dpsi[i] * (1 - slow) + tmp[i] * slow;
            continue;
        }
        cplx g;
        const cplx iv = CMPLX(-cimag(v[i]), creal(v[i]));          /* i v */
        const cplx ivc = CMPLX(cimag(v[i]), creal(v[i]));          /* i conj(v) */
        if (precer == 1) g = 1. - iv / eps;
        else if (precer == 2) g = 1. - ivc / eps;
        else g = CMPLX(2., 0.) / (1. + iv / eps);
        g *= slow;
        dpsi[i] = (1. - g) * dpsi[i] + g * tmp[i];
    }
}

/* `order` iterations of the naive or the preconditioned series on dpsi_io */
int orc_born_iter1d(size_t n, double dx, double en, double eps, double mass, double hbar, int order,
                    int preconditional, int precer, double slow, const double *psi0_in,
                    const double *v_in, double *dpsi_io)
{
    const cplx *psi0 = (const cplx *)psi0_in, *v = (const cplx *)v_in;
    cplx *dpsi = (cplx *)dpsi_io;
    fft_plan fwd, inv;
    if (plan_init(&fwd, n, 0)) return -1;
    if (plan_init(&inv, n, 1)) { plan_free(&fwd); return -1; }
    cplx *a = (cplx *)malloc(sizeof(cplx) * n), *k = (cplx *)malloc(sizeof(cplx) * n);
    const double dp = 2 * kPi / (dx * n) * hbar, d = dp * dp / (2 * mass);
    for (int it = 0; it < order; ++it) {
        born_pre(n, preconditional, eps, psi0, v, dpsi, a);
        plan_exec(&fwd, a, k);
        for (size_t i = 0; i < n; ++i) {
            const double f = (double)fold_half(i, n);
            k[i] = k[i] / CMPLX(en - f * f * d, eps);
            k[i] = CMPLX(creal(k[i]) * (1. / n), cimag(k[i]) * (1. / n));
        }
        plan_exec(&inv, k, a);
        if (preconditional) born_post(n, precer, slow, eps, v, a, dpsi);
        else memcpy(dpsi, a, sizeof(cplx) * n);
    }
    free(a); free(k);
    plan_free(&fwd); plan_free(&inv);
    return 0;
}

/* R and T (ComputeRT) */
void orc_born_rt1d(size_t n, double x0, double dx, double en, double direction, double mass, double hbar,
                   const double *psi0_in, const double *dpsi_in, const double *v_in, double *R, double *T)
{
    const cplx *psi0 = (const cplx *)psi0_in, *dpsi = (const cplx *)dpsi_in, *v = (const cplx *)v_in;
    const double k0 = sqrt(2 * en * mass) / hbar;
    const double dir = direction > 0 ? 1 : -1;
    cplx r = 0, t = 0;
    for (size_t i = 0; i < n; ++i) {
        const double x = x0 + dx * i;
        r += (psi0[i] + dpsi[i]) * creal(v[i]) * cexp(I * (-dir * k0) * (-x));
        t += (psi0[i] + dpsi[i]) * creal(v[i]) * cexp(I * (+dir * k0) * (-x));
    }
    const cplx f = dx * mass / (hbar * hbar * fabs(k0) * I);
    const cplx rr = r * f, tt = t * f + 1;
    *R = creal(rr) * creal(rr) + cimag(rr) * cimag(rr);
    *T = creal(tt) * creal(tt) + cimag(tt) * cimag(tt);
}

/* 2D: `order` iterations (2D transforms as orc_fft2d) and the delta-psi norm
 * sqrt(sum |psi - psi_start|^2 / sum |psi|^2) */
int orc_born_iter2d(size_t nx, size_t ny, double dx, double dy, double en, double eps, double mass,
                    double hbar, int order, int preconditional, int precer, double slow,
                    const double *psi0_in, const double *v_in, double *dpsi_io, double *delta_norm)
{
    const size_t n = nx * ny;
    const cplx *psi0 = (const cplx *)psi0_in, *v = (const cplx *)v_in;
    cplx *dpsi = (cplx *)dpsi_io;
    fft_plan fx, fy, ix, iy;
    if (plan_init(&fx, nx, 0) || plan_init(&fy, ny, 0) || plan_init(&ix, nx, 1) || plan_init(&iy, ny, 1))
        return -1;
    cplx *a = (cplx *)malloc(sizeof(cplx) * n), *k = (cplx *)malloc(sizeof(cplx) * n);
    cplx *last = (cplx *)malloc(sizeof(cplx) * n);
    cplx *ci = (cplx *)malloc(sizeof(cplx) * nx), *co = (cplx *)malloc(sizeof(cplx) * nx);
    memcpy(last, dpsi, sizeof(cplx) * n);
    const double dpx = 2 * kPi / (dx * nx) * hbar, ddx = dpx * dpx / (2 * mass);
    const double dpy = 2 * kPi / (dy * ny) * hbar, ddy = dpy * dpy / (2 * mass);
    for (int it = 0; it < order; ++it) {
        born_pre(n, preconditional, eps, psi0, v, dpsi, a);
        fft2d_exec(&fx, &fy, nx, ny, a, k, ci, co);
        for (size_t i = 0; i < nx; ++i)
            for (size_t j = 0; j < ny; ++j) {
                const double fi = (double)fold_half(i, nx), fj = (double)fold_half(j, ny);
                const double t = fi * fi * ddx + fj * fj * ddy;
                cplx *p = &k[i * ny + j];
                *p = *p / CMPLX(en - t, eps);
                *p = CMPLX(creal(*p) * (1. / n), cimag(*p) * (1. / n));
            }
        fft2d_exec(&ix, &iy, nx, ny, k, a, ci, co);
        if (preconditional) born_post(n, precer, slow, eps, v, a, dpsi);
        else memcpy(dpsi, a, sizeof(cplx) * n);
    }
    const double num = TR_SUM(n, abs2c(dpsi[i] - last[i]));  /* MinusNorm2 */
    const double den = TR_SUM(n, abs2c(dpsi[i]));
    *delta_norm = sqrt(num / den);
    free(a); free(k); free(last); free(ci); free(co);
    plan_free(&fx); plan_free(&fy); plan_free(&ix); plan_free(&iy);
    return 0;
}

double orc_born_xsec2d(size_t nx, size_t ny, double x0, double dx, double y0, double dy, double en,
                       double mass, double hbar, const double *psi0_in, const double *dpsi_in,
                       const double *v_in, double cosx, double cosy)
{
    const cplx *psi0 = (const cplx *)psi0_in, *dpsi = (const cplx *)dpsi_in, *v = (const cplx *)v_in;
    const double k0 = sqrt(2 * en * mass) / hbar;
    const double nm = 1 / sqrt(cosx * cosx + cosy * cosy);
    const double kx = k0 * (cosx * nm), ky = k0 * (cosy * nm);
    cplx r = 0;
    for (size_t i = 0; i < nx; ++i)
        for (size_t j = 0; j < ny; ++j) {
            const size_t idx = i * ny + j;
            const double x = x0 + dx * i, y = y0 + dy * j;
            r += (psi0[idx] + dpsi[idx]) * creal(v[idx]) * cexp(-I * (kx * x + ky * y));
        }
    const cplx s = r * (2 * mass) / (hbar * hbar) * dx * dy * (1. / 4);
    return (creal(s) * creal(s) + cimag(s) * cimag(s)) * (2 / (kPi * k0));
}

/* ------------------------------------------------------------------------ */
/* 3D: grid index (ix*ny + iy)*nz + iz (CalGlobalIdx, include/QuSim.h:54-61) */
/* Transform: z lines, then y lines, then x lines, as KissFourierTransform3D */
/* (src/FourierTransform.cpp:379-440).                                      */
/* The reference has FFT3D and a 3D kinetic multiply (MulExpK3D,            */
/* src/DeviceTemplate.h:851-879, 1581-1589) but no 3D evolver; the 3D split-operator   */
/* step below is SplittingMethod2D's (ExpV: psi *= exp(-i dt c V / hbar);    */
/* ExpT: FFT, * exp(-i dt d (fold(i)^2 DTx + fold(j)^2 DTy + fold(k)^2 DTz)  */
/* / hbar), iFFT, / N; O2 and O4 sequences, src/SplittingMethod2D.cpp:38-121) */
/* with the third axis added.                                              */
/* ------------------------------------------------------------------------ */

static void fft3d_exec(const fft_plan *px, const fft_plan *py, const fft_plan *pz, size_t nx, size_t ny,
                       size_t nz, const cplx *in, cplx *out, cplx *li, cplx *lo)
{
    for (size_t i = 0; i < nx; ++i)
        for (size_t j = 0; j < ny; ++j) plan_exec(pz, in + (i * ny + j) * nz, out + (i * ny + j) * nz);
    for (size_t i = 0; i < nx; ++i)
        for (size_t k = 0; k < nz; ++k) {
            for (size_t j = 0; j < ny; ++j) li[j] = out[(i * ny + j) * nz + k];
            plan_exec(py, li, lo);
            for (size_t j = 0; j < ny; ++j) out[(i * ny + j) * nz + k] = lo[j];
        }
    for (size_t j = 0; j < ny; ++j)
        for (size_t k = 0; k < nz; ++k) {
            for (size_t i = 0; i < nx; ++i) li[i] = out[(i * ny + j) * nz + k];
            plan_exec(px, li, lo);
            for (size_t i = 0; i < nx; ++i) out[(i * ny + j) * nz + k] = lo[i];
        }
}

static size_t max3(size_t a, size_t b, size_t c) { return a > b ? (a > c ? a : c) : (b > c ? b : c); }

int orc_fft3d(size_t nx, size_t ny, size_t nz, int inverse, const double *in, double *out)
{
    fft_plan px, py, pz;
    if (plan_init(&px, nx, inverse) || plan_init(&py, ny, inverse) || plan_init(&pz, nz, inverse)) return -1;
    const size_t m = max3(nx, ny, nz);
    cplx *li = (cplx *)malloc(sizeof(cplx) * m), *lo = (cplx *)malloc(sizeof(cplx) * m);
    fft3d_exec(&px, &py, &pz, nx, ny, nz, (const cplx *)in, (cplx *)out, li, lo);
    free(li); free(lo);
    plan_free(&px); plan_free(&py); plan_free(&pz);
    return 0;
}

typedef struct {
    size_t nx, ny, nz, n;
    int order;
    fft_plan fx, fy, fz, ix, iy, iz;
    cplx *ft, *li, *lo;
    cplx *ev[2];
    cplx *et[2];
} ev3d;

static void ev3d_free(ev3d *e)
{
    plan_free(&e->fx); plan_free(&e->fy); plan_free(&e->fz);
    plan_free(&e->ix); plan_free(&e->iy); plan_free(&e->iz);
    free(e->ft); free(e->li); free(e->lo);
    for (int k = 0; k < 2; ++k) { free(e->ev[k]); free(e->et[k]); }
}

static int ev3d_init(ev3d *e, size_t nx, size_t ny, size_t nz, double dx, double dy, double dz, double mass,
                     double hbar, double dt_re, double dt_im, int order, const double *V)
{
    memset(e, 0, sizeof(*e));
    if (nx < 2 || ny < 2 || nz < 2 || (order != 2 && order != 4)) return -1;
    e->nx = nx; e->ny = ny; e->nz = nz; e->n = nx * ny * nz; e->order = order;
    if (plan_init(&e->fx, nx, 0) || plan_init(&e->fy, ny, 0) || plan_init(&e->fz, nz, 0) ||
        plan_init(&e->ix, nx, 1) || plan_init(&e->iy, ny, 1) || plan_init(&e->iz, nz, 1)) return -1;
    const size_t m = max3(nx, ny, nz);
    e->ft = (cplx *)malloc(sizeof(cplx) * e->n);
    e->li = (cplx *)malloc(sizeof(cplx) * m);
    e->lo = (cplx *)malloc(sizeof(cplx) * m);
    const cplx dt = dt_re + I * dt_im;
    double c1, c2, d1, d2;
    orc_splitting_constants(&c1, &c2, &d1, &d2);
    const double vc[2] = {order == 2 ? 0.5 : c1, c2};
    const double tc[2] = {order == 2 ? 1.0 : d1, d2};
    const int ntab = order == 2 ? 1 : 2;
    const double dkx = 2 * kPi / (dx * nx), dky = 2 * kPi / (dy * ny), dkz = 2 * kPi / (dz * nz);
    const double DTx = (dkx * hbar) * (dkx * hbar) / (2 * mass);
    const double DTy = (dky * hbar) * (dky * hbar) / (2 * mass);
    const double DTz = (dkz * hbar) * (dkz * hbar) / (2 * mass);
    const cplx alpha = -I * dt / hbar;
    for (int k = 0; k < ntab; ++k) {
        e->ev[k] = (cplx *)malloc(sizeof(cplx) * e->n);
        e->et[k] = (cplx *)malloc(sizeof(cplx) * e->n);
        const cplx f = expv_coef(dt, vc[k], hbar);
        for (size_t i = 0; i < e->n; ++i) e->ev[k][i] = cexp(f * V[i]);
        const cplx a = alpha * tc[k];
        for (size_t i = 0; i < nx; ++i) {
            const double fi = (double)fold_half(i, nx);
            for (size_t j = 0; j < ny; ++j) {
                const double fj = (double)fold_half(j, ny);
                for (size_t l = 0; l < nz; ++l) {
                    const double fl = (double)fold_half(l, nz);
                    e->et[k][(i * ny + j) * nz + l] = cexp(a * ((fi * fi) * DTx + (fj * fj) * DTy + (fl * fl) * DTz));
                }
            }
        }
    }
    return 0;
}

static void ev3d_expt(ev3d *e, cplx *psi, const cplx *tab)
{
    fft3d_exec(&e->fx, &e->fy, &e->fz, e->nx, e->ny, e->nz, psi, e->ft, e->li, e->lo);
    ev2d_mul(e->ft, tab, e->n);
    fft3d_exec(&e->ix, &e->iy, &e->iz, e->nx, e->ny, e->nz, e->ft, psi, e->li, e->lo);
    const double s = 1.0 / (double)e->n;
    for (size_t i = 0; i < e->n; ++i) psi[i] = psi[i] * s;
}

static void ev3d_step(ev3d *e, cplx *psi)
{
    if (e->order == 2) {
        ev2d_mul(psi, e->ev[0], e->n);
        ev3d_expt(e, psi, e->et[0]);
        ev2d_mul(psi, e->ev[0], e->n);
    } else {
        ev2d_mul(psi, e->ev[0], e->n);
        ev3d_expt(e, psi, e->et[0]);
        ev2d_mul(psi, e->ev[1], e->n);
        ev3d_expt(e, psi, e->et[1]);
        ev2d_mul(psi, e->ev[1], e->n);
        ev3d_expt(e, psi, e->et[0]);
        ev2d_mul(psi, e->ev[0], e->n);
    }
}

int orc_evolve3d(size_t nx, size_t ny, size_t nz, double dx, double dy, double dz, double mass, double hbar,
                 double dt_re, double dt_im, int order, double *psi_io, const double *V, uint64_t nsteps)
{
    ev3d e;
    if (ev3d_init(&e, nx, ny, nz, dx, dy, dz, mass, hbar, dt_re, dt_im, order, V)) { ev3d_free(&e); return -1; }
    for (uint64_t s = 0; s < nsteps; ++s) ev3d_step(&e, (cplx *)psi_io);
    ev3d_free(&e);
    return 0;
}

/* <T> = sum |FFT3D psi|^2 (fold(i)^2 DTx + fold(j)^2 DTy + fold(k)^2 DTz) / sum |FFT3D psi|^2 */
double orc_kinen3d(size_t nx, size_t ny, size_t nz, double dx, double dy, double dz, double mass, double hbar,
                   const double *psi_in)
{
    fft_plan px, py, pz;
    if (plan_init(&px, nx, 0) || plan_init(&py, ny, 0) || plan_init(&pz, nz, 0)) return NAN;
    const size_t n = nx * ny * nz, m = max3(nx, ny, nz);
    cplx *ft = (cplx *)malloc(sizeof(cplx) * n);
    cplx *li = (cplx *)malloc(sizeof(cplx) * m), *lo = (cplx *)malloc(sizeof(cplx) * m);
    fft3d_exec(&px, &py, &pz, nx, ny, nz, (const cplx *)psi_in, ft, li, lo);
    const double dkx = 2 * kPi / (dx * nx), dky = 2 * kPi / (dy * ny), dkz = 2 * kPi / (dz * nz);
    const double DTx = (dkx * hbar) * (dkx * hbar) / (2 * mass);
    const double DTy = (dky * hbar) * (dky * hbar) / (2 * mass);
    const double DTz = (dkz * hbar) * (dkz * hbar) / (2 * mass);
    double kin = 0;
    for (size_t i = 0; i < nx; ++i) {
        const double fi = (double)fold_half(i, nx);
        for (size_t j = 0; j < ny; ++j) {
            const double fj = (double)fold_half(j, ny);
            for (size_t l = 0; l < nz; ++l) {
                const double fl = (double)fold_half(l, nz);
                const cplx u = ft[(i * ny + j) * nz + l];
                kin += (creal(u) * creal(u) + cimag(u) * cimag(u)) * ((fi * fi) * DTx + (fj * fj) * DTy + (fl * fl) * DTz);
            }
        }
    }
    const double nn = norm2_raw(ft, n);
    free(ft); free(li); free(lo);
    plan_free(&px); plan_free(&py); plan_free(&pz);
    return kin / nn;
}
