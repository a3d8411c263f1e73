// Thin extern "C" driver over the reference's own SplittingMethod1D/2D,
// compiled from the reference sources in place (oracle/Makefile).  It is the
// "reference" leg of the oracle: it validates the C restatement
// (oracle/qusim_oracle.c) and times the reference's CPU path.  Test
// infrastructure only.
//
// The evolvers are driven through QuEvolverImpl::Step()
// (src/EvolverImpl.cpp:56-68), exactly as Evolver::step() does
// (src/QuSim.cpp:39-42), with Options() defaults: device CPU_SEQ, KISS FFT,
// "batch" = the number of steps requested.
#include "SplittingMethod1D.h"
#include "SplittingMethod2D.h"
#include "OptionsImpl.h"
#include <cmath>
#include <cstdint>
#include <cstring>
#include <exception>

namespace {

// Sample a grid array through the reference's x -> value functor interface:
// InitPsi/InitPotential call the functor at x_i = x0 + i*dx
// (src/EvolverImpl.h:95-98), so the index is recovered by rounding.
struct Grid1 {
    double x0, dx; size_t n; const double *re_im; const double *real;
    Complex operator()(Real x) const {
        long long i = llround((x - x0) / dx);
        if (i < 0) i = 0;
        if ((size_t)i >= n) i = (long long)n - 1;
        if (re_im) return Complex(re_im[2 * i], re_im[2 * i + 1]);
        return Complex(real[i], 0);
    }
};
struct Grid2 {
    double x0, dx, y0, dy; size_t nx, ny; const double *re_im; const double *real;
    Complex operator()(Real x, Real y) const {
        long long i = llround((x - x0) / dx), j = llround((y - y0) / dy);
        if (i < 0) i = 0;
        if ((size_t)i >= nx) i = (long long)nx - 1;
        if (j < 0) j = 0;
        if ((size_t)j >= ny) j = (long long)ny - 1;
        size_t k = (size_t)i * ny + (size_t)j;
        if (re_im) return Complex(re_im[2 * k], re_im[2 * k + 1]);
        return Complex(real[k], 0);
    }
};

}  // namespace

extern "C" {

// psi_io: n complex (re,im) in/out.  Runs `calls` Step() calls of `batch`
// steps each; fnes renormalises after each call.  kin/pot/norm receive the
// reference's KinEn()/PotEn()/Norm2() after the run (may be null).
int ref_evolve1d(size_t n, double x0, double x1, double mass, double hbar,
                 double dt_re, double dt_im, int order, int wall, int fnes,
                 double *psi_io, const double *V, uint64_t batch, uint64_t calls,
                 double *norm, double *kin, double *pot)
{
    try {
        OptionsImpl opts;
        opts.SetInt("batch", (Int)batch);
        SplittingMethod1D sm;
        const double dx = (x1 - x0) / n;
        Grid1 gp{x0, dx, n, psi_io, nullptr}, gv{x0, dx, n, nullptr, V};
        sm.InitSystem1D(gp, false, Complex(dt_re, dt_im), fnes != 0, gv, x0, x1, n,
                        wall ? BoundaryCondition::InfiniteWall : BoundaryCondition::Period,
                        order == 4 ? SolverMethod::SplittingMethodO4 : SolverMethod::SplittingMethodO2,
                        mass, hbar, opts);
        for (uint64_t c = 0; c < calls; ++c) sm.Step();
        std::memcpy(psi_io, sm.fPsi, sizeof(double) * 2 * n);
        if (norm) *norm = sm.Norm2();
        if (kin) *kin = sm.KinEn();
        if (pot) *pot = sm.PotEn();
        return 0;
    } catch (std::exception &) {
        return -1;
    }
}

int ref_evolve2d(size_t nx, size_t ny, double x0, double x1, double y0, double y1,
                 double mass, double hbar, double dt_re, double dt_im, int order, int fnes,
                 double *psi_io, const double *V, uint64_t batch, uint64_t calls,
                 double *norm, double *kin, double *pot)
{
    try {
        OptionsImpl opts;
        opts.SetInt("batch", (Int)batch);
        SplittingMethod2D sm;
        const double dx = (x1 - x0) / nx, dy = (y1 - y0) / ny;
        Grid2 gp{x0, dx, y0, dy, nx, ny, psi_io, nullptr}, gv{x0, dx, y0, dy, nx, ny, nullptr, V};
        sm.InitSystem2D(gp, false, Complex(dt_re, dt_im), fnes != 0, gv, x0, x1, nx, y0, y1, ny,
                        BoundaryCondition::Period,
                        order == 4 ? SolverMethod::SplittingMethodO4 : SolverMethod::SplittingMethodO2,
                        mass, hbar, opts);
        for (uint64_t c = 0; c < calls; ++c) sm.Step();
        std::memcpy(psi_io, sm.fPsi, sizeof(double) * 2 * nx * ny);
        if (norm) *norm = sm.Norm2();
        if (kin) *kin = sm.KinEn();
        if (pot) *pot = sm.PotEn();
        return 0;
    } catch (std::exception &) {
        return -1;
    }
}

// The reference's FourierTransform1D/2D with the KISS backend
// (src/FourierTransform.cpp:130-146, 362-377).
int ref_fft1d(size_t n, int inverse, const double *in, double *out)
{
    try {
        std::unique_ptr<FourierTransform1D> f(FourierTransform1D::Create(n, inverse != 0, FourierTransformLibrary::KISS));
        f->Transform((const Complex *)in, (Complex *)out);
        return 0;
    } catch (std::exception &) {
        return -1;
    }
}

int ref_fft2d(size_t nx, size_t ny, int inverse, const double *in, double *out)
{
    try {
        std::unique_ptr<FourierTransform2D> f(FourierTransform2D::Create(nx, ny, inverse != 0, FourierTransformLibrary::KISS));
        f->Transform((const Complex *)in, (Complex *)out);
        return 0;
    } catch (std::exception &) {
        return -1;
    }
}

}  // extern "C"
