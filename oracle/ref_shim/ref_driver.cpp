// Thin extern "C" driver over the reference's own SplittingMethod1D/2D and
// Born-series solvers QuPerturbation1DImpl/2DImpl, compiled from the reference sources in place (oracle/Makefile).  It is the
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
#include "Perturbation1DImpl.h"
#include "Perturbation2DImpl.h"
#include "OptionsImpl.h"
#include "Cal.h"
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

// KissFourierTransform3D (src/FourierTransform.cpp:379-440, created as
// FourierTransform3D::Create(n1, n2, n3) at :521-536): n1 = nx slowest, n3 = nz
// contiguous.
int ref_fft3d(size_t nx, size_t ny, size_t nz, int inverse, const double *in, double *out)
{
    try {
        std::unique_ptr<FourierTransform3D> f(FourierTransform3D::Create(nx, ny, nz, inverse != 0, FourierTransformLibrary::KISS));
        f->Transform((const Complex *)in, (Complex *)out);
        return 0;
    } catch (std::exception &) {
        return -1;
    }
}

// Born-series scattering solvers, driven as QuPerturbation1D/2D::init and
// Compute() drive them (src/QuSim.cpp:499-505, 620-630): the impl's
// InitPerturbation1D/2D (src/Perturbation1DImpl.cpp:7-42,
// src/Perturbation2DImpl.cpp:4-47) then `computes` Compute() calls.
// V: n complex (re,im) sampled at the grid points.  Outputs (each may be
// null): dpsi (the scattered part fPsiX), psi0, v (after the absorbing layer
// the preconditioned series adds), scal[0..2] = R, T, epsilon in use (1D) or
// delta-psi norm, epsilon in use (2D).  prec: null = the options' default.
static void born_opts(OptionsImpl &opts, int order, int preconditional, const char *prec, double slow)
{
    opts.SetInt("order", (Int)order);
    opts.SetReal("slow", slow);
    // OptionsImpl::GetBool(key, default) (src/OptionsImpl.cpp:88-91) returns
    // whether the key is present, not its value, so the key is set only when
    // the preconditioned series is wanted
    if (preconditional) opts.SetBool("preconditional", true);
    if (prec) opts.SetString("preconditioner", prec);
}

int ref_born1d(size_t n, double x0, double x1, const double *V, double en, double epsilon,
               double direction, double mass, double hbar, int order, int preconditional,
               const char *prec, double slow, int computes, double *dpsi, double *psi0,
               double *v, double *scal)
{
    try {
        OptionsImpl opts;
        born_opts(opts, order, preconditional, prec, slow);
        QuPerturbation1DImpl impl;
        const double dx = (x1 - x0) / n;
        Grid1 gv{x0, dx, n, V, nullptr};
        impl.InitPerturbation1D(gv, x0, x1, n, en, epsilon, direction, SolverMethod::BornSerise,
                                mass, hbar, opts);
        for (int c = 0; c < computes; ++c) impl.Compute();
        if (dpsi) std::memcpy(dpsi, impl.fPsiX, sizeof(double) * 2 * n);
        if (psi0) std::memcpy(psi0, impl.fPsi0X, sizeof(double) * 2 * n);
        if (v) std::memcpy(v, impl.fV, sizeof(double) * 2 * n);
        if (scal) {
            scal[0] = impl.fR;
            scal[1] = impl.fT;
            scal[2] = impl.fEpsilon;
        }
        return 0;
    } catch (std::exception &) {
        return -1;
    }
}

// xsec: ncos (cosx, cosy) pairs in, ComputeXSection of each out (after the
// last Compute); tot: ComputeTotalXSection(ntot) when ntot > 0.
int ref_born2d(size_t nx, size_t ny, double x0, double x1, double y0, double y1, const double *V,
               double en, double epsilon, double dirx, double diry, double mass, double hbar,
               int order, int preconditional, const char *prec, double slow, int computes,
               double *dpsi, double *psi0, double *v, double *scal, const double *cosxy,
               int ncos, double *xsec, int ntot, double *tot)
{
    try {
        OptionsImpl opts;
        born_opts(opts, order, preconditional, prec, slow);
        QuPerturbation2DImpl impl;
        const double dx = (x1 - x0) / nx, dy = (y1 - y0) / ny;
        Grid2 gv{x0, dx, y0, dy, nx, ny, V, nullptr};
        impl.InitPerturbation2D(gv, x0, x1, nx, y0, y1, ny, en, epsilon, dirx, diry,
                                SolverMethod::BornSerise, mass, hbar, opts);
        for (int c = 0; c < computes; ++c) impl.Compute();
        const size_t n = nx * ny;
        if (dpsi) std::memcpy(dpsi, impl.fPsiX, sizeof(double) * 2 * n);
        if (psi0) std::memcpy(psi0, impl.fPsi0X, sizeof(double) * 2 * n);
        if (v) std::memcpy(v, impl.fV, sizeof(double) * 2 * n);
        if (scal) {
            scal[0] = impl.fNormDeltaPsi;
            scal[1] = impl.fEpsilon;
        }
        for (int i = 0; i < ncos; ++i) xsec[i] = impl.ComputeXSection(cosxy[2 * i], cosxy[2 * i + 1]);
        if (ntot > 0 && tot) *tot = impl.ComputeTotalXSection(ntot);
        return 0;
    } catch (std::exception &) {
        return -1;
    }
}

// The reference's expression calculator (src/Cal.cpp): nvars variables
// names[i] = values[2i] + i values[2i + 1], then Val(); out = (re, im).
// Returns -1 (and leaves out) when the expression does not parse.
int ref_cal_eval(const char *expr, int nvars, const char *const *names, const double *values, double *out)
{
    try {
        Cal cal(expr);
        for (int i = 0; i < nvars; ++i) cal.SetVarVal(names[i], CCom(values[2 * i], values[2 * i + 1]));
        const CCom r = cal.Val();
        out[0] = r.real();
        out[1] = r.imag();
        return 0;
    } catch (std::exception &) {
        return -1;
    }
}

}  // extern "C"
