// ref_binding.cpp -- the binding a maintainer of the reference adds to select
// the GB300 engine (libqsg.so) from inside QuSim, compiled against the
// reference's own unmodified headers and linked with its own objects.
//
// The reference picks the evolver implementation in Evolver1D::init /
// Evolver2D::init (src/QuSim.cpp:90-100, 161-169) and the device from the
// Options key "device" (src/DeviceType.h:9-22).  Its plugin point is the
// QuEvolverImpl virtual interface (src/EvolverImpl.h:54-57): Step,
// UpdatePsi, CalKinEn, CalPotEn.  This file holds
//   - SplittingMethodGb300_1D / _2D: QuEvolver1DImpl / QuEvolver2DImpl
//     subclasses whose hot-path virtuals forward to the C ABI (include/qsg.h);
//     the base classes still sample psi0 and V on the host exactly as before
//     (src/EvolverImpl1D.cpp:33-81, src/EvolverImpl2D.cpp:39-98), on a CPU_SEQ
//     device, so fPsi / fPsiHost stay the host view GetPsi() returns;
//   - make_impl_1d / make_impl_2d: the implementation choice of Evolver1D::init
//     and Evolver2D::init with the one added branch for "device" = "GPU_GB300".
//     In the reference itself that branch goes into src/QuSim.cpp, and
//     DeviceType (src/Device.h) / GetDeviceType (src/DeviceType.h) gain
//     GPU_GB300; compiled here against the unmodified headers, the new device
//     is recognised by its string before GetDeviceType sees it.
//
// main() drives an implementation the way Evolver::step() does
// (src/QuSim.cpp:39-42, QuEvolverImpl::Step per call), on the reference's
// tunnelling scenario (applications/QuEvol1DPrecision/QuSimPrecision.cpp:
// 106-120) and a 2D packet, and prints one JSON line:
//   ref_binding <device> [fp64|mixed]
// With device CPU_SEQ the reference's own SplittingMethod1D/2D run; with
// GPU_GB300 the engine does, and without a GPU its error comes back as the
// std::runtime_error the reference raises for device failures.
#include <cmath>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>

#include "DeviceType.h"
#include "EvolverImpl.h"
#include "OptionsImpl.h"
#include "SplittingMethod1D.h"
#include "SplittingMethod2D.h"
#include "qsg.h"

namespace {

void check(int rc)
{
    if (rc) throw std::runtime_error(std::string("GPU_GB300: ") + qsg_last_error());
}

bool is_gb300(OptionsImpl const &opts) { return opts.GetString("device", std::string("CPU_SEQ")) == "GPU_GB300"; }

// the engine's precision and 2D form from the options ("precision": "fp64" |
// "mixed"; "form": "momentum" | "direct")
int precision_of(OptionsImpl const &opts)
{
    return opts.GetString("precision", std::string("fp64")) == "mixed" ? QSG_MIXED : QSG_FP64;
}

// the base classes sample on a CPU_SEQ device: psi0 / V land in host memory
OptionsImpl host_options(OptionsImpl const &opts)
{
    OptionsImpl host = opts;
    host.SetString("device", "CPU_SEQ");
    return host;
}

int order_of(SolverMethod solver) { return solver == SolverMethod::SplittingMethodO4 ? 4 : 2; }

}  // namespace

struct SplittingMethodGb300_1D : QuEvolver1DImpl {
    qsg_ctx *fCtx = nullptr;
    qsg_inst *fInst = nullptr;

    void InitSystem1D(std::function<Complex(Real)> const &psi, bool force_normalization, Complex dt,
                      bool force_normalization_each_step, std::function<Complex(Real)> const &v, Real x0, Real x1,
                      size_t n, BoundaryCondition b, SolverMethod solver, Real mass, Real hbar,
                      OptionsImpl const &opts) override
    {
        QuEvolver1DImpl::InitSystem1D(psi, force_normalization, dt, force_normalization_each_step, v, x0, x1, n, b,
                                      solver, mass, hbar, host_options(opts));
        check(qsg_init((int)opts.GetInt("device_ordinal", 0), 0, &fCtx));
        check(qsg_create_1d(fCtx, n, fDx, mass, hbar, dt.real(), dt.imag(), order_of(solver), precision_of(opts),
                            b == BoundaryCondition::InfiniteWall ? QSG_INFINITE_WALL : QSG_PERIOD,
                            reinterpret_cast<double const *>(fPsi), fV, &fInst));
    }
    // QuEvolverImpl::Step (src/EvolverImpl.cpp:56-68): fBatchSize steps, the
    // renormalisation when force_normalization_each_step, the host copy
    void Step() override
    {
        check(qsg_step(fInst, fBatchSize, fFNES ? 1 : 0));
        fStep += fBatchSize;
        check(qsg_get_psi(fInst, reinterpret_cast<double *>(fPsi)));
    }
    void UpdatePsi() override
    {
        check(qsg_step(fInst, fBatchSize, 0));
        fStep += fBatchSize;
    }
    Real CalKinEn() const override
    {
        double k = 0;
        check(qsg_energies(fInst, &k, nullptr));
        return k;
    }
    Real CalPotEn() const override
    {
        double p = 0;
        check(qsg_energies(fInst, nullptr, &p));
        return p;
    }
    ~SplittingMethodGb300_1D()
    {
        qsg_destroy(fInst);
        qsg_ctx_destroy(fCtx);
    }
};

struct SplittingMethodGb300_2D : QuEvolver2DImpl {
    qsg_ctx *fCtx = nullptr;
    qsg_inst *fInst = nullptr;

    void InitSystem2D(std::function<Complex(Real, Real)> const &psi, bool force_normalization, Complex dt,
                      bool force_normalization_each_step, std::function<Complex(Real, Real)> const &v, Real x0,
                      Real x1, size_t nx, Real y0, Real y1, size_t ny, BoundaryCondition b, SolverMethod solver,
                      Real mass, Real hbar, OptionsImpl const &opts) override
    {
        // periodic only, as SplittingMethod2D (src/SplittingMethod2D.cpp:21-29)
        if (b != BoundaryCondition::Period) throw std::runtime_error("unsupported boundary condition");
        QuEvolver2DImpl::InitSystem2D(psi, force_normalization, dt, force_normalization_each_step, v, x0, x1, nx, y0,
                                      y1, ny, b, solver, mass, hbar, host_options(opts));
        check(qsg_init((int)opts.GetInt("device_ordinal", 0), 0, &fCtx));
        check(qsg_create_2d(fCtx, nx, ny, fDx, fDy, mass, hbar, dt.real(), dt.imag(), order_of(solver),
                            precision_of(opts), reinterpret_cast<double const *>(fPsi), fV, &fInst));
        if (precision_of(opts) == QSG_MIXED && opts.GetString("form", std::string("momentum")) == "direct")
            check(qsg_set_form(fInst, QSG_FORM_DIRECT));
    }
    void Step() override
    {
        check(qsg_step(fInst, fBatchSize, fFNES ? 1 : 0));
        fStep += fBatchSize;
        check(qsg_get_psi(fInst, reinterpret_cast<double *>(fPsi)));
    }
    void UpdatePsi() override
    {
        check(qsg_step(fInst, fBatchSize, 0));
        fStep += fBatchSize;
    }
    Real CalKinEn() const override
    {
        double k = 0;
        check(qsg_energies(fInst, &k, nullptr));
        return k;
    }
    Real CalPotEn() const override
    {
        double p = 0;
        check(qsg_energies(fInst, nullptr, &p));
        return p;
    }
    ~SplittingMethodGb300_2D()
    {
        qsg_destroy(fInst);
        qsg_ctx_destroy(fCtx);
    }
};

// Evolver1D::init's choice (src/QuSim.cpp:90-100) for the split-operator
// solvers, with the GB300 branch; other devices go to GetDeviceType as before
// (an unknown one raises std::invalid_argument there)
QuEvolver1DImpl *make_impl_1d(SolverMethod solver, OptionsImpl const &opts)
{
    if (solver != SolverMethod::SplittingMethodO2 && solver != SolverMethod::SplittingMethodO4)
        throw std::runtime_error("unspported solver");
    if (is_gb300(opts)) return new SplittingMethodGb300_1D();
    GetDeviceType(opts);
    return new SplittingMethod1D();
}

// Evolver2D::init's choice (src/QuSim.cpp:161-169)
QuEvolver2DImpl *make_impl_2d(SolverMethod solver, OptionsImpl const &opts)
{
    if (solver != SolverMethod::SplittingMethodO2 && solver != SolverMethod::SplittingMethodO4)
        throw std::runtime_error("unsupported solver");
    if (is_gb300(opts)) return new SplittingMethodGb300_2D();
    GetDeviceType(opts);
    return new SplittingMethod2D();
}

namespace {

Complex gauss(Real x, Real mu, Real sigma)
{
    const Real t = (x - mu) / sigma;
    return 1.0 / (std::sqrt(2 * 3.14159265358979323846) * sigma) * std::exp(-0.5 * t * t);
}

}  // namespace

int main(int argc, char **argv)
{
    const std::string device = argc > 1 ? argv[1] : "CPU_SEQ";
    const std::string precision = argc > 2 ? argv[2] : "fp64";
    OptionsImpl opts;
    opts.SetString("device", device);
    opts.SetString("precision", precision);
    opts.SetInt("batch", 100);
    try {
        // the transmission scenario: t = 64 in 32 calls of 100 O4 steps
        std::unique_ptr<QuEvolver1DImpl> e(make_impl_1d(SolverMethod::SplittingMethodO4, opts));
        e->InitSystem1D([](Real x) { return gauss(x, -20, 5) * std::exp(Complex(0, 1) * x); }, true, 0.02, false,
                        [](Real x) { return Complex(std::exp(-x * x), 0); }, -100, 100, 2048,
                        BoundaryCondition::Period, SolverMethod::SplittingMethodO4, 1, 1, opts);
        const double norm0 = e->Norm2();
        while ((e->Time()).real() < 64 - 1e-9) e->Step();
        // Norm2(x0, x1), PotEn and KinEn of the reference's base class and virtuals
        const double trans = e->Norm2(0.0, 100.0);
        const double kin = e->KinEn(), pot = e->PotEn();

        // 2D: O2, force-normalised each step (QuEvolverImpl::Step's renormalisation)
        OptionsImpl o2 = opts;
        o2.SetInt("batch", 10);
        std::unique_ptr<QuEvolver2DImpl> f(make_impl_2d(SolverMethod::SplittingMethodO2, o2));
        f->InitSystem2D(
            [](Real x, Real y) { return std::exp(Complex(0, 1.5) * x) * std::exp(-((x + 5) * (x + 5) + y * y) / 16); },
            true, Complex(0.01, 0), true, [](Real x, Real y) { return Complex(std::exp(-(x * x + y * y) / 4), 0); },
            -25.6, 25.6, 256, -25.6, 25.6, 256, BoundaryCondition::Period, SolverMethod::SplittingMethodO2, 1, 1, o2);
        for (int i = 0; i < 5; ++i) f->Step();
        const double norm2d = f->Norm2(), kin2d = f->KinEn(), pot2d = f->PotEn();
        const Complex psi2d = f->fPsiHost[128 * 256 + 140];
        std::printf(
            "{\"device\": \"%s\", \"precision\": \"%s\", \"norm0\": %.17g, \"time\": %.17g, \"transmission\": %.17g, "
            "\"kin\": %.17g, \"pot\": %.17g, \"psi_1000_re\": %.17g, \"norm2d\": %.17g, \"kin2d\": %.17g, "
            "\"pot2d\": %.17g, \"psi2d_re\": %.17g, \"psi2d_im\": %.17g}\n",
            device.c_str(), precision.c_str(), norm0, e->Time().real(), trans, kin, pot, e->fPsiHost[1000].real(),
            norm2d, kin2d, pot2d, psi2d.real(), psi2d.imag());
    } catch (std::invalid_argument &ex) {
        std::printf("{\"device\": \"%s\", \"invalid_argument\": \"%s\"}\n", device.c_str(), ex.what());
    } catch (std::runtime_error &ex) {
        std::printf("{\"device\": \"%s\", \"runtime_error\": \"%s\"}\n", device.c_str(), ex.what());
    }
    return 0;
}
