// C++ host API check (include/qusim_gb300/Evolver.h over libqsg.so): the
// reference's own precision-app scenario written against the reference-style
// API, switched to the GB300 device.  Prints one JSON line.
//
// Scenario (applications/QuEvol1DPrecision/QuSimPrecision.cpp:106-120):
// psi0 = gauss(x, -20, 5) * exp(I x) on [-100, 100), V = exp(-x^2), hbar = m = 1,
// evolved to t = 64; the transmitted probability Norm2(0, 100) is 0.15937744085.
#include <cmath>
#include <cstdio>
#include <stdexcept>

#include "qusim_gb300/Evolver.h"

using namespace qusim_gb300;

static Complex gauss(Real x, Real mu, Real sigma)
{
    const Real t = (x - mu) / sigma;
    return 1.0 / (std::sqrt(2 * 3.14159265358979323846) * sigma) * std::exp(-0.5 * t * t);
}

int main(int argc, char **argv)
{
    const bool mixed = argc > 1 && std::string(argv[1]) == "mixed";
    Options o;
    o.Gb300().Batch(100);
    if (mixed) o.PrecisionMixed();

    Evolver1D e;
    e.init([](Real x) { return gauss(x, -20, 5) * std::exp(Complex(0, 1) * x); }, true, 0.02, false,
           [](Real x) { return Complex(std::exp(-x * x), 0); }, -100, 100, 2048, BoundaryCondition::Period,
           SolverMethod::SplittingMethodO4, 1, 1, o);
    const double n0 = e.Norm2();
    while (e.Time() < 64 - 1e-9) e.step();
    const double trans = e.Norm2(0.0, 100.0);
    const double kin = e.KinEn(), pot = e.PotEn();
    const auto psi = e.GetPsi();

    // 2D: a packet in a bump, O2, force-normalised each step
    Evolver2D f;
    f.init([](Real x, Real y) { return std::exp(Complex(0, 1.5) * x) * std::exp(-((x + 5) * (x + 5) + y * y) / 16); },
           true, Complex(0.01, 0), true, [](Real x, Real y) { return Complex(std::exp(-(x * x + y * y) / 4), 0); },
           -25.6, 25.6, 256, -25.6, 25.6, 256, BoundaryCondition::Period, SolverMethod::SplittingMethodO2, 1, 1,
           Options().Gb300().Batch(10));
    for (int i = 0; i < 5; ++i) f.step();
    const double n2d = f.Norm2();

    bool threw = false;
    try {
        Evolver2D g;
        g.init([](Real, Real) { return Complex(1, 0); }, false, 0.01, false, [](Real, Real) { return Complex(0, 0); },
               0, 1, 128, 0, 1, 128, BoundaryCondition::InfiniteWall, SolverMethod::SplittingMethodO2, 1, 1,
               Options().Gb300());
    } catch (std::runtime_error &) {
        threw = true;
    }
    bool bad_device = false;
    try {
        Evolver1D g;
        g.init([](Real) { return Complex(1, 0); }, false, 0.01, false, [](Real) { return Complex(0, 0); }, 0, 1, 128,
               BoundaryCondition::Period, SolverMethod::SplittingMethodO2, 1, 1, Options());
    } catch (std::invalid_argument &) {
        bad_device = true;
    }
    // Born series through QuPerturbation1D / 2D: the preconditioned setting of
    // applications/QuScattering1DPrecision (QuScattering1DPrecision.cpp:211-215) on a
    // power-of-two grid, and a 2D case
    Options bo = Options().Gb300().Order(5).Preconditional(true);
    if (mixed) bo.PrecisionMixed();
    QuPerturbation1D per;
    per.init([](Real x) { return Complex(0.5 * std::exp(-x * x), 0); }, -100, 100, 2048, 0.5, 0.51, 1,
             SolverMethod::BornSerise, 1, 1, bo);
    per.Compute();
    const double R = per.GetR(), T = per.GetT(), eps = per.GetEpsilon();
    Options bo2 = Options().Gb300().Order(3).Preconditional(true).Hao2Preconditioner().Slow(0.5);
    if (mixed) bo2.PrecisionMixed();
    QuPerturbation2D per2;
    per2.init([](Real x, Real y) { return Complex(0.3 * std::exp(-(x * x + y * y) / 4), 0); }, -45, 45, 128, -45, 45,
              128, 2.0, 0.0, 1, 0, SolverMethod::BornSerise, 1, 1, bo2);
    per2.Compute();
    const double xs = per2.ComputeXSection(1, 0), dn = per2.GetDeltaPsiNorm();

    // the same tunnelling run with the reference's expression strings (FunctorWrapper)
    Evolver1D ex;
    ex.init(FunctorWrapper("gauss(x,-20,5)*exp(I*x)"), true, 0.02, false, FunctorWrapper("exp(-x*x)"), -100, 100,
            2048, BoundaryCondition::Period, SolverMethod::SplittingMethodO4, 1, 1, o);
    while (ex.Time() < 64 - 1e-9) ex.step();
    const double trans_expr = ex.Norm2(0.0, 100.0);
    Calculator cal("a*x^2 + I");
    cal.SetVaraible("a", 2.0);
    cal.SetVaraible("x", 3.0);
    const Complex calv = cal.Evaluate();

    std::printf("{\"norm0\": %.17g, \"time\": %.17g, \"transmission\": %.17g, \"kin\": %.17g, \"pot\": %.17g, "
                "\"psi0\": [%.17g, %.17g], \"norm2d\": %.17g, \"wall2d_throws\": %s, \"bad_device_throws\": %s, "
                "\"born_R\": %.17g, \"born_T\": %.17g, \"born_eps\": %.17g, \"born2d_xsec0\": %.17g, "
                "\"born2d_delta\": %.17g, \"transmission_expr\": %.17g, \"calculator\": [%.17g, %.17g]}\n",
                n0, e.Time(), trans, kin, pot, psi[0].real(), psi[0].imag(), n2d, threw ? "true" : "false",
                bad_device ? "true" : "false", R, T, eps, xs, dn, trans_expr, calv.real(), calv.imag());
    return 0;
}
