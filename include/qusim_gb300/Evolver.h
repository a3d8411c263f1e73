// qusim_gb300/Evolver.h -- C++ host API for the GPU_GB300 split-operator device.
//
// The same Evolver1D / Evolver2D / Options surface as the reference's
// include/QuSim.h (Evolver: QuSim.h:540-597, Options: QuSim.h:286-458), header
// only, calling libqsg.so through its C ABI (qsg.h).  A program written
// against the reference's split-operator path
//
//     Evolver1D e;
//     e.init(psi, true, dt, false, V, x0, x1, n, BoundaryCondition::Period,
//            SolverMethod::SplittingMethodO2, mass, hbar, Options().Batch(10));
//     e.step(); e.Norm2(); e.GetPsi(); ...
//
// switches to the GB300 engine with Options().Gb300() and this header.  As in
// the reference, psi and V are functors sampled on the host at
// x_i = x0 + i*dx (src/EvolverImpl1D.cpp:33-81, src/EvolverImpl2D.cpp:39-98),
// only the real part of V is kept, and errors are C++ exceptions:
// std::invalid_argument for a bad device / option, std::runtime_error for an
// unsupported solver or boundary condition and for engine failures.
#pragma once

#include <cmath>
#include <complex>
#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../qsg.h"

namespace qusim_gb300 {

using Real = double;
using Complex = std::complex<double>;

enum class BoundaryCondition { Period, InfiniteWall };
enum class SolverMethod { Unknown, SplittingMethodO2, SplittingMethodO4, BornSerise };

template <class T> struct VectorView {
    VectorView(T const *d, size_t s) : fData(d), fSize(s) {}
    T const *begin() const { return fData; }
    T const *end() const { return fData + fSize; }
    size_t size() const { return fSize; }
    T const &operator[](size_t i) const { return fData[i]; }
    T const &operator()(size_t i) const { return fData[i]; }

  private:
    T const *fData;
    size_t fSize;
};

// rows = x (nx), cols = y (ny), element (ix, iy) at iy + ix*ny (QuSim.h:47-52)
template <class T> struct MatrixView {
    MatrixView(T const *d, size_t rows, size_t cols) : fData(d), fRows(rows), fCols(cols) {}
    T const *data() const { return fData; }
    size_t size() const { return fRows * fCols; }
    size_t rows() const { return fRows; }
    size_t cols() const { return fCols; }
    T const &operator()(size_t row, size_t col) const { return fData[col + row * fCols]; }

  private:
    T const *fData;
    size_t fRows, fCols;
};

// Key/value options as in the reference.  Keys read here:
//   "device"       must be "GPU_GB300" (Gb300())
//   "batch"        steps per step() call (QuSim.h:386-390, EvolverImpl.cpp:19)
//   "precision"    "fp64" (default) or "mixed"
//   "hbm_budget"   device-memory bound of the context in bytes (0 = none)
//   "device_ordinal"
//   Born-series solvers (QuSim.h:288-333): "order", "preconditional",
//   "preconditioner" ("Vellekoop", "Hao1", "Hao2", "BornIndentity"), "slow"
struct Options {
    Options &Gb300() { return SetString("device", "GPU_GB300"); }
    Options &Order(int64_t n) { return SetInt("order", n); }
    Options &Preconditional(bool v) { return SetInt("preconditional", v ? 1 : 0); }
    Options &Slow(double v) { return SetReal("slow", v); }
    Options &VellekoopPreconditioner() { return SetString("preconditioner", "Vellekoop"); }
    Options &Hao1Preconditioner() { return SetString("preconditioner", "Hao1"); }
    Options &Hao2Preconditioner() { return SetString("preconditioner", "Hao2"); }
    Options &BornIdentityPreconditioner() { return SetString("preconditioner", "BornIndentity"); }
    Options &SetReal(char const *k, double v)
    {
        fReals[k] = v;
        return *this;
    }
    double GetReal(char const *k, double dflt) const
    {
        auto it = fReals.find(k);
        return it == fReals.end() ? dflt : it->second;
    }
    Options &Batch(int64_t n) { return SetInt("batch", n); }
    Options &PrecisionFp64() { return SetString("precision", "fp64"); }
    Options &PrecisionMixed() { return SetString("precision", "mixed"); }
    // complex64 2D state form (qsg_set_form): "momentum" (default) or "direct"
    Options &FormMomentum() { return SetString("form", "momentum"); }
    Options &FormDirect() { return SetString("form", "direct"); }
    Options &HbmBudget(int64_t bytes) { return SetInt("hbm_budget", bytes); }
    Options &DeviceOrdinal(int64_t i) { return SetInt("device_ordinal", i); }
    Options &SetInt(char const *k, int64_t v)
    {
        fInts[k] = v;
        return *this;
    }
    Options &SetString(char const *k, char const *v)
    {
        fStrings[k] = v;
        return *this;
    }
    int64_t GetInt(char const *k, int64_t dflt) const
    {
        auto it = fInts.find(k);
        return it == fInts.end() ? dflt : it->second;
    }
    std::string GetString(char const *k, std::string const &dflt) const
    {
        auto it = fStrings.find(k);
        return it == fStrings.end() ? dflt : it->second;
    }

  private:
    std::map<std::string, int64_t> fInts;
    std::map<std::string, std::string> fStrings;
    std::map<std::string, double> fReals;
};

namespace detail {

inline void check(int rc)
{
    if (rc != QSG_OK) throw std::runtime_error(std::string("qsg: ") + qsg_last_error());
}

// one context per (device, budget), shared by the evolvers of a process
inline std::shared_ptr<qsg_ctx> context(int device, int64_t budget)
{
    static std::map<std::pair<int, int64_t>, std::weak_ptr<qsg_ctx>> cache;
    auto key = std::make_pair(device, budget);
    if (auto p = cache[key].lock()) return p;
    qsg_ctx *c = nullptr;
    check(qsg_init(device, (size_t)budget, &c));
    std::shared_ptr<qsg_ctx> p(c, qsg_ctx_destroy);
    cache[key] = p;
    return p;
}

inline int device_precision(Options const &o)
{
    const std::string dev = o.GetString("device", "CPU_SEQ");
    if (dev != "GPU_GB300")
        throw std::invalid_argument("invalid device: " + dev + " (this library serves GPU_GB300; use Options().Gb300())");
    const std::string p = o.GetString("precision", "fp64");
    if (p == "fp64") return QSG_FP64;
    if (p == "mixed") return QSG_MIXED;
    throw std::invalid_argument("invalid precision: " + p);
}

inline int order_of(SolverMethod s)
{
    if (s == SolverMethod::SplittingMethodO2) return 2;
    if (s == SolverMethod::SplittingMethodO4) return 4;
    throw std::runtime_error("unspported solver");
}

}  // namespace detail

// The reference's expression calculator API (include/QuSim.h:502-538) over
// qsg_expr_eval: the same language (src/Cal.cpp), evaluated by libqsg.so on
// the host.  A FunctorWrapper / Functor2DWrapper can be passed to
// Evolver1D / Evolver2D::init wherever a functor is taken.
class Calculator {
public:
    explicit Calculator(char const *expr) : fExpr(expr)
    {
        // syntax errors throw here, as the reference's constructor does; an
        // undefined variable waits until Evaluate
        double out[2];
        const int rc = qsg_expr_eval(fExpr.c_str(), 0, nullptr, nullptr, out);
        if (rc != QSG_OK && std::string(qsg_last_error()).find("var not defined") == std::string::npos)
            detail::check(rc);
    }
    Calculator(Calculator const &) = delete;
    Calculator &operator=(Calculator const &) = delete;
    Complex &SetVaraible(char const *name, Complex v)
    {
        fVars[name] = v;
        return fVars[name];
    }
    Complex &GetVaraible(char const *name) { return fVars.at(name); }
    Complex Evaluate()
    {
        std::vector<char const *> names;
        std::vector<double> vals;
        for (auto const &kv : fVars) {
            names.push_back(kv.first.c_str());
            vals.push_back(kv.second.real());
            vals.push_back(kv.second.imag());
        }
        double out[2];
        detail::check(qsg_expr_eval(fExpr.c_str(), (int)names.size(), names.data(), vals.data(), out));
        return Complex(out[0], out[1]);
    }

private:
    std::string fExpr;
    std::map<std::string, Complex> fVars;
};

struct FunctorWrapper {
    explicit FunctorWrapper(char const *expr) : fCal(std::make_shared<Calculator>(expr)) {}
    Complex operator()(Real x) const
    {
        fCal->SetVaraible("x", x);
        return fCal->Evaluate();
    }

private:
    std::shared_ptr<Calculator> fCal;
};

struct Functor2DWrapper {
    explicit Functor2DWrapper(char const *expr) : fCal(std::make_shared<Calculator>(expr)) {}
    Complex operator()(Real x, Real y) const
    {
        fCal->SetVaraible("x", x);
        fCal->SetVaraible("y", y);
        return fCal->Evaluate();
    }

private:
    std::shared_ptr<Calculator> fCal;
};

class Evolver {
  public:
    Evolver(Evolver const &) = delete;
    Evolver &operator=(Evolver const &) = delete;
    virtual ~Evolver()
    {
        if (fInst) qsg_destroy(fInst);
    }

    // Evolver::step (QuSim.cpp:39-42 -> EvolverImpl.cpp:56-68): `batch` steps,
    // then renormalise when force_normalization_each_step.
    void step()
    {
        detail::check(qsg_step(fInst, (uint64_t)fBatch, fFNES ? 1 : 0));
        fPsiValid = false;
    }
    Real Norm2()
    {
        double v;
        detail::check(qsg_norm2(fInst, &v));
        return v;
    }
    Real Time()
    {
        uint64_t s;
        detail::check(qsg_steps_taken(fInst, &s));
        return (double(s) * fDt).real();
    }
    Real PotEn()
    {
        double p;
        detail::check(qsg_energies(fInst, nullptr, &p));
        return p;
    }
    Real KinEn()
    {
        double k;
        detail::check(qsg_energies(fInst, &k, nullptr));
        return k;
    }
    SolverMethod GetMethod() { return fMethod; }

  protected:
    Evolver() = default;

    void Setup(Complex dt, bool fnes, SolverMethod solver, Options const &opts, int *prec, int *order)
    {
        *prec = detail::device_precision(opts);
        *order = detail::order_of(solver);
        fCtx = detail::context((int)opts.GetInt("device_ordinal", 0), opts.GetInt("hbm_budget", 0));
        fDt = dt;
        fFNES = fnes;
        fBatch = opts.GetInt("batch", 1);
        fMethod = solver;
    }
    void FetchPsi()
    {
        if (!fPsiValid) {
            detail::check(qsg_get_psi(fInst, reinterpret_cast<double *>(fPsiHost.data())));
            fPsiValid = true;
        }
    }

    std::shared_ptr<qsg_ctx> fCtx;
    qsg_inst *fInst = nullptr;
    Complex fDt;
    bool fFNES = false;
    int64_t fBatch = 1;
    SolverMethod fMethod = SolverMethod::Unknown;
    std::vector<Complex> fPsiHost;
    std::vector<Real> fVHost;
    bool fPsiValid = false;
};

class Evolver1D : public Evolver {
  public:
    Evolver1D() = default;

    void init(std::function<Complex(Real)> const &psi, bool force_normalization, Complex dt,
              bool force_normalization_each_step, std::function<Complex(Real)> const &v, Real x0,
              Real x1, size_t n, BoundaryCondition b, SolverMethod solver, Real mass, Real hbar,
              Options const &opts)
    {
        int prec, order;
        Setup(dt, force_normalization_each_step, solver, opts, &prec, &order);
        fX0 = x0;
        fX1 = x1;
        fN = n;
        fDx = (x1 - x0) / n;
        fPsiHost.resize(n);
        fVHost.resize(n);
        for (size_t i = 0; i < n; ++i) {
            const Real x = fDx * i + x0;
            fPsiHost[i] = psi(x);
            fVHost[i] = v(x).real();
        }
        if (force_normalization) {
            double s = 0;
            for (auto const &c : fPsiHost) s += std::norm(c);
            const double sc = 1.0 / std::sqrt(s * fDx);
            for (auto &c : fPsiHost) c *= sc;
        }
        const int bc = b == BoundaryCondition::Period ? QSG_PERIOD : QSG_INFINITE_WALL;
        detail::check(qsg_create_1d(fCtx.get(), n, fDx, mass, hbar, dt.real(), dt.imag(), order, prec, bc,
                                    reinterpret_cast<double const *>(fPsiHost.data()), fVHost.data(), &fInst));
        fPsiValid = true;
    }

    VectorView<Complex> GetPsi()
    {
        FetchPsi();
        return VectorView<Complex>(fPsiHost.data(), fN);
    }
    VectorView<Real> GetV() { return VectorView<Real>(fVHost.data(), fN); }
    Real Xavg()
    {
        double v;
        detail::check(qsg_xavg(fInst, fX0, &v));
        return v;
    }
    size_t GetN() { return fN; }
    Real GetX0() { return fX0; }
    Real GetX1() { return fX1; }
    using Evolver::Norm2;
    Real Norm2(Real xa, Real xb)
    {
        double v;
        detail::check(qsg_norm2_range(fInst, fX0, xa, xb, &v));
        return v;
    }

  private:
    Real fX0 = 0, fX1 = 0, fDx = 0;
    size_t fN = 0;
};

class Evolver2D : public Evolver {
  public:
    Evolver2D() = default;

    void init(std::function<Complex(Real, Real)> const &psi, bool force_normalization, Complex dt,
              bool force_normalization_each_step, std::function<Complex(Real, Real)> const &v, Real x0,
              Real x1, size_t nx, Real y0, Real y1, size_t ny, BoundaryCondition b, SolverMethod solver,
              Real mass, Real hbar, Options const &opts)
    {
        int prec, order;
        Setup(dt, force_normalization_each_step, solver, opts, &prec, &order);
        if (b != BoundaryCondition::Period) throw std::runtime_error("unsupported boundary condition!");
        fNx = nx;
        fNy = ny;
        const Real dx = (x1 - x0) / nx, dy = (y1 - y0) / ny;
        fPsiHost.resize(nx * ny);
        fVHost.resize(nx * ny);
        for (size_t i = 0; i < nx; ++i)
            for (size_t j = 0; j < ny; ++j) {
                const Real x = dx * i + x0, y = dy * j + y0;
                fPsiHost[j + i * ny] = psi(x, y);
                fVHost[j + i * ny] = v(x, y).real();
            }
        if (force_normalization) {
            double s = 0;
            for (auto const &c : fPsiHost) s += std::norm(c);
            const double sc = 1.0 / std::sqrt(s * dx * dy);
            for (auto &c : fPsiHost) c *= sc;
        }
        detail::check(qsg_create_2d(fCtx.get(), nx, ny, dx, dy, mass, hbar, dt.real(), dt.imag(), order, prec,
                                    reinterpret_cast<double const *>(fPsiHost.data()), fVHost.data(), &fInst));
        if (prec == QSG_MIXED && opts.GetString("form", "momentum") == "direct")
            detail::check(qsg_set_form(fInst, QSG_FORM_DIRECT));
        fPsiValid = true;
    }

    MatrixView<Complex> GetPsi()
    {
        FetchPsi();
        return MatrixView<Complex>(fPsiHost.data(), fNx, fNy);
    }
    MatrixView<Real> GetV() { return MatrixView<Real>(fVHost.data(), fNx, fNy); }
    size_t GetNx() { return fNx; }
    size_t GetNy() { return fNy; }

  private:
    size_t fNx = 0, fNy = 0;
};

// ---------------------------------------------------------------------------
// Born-series scattering solvers: QuPerturbation1D / QuPerturbation2D
// (QuSim.h:643-806), over qsg_born_*.  As in the reference, V is a functor
// sampled at x_i = x0 + i*dx (complex: the absorbing layer of the
// preconditioned series goes into its imaginary part).  One difference: the
// reference's OptionsImpl::GetBool(key, default) returns whether the key is
// present (src/OptionsImpl.cpp:88-91), so there Preconditional(false) selects
// the preconditioned series; here the value is used.
// ---------------------------------------------------------------------------

namespace detail {
inline qsg_born_opts born_opts(Options const &o)
{
    qsg_born_opts b;
    qsg_born_default_opts(&b);
    b.order = (int)o.GetInt("order", 1);
    b.preconditional = (int)o.GetInt("preconditional", 0);
    b.slow = o.GetReal("slow", 1.0);
    const std::string p = o.GetString("preconditioner", "Vellekoop");
    if (p == "Vellekoop") b.preconditioner = QSG_BORN_VELLEKOOP;
    else if (p == "Hao1") b.preconditioner = QSG_BORN_HAO1;
    else if (p == "Hao2") b.preconditioner = QSG_BORN_HAO2;
    else if (p == "BornIndentity") b.preconditioner = QSG_BORN_IDENTITY;
    else throw std::runtime_error("Unknown preconditioner");
    return b;
}
}  // namespace detail

class QuScatteringProblemSolver {
  public:
    QuScatteringProblemSolver(QuScatteringProblemSolver const &) = delete;
    QuScatteringProblemSolver &operator=(QuScatteringProblemSolver const &) = delete;
    virtual ~QuScatteringProblemSolver()
    {
        if (fBorn) qsg_born_destroy(fBorn);
    }
    void Compute()
    {
        detail::check(qsg_born_compute(fBorn));
        fPsiValid = false;
    }
    Real GetEnergy() { return fE; }
    Real GetMomentum() { return std::sqrt(2 * fMass * fE); }
    SolverMethod GetMethod() { return SolverMethod::BornSerise; }
    Real GetEpsilon()
    {
        double e;
        detail::check(qsg_born_epsilon(fBorn, &e));
        return e;
    }

  protected:
    QuScatteringProblemSolver() = default;
    int Setup(SolverMethod met, Real en, Real mass, Real hbar, Options const &opts)
    {
        if (met != SolverMethod::BornSerise) throw std::runtime_error("not support method!");
        const int prec = detail::device_precision(opts);
        fCtx = detail::context((int)opts.GetInt("device_ordinal", 0), opts.GetInt("hbm_budget", 0));
        fE = en;
        fMass = mass;
        fHbar = hbar;
        return prec;
    }
    void Fetch(int what, std::vector<Complex> &dst)
    {
        detail::check(qsg_born_get(fBorn, what, reinterpret_cast<double *>(dst.data())));
    }

    std::shared_ptr<qsg_ctx> fCtx;
    qsg_born *fBorn = nullptr;
    Real fE = 0, fMass = 1, fHbar = 1;
    std::vector<Complex> fPsi, fPsi0, fV;
    bool fPsiValid = false;
};

class QuPerturbation1D : public QuScatteringProblemSolver {
  public:
    QuPerturbation1D() = default;
    void init(std::function<Complex(Real)> const &v, Real x0, Real x1, size_t n, Real en, Real epsilon,
              Real direction, SolverMethod met, Real mass, Real hbar, Options const &opts)
    {
        const int prec = Setup(met, en, mass, hbar, opts);
        fN = n;
        fDx = (x1 - x0) / n;
        std::vector<Complex> V(n);
        for (size_t i = 0; i < n; ++i) V[i] = v(x0 + fDx * i);
        const qsg_born_opts o = detail::born_opts(opts);
        detail::check(qsg_born_create_1d(fCtx.get(), n, x0, x1, reinterpret_cast<double const *>(V.data()), en,
                                         epsilon, direction, mass, hbar, &o, prec, &fBorn));
        fPsi.resize(n);
        fPsi0.resize(n);
        fV.resize(n);
        Fetch(QSG_BORN_PSI0, fPsi0);
        Fetch(QSG_BORN_V, fV);
    }
    VectorView<Complex> GetPsi()
    {
        if (!fPsiValid) {
            Fetch(QSG_BORN_PSI, fPsi);
            fPsiValid = true;
        }
        return VectorView<Complex>(fPsi.data(), fN);
    }
    VectorView<Complex> GetPsi0() { return VectorView<Complex>(fPsi0.data(), fN); }
    VectorView<Complex> GetV() { return VectorView<Complex>(fV.data(), fN); }
    size_t GetNPoints() { return fN; }
    Real GetT()
    {
        double r, t;
        detail::check(qsg_born_rt(fBorn, &r, &t));
        return t;
    }
    Real GetR()
    {
        double r, t;
        detail::check(qsg_born_rt(fBorn, &r, &t));
        return r;
    }
    // src/Perturbation1DImpl.h:22-61
    Real GetMaxMomentum() { return 2 * M_PI / fDx * fHbar; }
    Real GetMaxEnergy() { return 0.5 * GetMaxMomentum() * GetMaxMomentum() / fMass; }
    Real GetMomentumGap() { return 2 * M_PI / (fDx * fN) * fHbar; }
    Real GetEpsilonMomentumWidth() { return fMass * std::abs(GetEpsilon()) / std::sqrt(2 * fMass * fE); }
    Real GetEnergyGap() { return std::sqrt(2 * fMass * fE) / fMass * GetMomentumGap(); }
    Real GetEpsilonDecayLength() { return 2 * M_PI / (GetMomentum() / fHbar * GetEpsilon() / (2 * fE)); }
    Real GetEpsilonBoundaryError()
    {
        return std::exp(-(fN * fDx / 2) * (GetMomentum() / fHbar) * GetEpsilon() / (2 * fE));
    }

  private:
    size_t fN = 0;
    Real fDx = 0;
};

class QuPerturbation2D : public QuScatteringProblemSolver {
  public:
    QuPerturbation2D() = default;
    void init(std::function<Complex(Real, Real)> const &v, Real x0, Real x1, size_t nx, Real y0, Real y1, size_t ny,
              Real en, Real epsilon, Real directionx, Real directiony, SolverMethod met, Real mass, Real hbar,
              Options const &opts)
    {
        const int prec = Setup(met, en, mass, hbar, opts);
        fNx = nx;
        fNy = ny;
        const Real dx = (x1 - x0) / nx, dy = (y1 - y0) / ny;
        std::vector<Complex> V(nx * ny);
        for (size_t i = 0; i < nx; ++i)
            for (size_t j = 0; j < ny; ++j) V[j + i * ny] = v(x0 + dx * i, y0 + dy * j);
        const qsg_born_opts o = detail::born_opts(opts);
        detail::check(qsg_born_create_2d(fCtx.get(), (int)nx, (int)ny, x0, x1, y0, y1,
                                         reinterpret_cast<double const *>(V.data()), en, epsilon, directionx,
                                         directiony, mass, hbar, &o, prec, &fBorn));
        fPsi.resize(nx * ny);
        fPsi0.resize(nx * ny);
        fV.resize(nx * ny);
        Fetch(QSG_BORN_PSI0, fPsi0);
        Fetch(QSG_BORN_V, fV);
    }
    MatrixView<Complex> GetPsi()
    {
        if (!fPsiValid) {
            Fetch(QSG_BORN_PSI, fPsi);
            fPsiValid = true;
        }
        return MatrixView<Complex>(fPsi.data(), fNx, fNy);
    }
    MatrixView<Complex> GetPsi0() { return MatrixView<Complex>(fPsi0.data(), fNx, fNy); }
    MatrixView<Complex> GetV() { return MatrixView<Complex>(fV.data(), fNx, fNy); }
    Real ComputeXSection(Real cosx, Real cosy)
    {
        const double cs[2] = {cosx, cosy};
        double out;
        detail::check(qsg_born_xsection(fBorn, 1, cs, &out));
        return out;
    }
    Real ComputeTotalXSection(int64_t n)
    {
        double out;
        detail::check(qsg_born_total_xsection(fBorn, (int)n, &out));
        return out;
    }
    Real GetDeltaPsiNorm()
    {
        double out;
        detail::check(qsg_born_delta_norm(fBorn, &out));
        return out;
    }

  private:
    size_t fNx = 0, fNy = 0;
};

}  // namespace qusim_gb300
