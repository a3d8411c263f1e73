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
enum class SolverMethod { Unknown, SplittingMethodO2, SplittingMethodO4 };

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
struct Options {
    Options &Gb300() { return SetString("device", "GPU_GB300"); }
    Options &Batch(int64_t n) { return SetInt("batch", n); }
    Options &PrecisionFp64() { return SetString("precision", "fp64"); }
    Options &PrecisionMixed() { return SetString("precision", "mixed"); }
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
        throw std::invalid_argument("invalid device: " + dev + " (this build serves GPU_GB300; use Options().Gb300())");
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

}  // namespace qusim_gb300
