// qsg_born_api.cu -- C ABI of the Born-series scattering solvers (include/qsg.h,
// qsg_born_*): set-up on the host as the reference does it, the update
// schedule on the device (qsg_born.cuh), observables.
//
// Set-up (FP64, host, once), as QuPerturbation1DImpl / 2DImpl::Init* and
// ScatteringSolver*Impl::Init* do it:
//   psi0 = exp(i k0 d.r), k0 = sqrt(2 m E) / hbar    (ScatteringSolverImpl.cpp:60-67, 154-163)
//   preconditioned: box >= 24 wavelengths, absorbing layer cal_v15 added to Im V
//   (Perturbation1DImpl.cpp:22-33, Perturbation2DImpl.cpp:22-38,
//   Perburbation.h:47-57, 80-95, 131-148), epsilon raised to GetEpsilon's
//   minimum (Perburbation.h:326-341)
// Compute (device), order K >= 1 (R = real-space pass, C = k-space pass):
//   2D:   R(dpsi -> pre -> F_y -> x split) then K times C(F_x, G0/N, F_x^-1)
//         and R([x split^-1 ->] F_y^-1 -> post [-> pre -> F_y -> x split]);
//         the last R also sums the
//         delta-psi norm.  dpsi ping-pongs between two buffers so the value at
//         the start of the compute survives until then (fLastPsiX,
//         Perturbation2DImpl.cpp:51).
//   1D:   n <= 8192 (complex64) / 4096 (complex128): one launch of k_born1d;
//         else the same schedule with the four-step passes; the last one sums
//         the reflection / transmission amplitudes (ComputeRT).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <string>
#include <vector>

#include "../../include/qsg.h"
#include "qsg_born_launch.h"
#include "qsg_host.h"

using namespace qsg_host;
using cd = std::complex<double>;

struct qsg_born {
    qsg_ctx *ctx = nullptr;
    int dim = 1, prec = 0;
    uint64_t n = 0;
    int nx = 0, ny = 1;
    int n1 = 0, n2 = 0;
    bool resident = false;
    double x0 = 0, x1 = 0, y0 = 0, y1 = 0, dx = 0, dy = 0;
    double en = 0, eps = 0, mass = 1, hbar = 1, k0 = 0, dirx = 1, diry = 0;
    qsg_born_opts opts{};
    qsg::BornOps ops{};
    bool needs_old = false;   // the post-update reads dpsi before the update
    void *dpsi[2] = {nullptr, nullptr};
    int cur = 0;
    void *tmp = nullptr, *psi0 = nullptr, *V = nullptr, *ex = nullptr, *ey = nullptr;
    double *gx = nullptr, *gy = nullptr;
    float2 *gx2 = nullptr, *gy2 = nullptr;  // hi + lo float forms
    const void *tw_a = nullptr, *tw_b = nullptr, *tw_n = nullptr;
    int g = 1;                 // 2D x split: column blocks of nx / g rows
    double *parts = nullptr;   // device partials of the last pass
    double *hparts = nullptr;  // pinned mirror
    int nparts = 0;            // doubles
    cudaEvent_t done = nullptr;
    bool pending = false, computed = false;
    double R = 0, T = 0, delta = 0;
    std::vector<cd> vhost, psi0host;  // V (with the layer) and, in 1D, psi0, in FP64
    // cross-section scratch (lazily allocated)
    double2 *xs_tab = nullptr;
    double *xs_parts = nullptr, *xs_hparts = nullptr;
    std::vector<void *> allocs;
    size_t bytes = 0;
};

namespace {

constexpr int kXsecBatch = 64;  // directions per cross-section launch

bool finite_pos(double v) { return std::isfinite(v) && v > 0; }

int born_alloc(qsg_born *b, size_t bytes, void **p)
{
    int rc = dev_alloc(b->ctx, bytes, p, &b->bytes);
    if (rc == QSG_OK) b->allocs.push_back(*p);
    return rc;
}

void born_free(qsg_born *b)
{
    if (!b) return;
    if (b->ctx) {
        for (void *p : b->allocs) cudaFreeAsync(p, b->ctx->st);
        b->ctx->in_use -= b->bytes;
    }
    if (b->hparts) cudaFreeHost(b->hparts);
    if (b->xs_hparts) cudaFreeHost(b->xs_hparts);
    if (b->done) cudaEventDestroy(b->done);
    delete b;
}

// fold_half of src/Perburbation.h:30-33
size_t fold_pb(size_t i, size_t n) { return i < n / 2 ? i : n - i; }

// cal_v15 (src/Perburbation.h:47-57): the absorbing layer, width 30 / k0
double cal_v15(double x, double k0, double e0)
{
    x *= k0;
    return (-0.8 * e0) * ((1 - x * x / (15. * 15)) > 0 ? std::exp(-0.015 * x * x * 1. / std::sqrt(1 - x * x / (15. * 15))) : 0);
}

// std::transform_reduce with the sequential policy, as the reference's CPU
// reductions evaluate it (src/DeviceTemplate.h:404-407): four at a time
template <class F> double tr_sum(size_t n, F f)
{
    double acc = 0;
    size_t i = 0;
    for (; n - i >= 4; i += 4) acc = acc + ((f(i) + f(i + 1)) + (f(i + 2) + f(i + 3)));
    for (; i < n; ++i) acc = acc + f(i);
    return acc;
}

// PreconditionalBornSeries::GetEpsilon (src/Perburbation.h:326-341)
double min_epsilon(const std::vector<cd> &v, int precer)
{
    auto abs2 = [&](size_t i) { return v[i].imag() * v[i].imag() + v[i].real() * v[i].real(); };
    if (precer == QSG_BORN_IDENTITY) {
        const double a = tr_sum(v.size(), [&](size_t i) { return v[i].imag(); });
        const double a2 = tr_sum(v.size(), abs2);
        return 0.5 * a2 / (-a);
    }
    double m = 0;
    for (size_t i = 0; i < v.size(); ++i) m = m >= abs2(i) ? m : abs2(i);
    return std::sqrt(m);
}

float2 hilo(double v)
{
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
}

// (2 pi hbar / (d n))^2 / 2m: PerburbationUtility::CalDp2Div2M (src/Perburbation.h:17-23)
double dp2div2m(double d, size_t n, double hbar, double mass)
{
    const double dp = 2 * kPi / (d * n) * hbar;
    return dp * dp / (2 * mass);
}

int check_opts(const qsg_born_opts *o, const char *who)
{
    if (!o) return QSG_OK;
    if (o->order < 1) return fail(QSG_ERR_ARG, std::string(who) + ": order must be >= 1");
    if (o->preconditioner < QSG_BORN_IDENTITY || o->preconditioner > QSG_BORN_HAO2)
        return fail(QSG_ERR_ARG, std::string(who) + ": unknown preconditioner");
    if (!std::isfinite(o->slow)) return fail(QSG_ERR_ARG, std::string(who) + ": slow must be finite");
    return QSG_OK;
}

void set_ops(qsg_born *b)
{
    b->ops.eps = b->eps;
    b->ops.slow = b->opts.slow;
    b->ops.pre = b->opts.preconditional ? 1 : 0;
    if (!b->opts.preconditional) {
        b->ops.post = qsg::BORN_POST_NEW;
    } else {
        switch (b->opts.preconditioner) {
        case QSG_BORN_IDENTITY: b->ops.post = b->opts.slow == 1. ? qsg::BORN_POST_NEW : qsg::BORN_POST_LINEAR; break;
        case QSG_BORN_VELLEKOOP: b->ops.post = qsg::BORN_POST_VELLEKOOP; break;
        case QSG_BORN_HAO1: b->ops.post = qsg::BORN_POST_HAO1; break;
        default: b->ops.post = qsg::BORN_POST_HAO2; break;
        }
    }
    b->needs_old = b->ops.post != qsg::BORN_POST_NEW;
}

// host complex128 -> device array of the solver's precision
int upload(qsg_born *b, void *dst, const cd *src, size_t n)
{
    if (b->prec == QSG_MIXED) {
        std::vector<float2> f(n);
        for (size_t i = 0; i < n; ++i) f[i] = make_float2((float)src[i].real(), (float)src[i].imag());
        QSG_CUDA(cudaMemcpyAsync(dst, f.data(), n * 8, cudaMemcpyHostToDevice, b->ctx->st));
        QSG_CUDA(cudaStreamSynchronize(b->ctx->st));  // f goes out of scope
    } else {
        QSG_CUDA(cudaMemcpyAsync(dst, src, n * 16, cudaMemcpyHostToDevice, b->ctx->st));
        QSG_CUDA(cudaStreamSynchronize(b->ctx->st));
    }
    return QSG_OK;
}

int common_buffers(qsg_born *b, int nbuf)
{
    int rc;
    const size_t bytes = b->n * csize(b->prec);
    for (int i = 0; i < nbuf; ++i) {
        if ((rc = born_alloc(b, bytes, &b->dpsi[i]))) return rc;
        QSG_CUDA(cudaMemsetAsync(b->dpsi[i], 0, bytes, b->ctx->st));
    }
    if ((rc = born_alloc(b, bytes, &b->V))) return rc;
    if ((rc = upload(b, b->V, b->vhost.data(), b->n))) return rc;
    void *p = nullptr;
    if ((rc = born_alloc(b, sizeof(double) * b->nparts, &p))) return rc;
    b->parts = (double *)p;
    QSG_CUDA(cudaMallocHost(&b->hparts, sizeof(double) * b->nparts));
    QSG_CUDA(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming));
    return QSG_OK;
}

int create_1d(qsg_born *b, const double *V, double direction)
{
    int rc;
    const size_t n = b->n;
    b->vhost.assign((const cd *)V, (const cd *)V + n);
    const double dir = direction < 0 ? -1. : direction > 0 ? 1. : 0.;
    b->dirx = dir > 0 ? 1 : -1;  // ScatteringSolverImpl.cpp:31-34
    b->psi0host.resize(n);
    for (size_t i = 0; i < n; ++i) {
        const double x = b->x0 + b->dx * i;
        b->psi0host[i] = std::exp(b->dirx * b->k0 * x * cd(0, 1));
    }
    if (b->opts.preconditional) {
        const double lambda = 2 * kPi / (std::sqrt(2 * b->mass * b->en) / b->hbar);
        if (n * b->dx < 24 * lambda) return fail(QSG_ERR_ARG, "qsg_born_create_1d: too small world size to fit 24 wave length");
        const double kk = std::sqrt(2 * b->mass * b->en) / b->hbar;
        if (kk * b->dx * n < 30) return fail(QSG_ERR_ARG, "qsg_born_create_1d: too small world to fit absb layer");
        for (size_t i = 0; i < n; ++i)
            b->vhost[i].imag(b->vhost[i].imag() + cal_v15(fold_pb(i, n) * b->dx, kk, b->en));
        const double me = min_epsilon(b->vhost, b->opts.preconditioner);
        if (b->eps < me) b->eps = me;
    }
    set_ops(b);
    b->resident = qsg::born1d_resident(b->prec, n);
    if (!b->resident) qsg::born_fs_split(n, &b->n1, &b->n2);
    b->nparts = b->resident ? 4 : 4 * qsg::born_fs_col_blocks(b->prec, b->n1, b->n2);
    if ((rc = common_buffers(b, 1))) return rc;
    if ((rc = born_alloc(b, n * csize(b->prec), &b->psi0))) return rc;
    if ((rc = upload(b, b->psi0, b->psi0host.data(), n))) return rc;
    const int E = qsg::born_e(b->prec);
    if (b->resident) {
        if ((rc = get_twiddles(b->ctx, b->prec, (int)n, E, &b->tw_a))) return rc;
    } else {
        if ((rc = born_alloc(b, n * csize(b->prec), &b->tmp))) return rc;
        if ((rc = get_twiddles(b->ctx, b->prec, b->n2, E, &b->tw_a))) return rc;
        if ((rc = get_twiddles(b->ctx, b->prec, b->n1, E, &b->tw_b))) return rc;
        // the four-step column pass's twiddles in its own row-major layout
        if ((rc = get_fs_grid(b->ctx, b->prec, b->n1, b->n2, &b->tw_n))) return rc;
    }
    return QSG_OK;
}

int create_2d(qsg_born *b, const double *V)
{
    int rc;
    const int nx = b->nx, ny = b->ny;
    const size_t n = b->n;
    b->vhost.assign((const cd *)V, (const cd *)V + n);
    for (size_t i = 0; i < n; ++i)
        if (std::isnan(b->vhost[i].real()) || std::isnan(b->vhost[i].imag()))
            return fail(QSG_ERR_ARG, "qsg_born_create_2d: nan in V at index " + std::to_string(i));
    if (b->opts.preconditional) {
        const double lambda = 2 * kPi / (std::sqrt(2 * b->mass * b->en) / b->hbar);
        if (nx * b->dx < 24 * lambda || ny * b->dy < 24 * lambda)
            return fail(QSG_ERR_ARG, "qsg_born_create_2d: too small size");
        const double kk = std::sqrt(2 * b->mass * b->en) / b->hbar;
        for (int i = 0; i < nx; ++i)
            for (int j = 0; j < ny; ++j) {
                cd &v = b->vhost[(size_t)i * ny + j];
                v.imag(v.imag() + (cal_v15(fold_pb(i, nx) * b->dx, kk, b->en) + cal_v15(fold_pb(j, ny) * b->dy, kk, b->en)));
            }
        const double me = min_epsilon(b->vhost, b->opts.preconditioner);
        if (b->eps < me) b->eps = me;
    }
    set_ops(b);
    b->nparts = 2 * qsg::born_row_blocks(b->prec, nx, ny);
    if ((rc = common_buffers(b, 2))) return rc;
    if ((rc = born_alloc(b, n * csize(b->prec), &b->tmp))) return rc;
    // psi0 = ex[i] ey[j]
    const double kx = b->k0 * b->dirx, ky = b->k0 * b->diry;
    std::vector<cd> ex(nx), ey(ny);
    for (int i = 0; i < nx; ++i) ex[i] = std::exp(cd(0, kx * (b->x0 + b->dx * i)));
    for (int j = 0; j < ny; ++j) ey[j] = std::exp(cd(0, ky * (b->y0 + b->dy * j)));
    if ((rc = born_alloc(b, nx * csize(b->prec), &b->ex))) return rc;
    if ((rc = born_alloc(b, ny * csize(b->prec), &b->ey))) return rc;
    if ((rc = upload(b, b->ex, ex.data(), nx))) return rc;
    if ((rc = upload(b, b->ey, ey.data(), ny))) return rc;
    // G0 tables: E - fold(kx)^2 DPx^2/2m and fold(ky)^2 DPy^2/2m (G02D, DeviceTemplate.h:906-931)
    const double ax = dp2div2m(b->dx, nx, b->hbar, b->mass), ay = dp2div2m(b->dy, ny, b->hbar, b->mass);
    std::vector<double> gx(nx), gy(ny);
    for (int i = 0; i < nx; ++i) {
        const double f = (double)(i > nx / 2 ? nx - i : i);
        gx[i] = b->en - f * f * ax;
    }
    for (int j = 0; j < ny; ++j) {
        const double f = (double)(j > ny / 2 ? ny - j : j);
        gy[j] = f * f * ay;
    }
    void *p = nullptr;
    if ((rc = born_alloc(b, nx * 8, &p))) return rc;
    b->gx = (double *)p;
    if ((rc = born_alloc(b, ny * 8, &p))) return rc;
    b->gy = (double *)p;
    QSG_CUDA(cudaMemcpyAsync(b->gx, gx.data(), nx * 8, cudaMemcpyHostToDevice, b->ctx->st));
    QSG_CUDA(cudaMemcpyAsync(b->gy, gy.data(), ny * 8, cudaMemcpyHostToDevice, b->ctx->st));
    std::vector<float2> gx2(nx), gy2(ny);
    for (int i = 0; i < nx; ++i) gx2[i] = hilo(gx[i]);
    for (int j = 0; j < ny; ++j) gy2[j] = hilo(gy[j]);
    if ((rc = born_alloc(b, nx * 8, &p))) return rc;
    b->gx2 = (float2 *)p;
    if ((rc = born_alloc(b, ny * 8, &p))) return rc;
    b->gy2 = (float2 *)p;
    QSG_CUDA(cudaMemcpyAsync(b->gx2, gx2.data(), nx * 8, cudaMemcpyHostToDevice, b->ctx->st));
    QSG_CUDA(cudaMemcpyAsync(b->gy2, gy2.data(), ny * 8, cudaMemcpyHostToDevice, b->ctx->st));
    QSG_CUDA(cudaStreamSynchronize(b->ctx->st));
    b->g = qsg::born_split(b->prec, nx, ny);
    const int m = nx / b->g;
    if ((rc = get_twiddles(b->ctx, b->prec, ny, qsg::born_e(b->prec), &b->tw_a))) return rc;
    if ((rc = get_twiddles(b->ctx, b->prec, m, qsg::born_col_e(b->prec, m), &b->tw_b))) return rc;
    if ((rc = get_circle(b->ctx, b->prec, nx, &b->tw_n))) return rc;
    return QSG_OK;
}

template <class T> int compute_2d(qsg_born *b)
{
    cudaStream_t st = b->ctx->st;
    const int K = b->opts.order;
    const int cur = b->cur, nxt = 1 - cur;
    qsg::BornRowArgs r{};
    r.V = b->V;
    r.ex = b->ex;
    r.ey = b->ey;
    r.tw = b->tw_a;
    r.tw_nx = b->tw_n;
    r.m = b->nx / b->g;
    r.ops = b->ops;
    r.in = b->dpsi[cur];
    r.tmp = b->tmp;
    r.in_k = 0;
    r.out_k = 1;
    {
        ProfScope ps(b->ctx, "born_row_pass", st);
        QSG_CUDA(qsg::born_row<T>(b->nx, b->ny, r, st));
    }
    qsg::BornColArgs c{};
    c.tmp = b->tmp;
    c.gx = b->gx;
    c.gy = b->gy;
    c.gx2 = b->gx2;
    c.gy2 = b->gy2;
    c.tw = b->tw_b;
    c.eps = b->eps;
    c.inv_n = 1.0 / (double)b->n;
    c.ny = b->ny;
    c.g = b->g;
    for (int i = 1; i <= K; ++i) {
        {
            ProfScope ps(b->ctx, "born_col_pass", st);
            QSG_CUDA(qsg::born_col<T>(b->nx, b->ny, c, st));
        }
        r.in = b->tmp;
        r.in_k = 1;
        r.dold = b->needs_old ? b->dpsi[i == 1 ? cur : nxt] : nullptr;
        if (i < K) {
            r.out_k = 1;
            r.dnew = b->needs_old ? b->dpsi[nxt] : nullptr;
        } else {
            r.out_k = 0;
            r.dnew = b->dpsi[nxt];
            r.dstart = b->dpsi[cur];
            r.partials = b->parts;
        }
        ProfScope ps(b->ctx, "born_row_pass", st);
        QSG_CUDA(qsg::born_row<T>(b->nx, b->ny, r, st));
    }
    b->cur = nxt;
    return QSG_OK;
}

template <class T> int compute_1d(qsg_born *b)
{
    cudaStream_t st = b->ctx->st;
    const double dk2 = dp2div2m(b->dx, b->n, b->hbar, b->mass);
    if (b->resident) {
        qsg::Born1DArgs a{};
        a.dpsi = b->dpsi[0];
        a.psi0 = b->psi0;
        a.V = b->V;
        a.tw = b->tw_a;
        a.en = b->en;
        a.dk2 = dk2;
        a.enf = hilo(b->en);
        a.dkf = hilo(dk2);
        a.inv_n = 1.0 / (double)b->n;
        a.sums = b->parts;
        a.ops = b->ops;
        a.order = b->opts.order;
        ProfScope ps(b->ctx, "born_1d", st);
        QSG_CUDA(qsg::born_1d<T>((int)b->n, a, st));
        return QSG_OK;
    }
    const int K = b->opts.order;
    qsg::BornFsColArgs c{};
    c.psi0 = b->psi0;
    c.V = b->V;
    c.tw = b->tw_a;
    c.tw_n = b->tw_n;
    c.ops = b->ops;
    c.n1 = b->n1;
    c.in = b->dpsi[0];
    c.tmp = b->tmp;
    c.in_k = 0;
    c.out_k = 1;
    {
        ProfScope ps(b->ctx, "born_fs_col_pass", st);
        QSG_CUDA(qsg::born_fs_col<T>(b->n1, b->n2, c, st));
    }
    qsg::BornFsRowArgs rr{};
    rr.tmp = b->tmp;
    rr.tw = b->tw_b;
    rr.en = b->en;
    rr.dk2 = dk2;
    rr.enf = hilo(b->en);
    rr.dkf = hilo(dk2);
    rr.eps = b->eps;
    rr.inv_n = 1.0 / (double)b->n;
    rr.n = (int)b->n;
    rr.n2 = b->n2;
    for (int i = 1; i <= K; ++i) {
        {
            ProfScope ps(b->ctx, "born_fs_row_pass", st);
            QSG_CUDA(qsg::born_fs_row<T>(b->n1, b->n2, rr, st));
        }
        c.in = b->tmp;
        c.in_k = 1;
        c.dold = b->needs_old ? b->dpsi[0] : nullptr;
        if (i < K) {
            c.out_k = 1;
            c.dnew = b->needs_old ? b->dpsi[0] : nullptr;
        } else {
            c.out_k = 0;
            c.dnew = b->dpsi[0];
            c.partials = b->parts;
        }
        ProfScope ps(b->ctx, "born_fs_col_pass", st);
        QSG_CUDA(qsg::born_fs_col<T>(b->n1, b->n2, c, st));
    }
    return QSG_OK;
}

// the reductions of the last compute, summed on the host in a fixed order
int finish(qsg_born *b)
{
    if (!b->pending) return QSG_OK;
    QSG_CUDA(cudaEventSynchronize(b->done));
    b->pending = false;
    const int stride = b->dim == 1 ? 4 : 2;
    double s[4] = {0, 0, 0, 0};
    for (int i = 0; i < b->nparts / stride; ++i)
        for (int k = 0; k < stride; ++k) s[k] += b->hparts[i * stride + k];
    if (b->dim == 1) {
        // ScatteringSolver1DImpl::ComputeRT (src/ScatteringSolverImpl.cpp:40-55)
        const cd r(s[0], s[1]), t(s[2], s[3]);
        const cd I(0, 1);
        const cd rr = r * b->dx * b->mass / (b->hbar * b->hbar * std::abs(b->k0) * I);
        const cd tt = t * b->dx * b->mass / (b->hbar * b->hbar * std::abs(b->k0) * I) + cd(1, 0);
        b->R = std::norm(rr);
        b->T = std::norm(tt);
    } else {
        b->delta = std::sqrt(s[0] / s[1]);
    }
    return QSG_OK;
}

int check_born(qsg_born *b, const char *who)
{
    if (!b || !b->ctx) return fail(QSG_ERR_ARG, std::string(who) + ": null solver");
    return QSG_OK;
}

}  // namespace

extern "C" {

void qsg_born_default_opts(qsg_born_opts *o)
{
    if (!o) return;
    o->order = 1;
    o->preconditional = 0;
    o->preconditioner = QSG_BORN_VELLEKOOP;
    o->slow = 1.0;
}

int qsg_born_create_1d(qsg_ctx *ctx, uint64_t n, double x0, double x1, const double *V, double en,
                       double epsilon, double direction, double mass, double hbar,
                       const qsg_born_opts *opts, int precision, qsg_born **out)
{
    if (!ctx || !V || !out) return fail(QSG_ERR_ARG, "qsg_born_create_1d: null argument");
    *out = nullptr;
    int rc;
    if ((rc = check_opts(opts, "qsg_born_create_1d"))) return rc;
    if (precision != QSG_FP64 && precision != QSG_MIXED)
        return fail(QSG_ERR_ARG, "qsg_born_create_1d: precision must be QSG_FP64 or QSG_MIXED");
    if (!std::isfinite(x0) || !std::isfinite(x1) || !(x1 > x0) || !finite_pos(en) || !finite_pos(mass) ||
        !finite_pos(hbar) || !std::isfinite(epsilon) || !std::isfinite(direction))
        return fail(QSG_ERR_ARG, "qsg_born_create_1d: need x1 > x0, en, mass, hbar > 0, finite epsilon and direction");
    if (!qsg::born1d_supported(precision, n))
        return fail(QSG_ERR_UNSUPPORTED, "qsg_born_create_1d: n=" + std::to_string(n) +
                                             " (supported: powers of two, 128 .. 2^22)");
    std::lock_guard<std::mutex> lk(ctx->mu);
    QSG_CUDA(cudaSetDevice(ctx->dev));
    qsg_born *b = new qsg_born;
    b->ctx = ctx;
    b->dim = 1;
    b->prec = precision;
    b->n = n;
    b->nx = (int)n;
    b->x0 = x0;
    b->x1 = x1;
    b->dx = (x1 - x0) / n;
    b->en = en;
    b->eps = epsilon;
    b->mass = mass;
    b->hbar = hbar;
    b->k0 = std::sqrt(2 * en * mass) / hbar;
    if (opts) b->opts = *opts; else qsg_born_default_opts(&b->opts);
    if ((rc = create_1d(b, V, direction))) {
        const std::string msg = g_last_error;
        born_free(b);
        return fail(rc, msg);
    }
    *out = b;
    return QSG_OK;
}

int qsg_born_create_2d(qsg_ctx *ctx, int nx, int ny, double x0, double x1, double y0, double y1,
                       const double *V, double en, double epsilon, double dirx, double diry,
                       double mass, double hbar, const qsg_born_opts *opts, int precision,
                       qsg_born **out)
{
    if (!ctx || !V || !out) return fail(QSG_ERR_ARG, "qsg_born_create_2d: null argument");
    *out = nullptr;
    int rc;
    if ((rc = check_opts(opts, "qsg_born_create_2d"))) return rc;
    if (precision != QSG_FP64 && precision != QSG_MIXED)
        return fail(QSG_ERR_ARG, "qsg_born_create_2d: precision must be QSG_FP64 or QSG_MIXED");
    if (!std::isfinite(x0) || !std::isfinite(x1) || !(x1 > x0) || !std::isfinite(y0) || !std::isfinite(y1) ||
        !(y1 > y0) || !finite_pos(en) || !finite_pos(mass) || !finite_pos(hbar) || !std::isfinite(epsilon) ||
        !std::isfinite(dirx) || !std::isfinite(diry) || (dirx == 0 && diry == 0))
        return fail(QSG_ERR_ARG, "qsg_born_create_2d: need x1 > x0, y1 > y0, en, mass, hbar > 0, finite epsilon, "
                                 "a nonzero direction");
    if (!qsg::born2d_supported(nx, ny))
        return fail(QSG_ERR_UNSUPPORTED, "qsg_born_create_2d: " + std::to_string(nx) + "x" + std::to_string(ny) +
                                             " (supported: powers of two, 64 .. 4096 per side)");
    std::lock_guard<std::mutex> lk(ctx->mu);
    QSG_CUDA(cudaSetDevice(ctx->dev));
    qsg_born *b = new qsg_born;
    b->ctx = ctx;
    b->dim = 2;
    b->prec = precision;
    b->nx = nx;
    b->ny = ny;
    b->n = (uint64_t)nx * ny;
    b->x0 = x0;
    b->x1 = x1;
    b->y0 = y0;
    b->y1 = y1;
    b->dx = (x1 - x0) / nx;
    b->dy = (y1 - y0) / ny;
    b->en = en;
    b->eps = epsilon;
    b->mass = mass;
    b->hbar = hbar;
    b->k0 = std::sqrt(2 * en * mass) / hbar;
    const double nm = 1 / std::sqrt(dirx * dirx + diry * diry);  // ScatteringSolverImpl.cpp:109-113
    b->dirx = dirx * nm;
    b->diry = diry * nm;
    if (opts) b->opts = *opts; else qsg_born_default_opts(&b->opts);
    if ((rc = create_2d(b, V))) {
        const std::string msg = g_last_error;
        born_free(b);
        return fail(rc, msg);
    }
    *out = b;
    return QSG_OK;
}

int qsg_born_compute(qsg_born *b)
{
    int rc;
    if ((rc = check_born(b, "qsg_born_compute"))) return rc;
    std::lock_guard<std::mutex> lk(b->ctx->mu);
    QSG_CUDA(cudaSetDevice(b->ctx->dev));
    if (b->dim == 2)
        rc = b->prec == QSG_MIXED ? compute_2d<float>(b) : compute_2d<double>(b);
    else
        rc = b->prec == QSG_MIXED ? compute_1d<float>(b) : compute_1d<double>(b);
    if (rc) return rc;
    QSG_CUDA(cudaMemcpyAsync(b->hparts, b->parts, sizeof(double) * b->nparts, cudaMemcpyDeviceToHost, b->ctx->st));
    QSG_CUDA(cudaEventRecord(b->done, b->ctx->st));
    b->pending = true;
    b->computed = true;
    return QSG_OK;
}

int qsg_born_get(qsg_born *b, int what, double *out)
{
    int rc;
    if ((rc = check_born(b, "qsg_born_get"))) return rc;
    if (!out) return fail(QSG_ERR_ARG, "qsg_born_get: null output");
    std::lock_guard<std::mutex> lk(b->ctx->mu);
    cd *o = (cd *)out;
    if (what == QSG_BORN_V) {
        std::copy(b->vhost.begin(), b->vhost.end(), o);
        return QSG_OK;
    }
    if (what == QSG_BORN_PSI0) {
        if (b->dim == 1) {
            std::copy(b->psi0host.begin(), b->psi0host.end(), o);
        } else {
            // exp((kx x + ky y) i), ScatteringSolverImpl.cpp:154-159
            const double kx = b->k0 * b->dirx, ky = b->k0 * b->diry;
            for (int i = 0; i < b->nx; ++i)
                for (int j = 0; j < b->ny; ++j)
                    o[(size_t)i * b->ny + j] = std::exp((kx * (b->x0 + b->dx * i) + ky * (b->y0 + b->dy * j)) * cd(0, 1));
        }
        return QSG_OK;
    }
    if (what != QSG_BORN_PSI) return fail(QSG_ERR_ARG, "qsg_born_get: unknown field");
    QSG_CUDA(cudaSetDevice(b->ctx->dev));
    const void *src = b->dpsi[b->dim == 2 ? b->cur : 0];
    if (b->prec == QSG_MIXED) {
        std::vector<float2> f(b->n);
        QSG_CUDA(cudaMemcpyAsync(f.data(), src, b->n * 8, cudaMemcpyDeviceToHost, b->ctx->st));
        QSG_CUDA(cudaStreamSynchronize(b->ctx->st));
        for (size_t i = 0; i < b->n; ++i) o[i] = cd(f[i].x, f[i].y);
    } else {
        QSG_CUDA(cudaMemcpyAsync(out, src, b->n * 16, cudaMemcpyDeviceToHost, b->ctx->st));
        QSG_CUDA(cudaStreamSynchronize(b->ctx->st));
    }
    return QSG_OK;
}

int qsg_born_rt(qsg_born *b, double *R, double *T)
{
    int rc;
    if ((rc = check_born(b, "qsg_born_rt"))) return rc;
    if (b->dim != 1) return fail(QSG_ERR_ARG, "qsg_born_rt: 1D solvers only");
    if (!b->computed) return fail(QSG_ERR_STATE, "qsg_born_rt: no compute yet");
    std::lock_guard<std::mutex> lk(b->ctx->mu);
    if ((rc = finish(b))) return rc;
    if (R) *R = b->R;
    if (T) *T = b->T;
    return QSG_OK;
}

int qsg_born_delta_norm(qsg_born *b, double *out)
{
    int rc;
    if ((rc = check_born(b, "qsg_born_delta_norm"))) return rc;
    if (b->dim != 2) return fail(QSG_ERR_ARG, "qsg_born_delta_norm: 2D solvers only");
    if (!out) return fail(QSG_ERR_ARG, "qsg_born_delta_norm: null output");
    std::lock_guard<std::mutex> lk(b->ctx->mu);
    if (!b->computed) {
        *out = 0;  // fNormDeltaPsi before any Compute (ScatteringSolverImpl.cpp:122)
        return QSG_OK;
    }
    if ((rc = finish(b))) return rc;
    *out = b->delta;
    return QSG_OK;
}

int qsg_born_epsilon(qsg_born *b, double *out)
{
    int rc;
    if ((rc = check_born(b, "qsg_born_epsilon"))) return rc;
    if (!out) return fail(QSG_ERR_ARG, "qsg_born_epsilon: null output");
    *out = b->eps;
    return QSG_OK;
}

int qsg_born_xsection(qsg_born *b, int count, const double *cosxy, double *out)
{
    int rc;
    if ((rc = check_born(b, "qsg_born_xsection"))) return rc;
    if (b->dim != 2) return fail(QSG_ERR_ARG, "qsg_born_xsection: 2D solvers only");
    if (count < 0 || (count > 0 && (!cosxy || !out))) return fail(QSG_ERR_ARG, "qsg_born_xsection: bad arguments");
    for (int a = 0; a < count; ++a)
        if (!std::isfinite(cosxy[2 * a]) || !std::isfinite(cosxy[2 * a + 1]) ||
            (cosxy[2 * a] == 0 && cosxy[2 * a + 1] == 0))
            return fail(QSG_ERR_ARG, "qsg_born_xsection: direction must be finite and nonzero");
    std::lock_guard<std::mutex> lk(b->ctx->mu);
    QSG_CUDA(cudaSetDevice(b->ctx->dev));
    const int nx = b->nx, ny = b->ny;
    const int blocks = qsg::born_xsec_blocks(nx);
    if (!b->xs_tab) {
        void *p = nullptr;
        if ((rc = born_alloc(b, sizeof(double2) * kXsecBatch * (size_t)(nx + ny), &p))) return rc;
        b->xs_tab = (double2 *)p;
        if ((rc = born_alloc(b, sizeof(double) * 2 * kXsecBatch * (size_t)blocks, &p))) return rc;
        b->xs_parts = (double *)p;
        QSG_CUDA(cudaMallocHost(&b->xs_hparts, sizeof(double) * 2 * kXsecBatch * (size_t)blocks));
    }
    std::vector<double2> tab((size_t)kXsecBatch * (nx + ny));
    for (int a0 = 0; a0 < count; a0 += kXsecBatch) {
        const int na = std::min(kXsecBatch, count - a0);
        std::vector<double> kxs(na), kys(na);
        for (int a = 0; a < na; ++a) {
            double cx = cosxy[2 * (a0 + a)], cy = cosxy[2 * (a0 + a) + 1];
            const double nm = 1 / std::sqrt(cx * cx + cy * cy);  // ScatteringSolverImpl.cpp:220-222
            cx *= nm;
            cy *= nm;
            kxs[a] = b->k0 * cx;
            kys[a] = b->k0 * cy;
            for (int i = 0; i < nx; ++i) {
                const cd w = std::exp(cd(0, -kxs[a] * (b->x0 + b->dx * i)));
                tab[(size_t)a * nx + i] = make_double2(w.real(), w.imag());
            }
            for (int j = 0; j < ny; ++j) {
                const cd w = std::exp(cd(0, -kys[a] * (b->y0 + b->dy * j)));
                tab[(size_t)na * nx + (size_t)a * ny + j] = make_double2(w.real(), w.imag());
            }
        }
        QSG_CUDA(cudaMemcpyAsync(b->xs_tab, tab.data(), sizeof(double2) * na * (size_t)(nx + ny),
                                 cudaMemcpyHostToDevice, b->ctx->st));
        qsg::BornXsecArgs x{};
        x.dpsi = b->dpsi[b->cur];
        x.V = b->V;
        x.ex = b->ex;
        x.ey = b->ey;
        x.ax = b->xs_tab;
        x.ay = b->xs_tab + (size_t)na * nx;
        x.partials = b->xs_parts;
        x.nx = nx;
        x.ny = ny;
        x.na = na;
        {
            ProfScope ps(b->ctx, "born_xsec", b->ctx->st);
            if (b->prec == QSG_MIXED)
                QSG_CUDA(qsg::born_xsec<float>(nx, x, b->ctx->st));
            else
                QSG_CUDA(qsg::born_xsec<double>(nx, x, b->ctx->st));
        }
        QSG_CUDA(cudaMemcpyAsync(b->xs_hparts, b->xs_parts, sizeof(double) * 2 * na * (size_t)blocks,
                                 cudaMemcpyDeviceToHost, b->ctx->st));
        QSG_CUDA(cudaStreamSynchronize(b->ctx->st));
        for (int a = 0; a < na; ++a) {
            cd r(0, 0);
            for (int c = 0; c < blocks; ++c)
                r += cd(b->xs_hparts[((size_t)c * na + a) * 2], b->xs_hparts[((size_t)c * na + a) * 2 + 1]);
            // ScatteringSolverImpl.cpp:245
            out[a0 + a] = std::norm(r * (2 * b->mass) / (b->hbar * b->hbar) * b->dx * b->dy * (1. / 4)) *
                          (2 / (kPi * b->k0));
        }
    }
    return QSG_OK;
}

int qsg_born_total_xsection(qsg_born *b, int n, double *out)
{
    int rc;
    if ((rc = check_born(b, "qsg_born_total_xsection"))) return rc;
    if (n < 1 || !out) return fail(QSG_ERR_ARG, "qsg_born_total_xsection: need n >= 1 and an output");
    // ComputeTotalXSection (ScatteringSolverImpl.cpp:252-266)
    std::vector<double> cs(2 * (size_t)n), xs(n);
    for (int i = 0; i < n; ++i) {
        const double theta = i * 2 * kPi / n;
        cs[2 * i] = std::cos(theta);
        cs[2 * i + 1] = std::sin(theta);
    }
    if ((rc = qsg_born_xsection(b, n, cs.data(), xs.data()))) return rc;
    double t = 0;
    for (int i = 0; i < n; ++i) t += xs[i];
    *out = t * (2 * kPi / n);
    return QSG_OK;
}

void qsg_born_destroy(qsg_born *b)
{
    if (!b) return;
    if (!b->ctx) {
        delete b;
        return;
    }
    std::lock_guard<std::mutex> lk(b->ctx->mu);
    born_free(b);
}

}  // extern "C"
