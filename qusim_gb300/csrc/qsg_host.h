// qsg_host.h -- host-side context and helpers shared by the C-ABI units
// (qsg_api.cu: evolvers and serving; qsg_born_api.cu: Born-series solvers):
// the context struct, error reporting, budgeted device allocation, twiddle
// tables and launch profiling.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/qsg.h"
#include "qsg_launch.h"

namespace qsg_host {

using qsg::Plan2D;

inline thread_local std::string g_last_error;

inline int fail(int code, const std::string &msg)
{
    g_last_error = msg;
    return code;
}

#define QSG_CUDA(call)                                                                     \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ == cudaErrorNotSupported)                                                   \
            return fail(QSG_ERR_UNSUPPORTED, std::string("unsupported size: ") + #call);   \
        if (e_ != cudaSuccess)                                                             \
            return fail(QSG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

inline constexpr double kPi = 3.141592653589793238462643383279502884197169399375;

struct ProfStat {
    uint64_t launches = 0;
    double total_ms = 0;
};

}  // namespace qsg_host

struct qsg_ctx {
    int dev = 0;
    cudaStream_t st = nullptr;
    size_t budget = 0, in_use = 0;
    std::mutex mu;
    std::map<std::tuple<int, int, int>, void *> tw_cache;  // (prec, L, E) -> stage-major twiddles
    std::map<std::pair<int, int>, void *> circle_cache;    // (prec, n) -> exp(-2 pi i m/n)
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    double *partials = nullptr;  // reduction partials
    int max_partials = 0;
    double *sums = nullptr;      // small device result buffer (8 doubles)
    bool col_tma = true;         // momentum-form column passes fed by tensor copies (QSG_COL_TMA=0: off)
    // four-step column passes fed by tensor copies (QSG_FS_TMA=1); off by default: on the 2048-instance
    // batch they measured slower than the load-instruction pass (511 against 471 ms of column passes per
    // 1000 steps: two CTAs per SM instead of three, and the twiddles still come from L2)
    bool fs_tma = false;
    double *host_sums = nullptr; // pinned mirror (slot 7: an instance's failure counter, copied for a check)
    // 1D periodic kinetic tables shared by the instances with the same (precision, size,
    // coefficient); key (precision, n1, n2, f) in the four-step layout, (precision, n, 0, f) in
    // the natural one: table pointer, bytes, instances using it
    struct SharedTable {
        void *p;
        size_t bytes;
        int users;
    };
    std::map<std::tuple<int, int, int, double, double>, SharedTable> fs_ktabs;
    int prof = 0;  // 0 off, 1 CUDA-event timing of every launch, 2 launch counts only
    // batch steps replayed from captured CUDA graphs (QSG_BATCH_GRAPHS=1); off by default: on the
    // 2048-instance batch the graph measured no faster than direct launches (7.34e10 against 7.41e10
    // site-steps/s, capture included), as the size classes already overlap on their streams
    bool graphs = false;
    // complex64 batches: the resident classes of length 1024 .. 8192 share one persistent
    // launch fed by a tile queue (QSG_BATCH_QUEUE=0: one launch per class instead)
    bool batch_queue = true;
    std::vector<std::tuple<std::string, cudaEvent_t, cudaEvent_t>> prof_pending;
    std::vector<cudaEvent_t> event_pool;
    std::map<std::string, qsg_host::ProfStat> prof_stats;
    std::vector<std::string> prof_names;  // stable storage for returned names
    std::string device_name;
    std::map<std::tuple<int, int, int>, qsg::Plan2D> plans;  // tuned plans: (prec, nx, ny) -> plan
    // tuned 1D plans: (prec, stepped length, wall extension) -> plan
    std::map<std::tuple<int, uint64_t, int>, qsg_plan1d> plans1d;
    bool plans_loaded = false;
};

namespace qsg_host {

inline size_t csize(int prec) { return prec == 1 ? 8 : 16; }

// Allocate device memory.  Instance memory, twiddle tables and scratch count
// against the context's HBM budget; the context's own fixed buffers (budgeted
// = false) do not.
inline int dev_alloc(qsg_ctx *ctx, size_t bytes, void **p, size_t *acct, bool budgeted = true)
{
    if (budgeted && ctx->budget && ctx->in_use + bytes > ctx->budget)
        return fail(QSG_ERR_BUDGET, "HBM budget exceeded: need " + std::to_string(bytes) + " more bytes, " +
                                        std::to_string(ctx->budget - ctx->in_use) + " left");
    // stream-ordered: a free does not stall other streams (cudaFree synchronises the device)
    cudaError_t e = cudaMallocAsync(p, bytes, ctx->st);
    if (e != cudaSuccess) return fail(QSG_ERR_CUDA, std::string("cudaMallocAsync: ") + cudaGetErrorString(e));
    if (budgeted) ctx->in_use += bytes;
    if (acct) *acct += bytes;
    return QSG_OK;
}

// twiddle table entry: complex128 {re, im}; complex64 {hi.re, hi.im, lo.re, lo.im}
// with hi = float(v), lo = float(v - hi)
// table precision codes: 0 complex128, 1 complex64 hi + lo (float4),
// 2 complex64 plain (float2, each factor rounded once)
inline size_t twsize(int prec) { return prec == 2 ? 8 : 16; }

inline void put_twiddle(int prec, unsigned char *dst, long double re, long double im)
{
    if (prec == 2) {
        const float v[2] = {(float)re, (float)im};
        std::memcpy(dst, v, 8);
    } else if (prec == 1) {
        const float hr = (float)re, hi = (float)im;
        float v[4] = {hr, hi, (float)(re - (long double)hr), (float)(im - (long double)hi)};
        std::memcpy(dst, v, 16);
    } else {
        double v[2] = {(double)re, (double)im};
        std::memcpy(dst, v, 16);
    }
}

// stage-major twiddles of qsg::Plan<L, E>, from long double
inline int get_twiddles(qsg_ctx *ctx, int prec, int L, int E, const void **out)
{
    auto key = std::make_tuple(prec, L, E);
    auto it = ctx->tw_cache.find(key);
    if (it != ctx->tw_cache.end()) {
        *out = it->second;
        return QSG_OK;
    }
    qsg::PlanRT p(L, E);
    const int size = p.tw_size() > 0 ? p.tw_size() : 1;
    std::vector<long double> re(size, 1.0L), im(size, 0.0L);
    int off = 0;
    const long double two_pi = 6.283185307179586476925286766559005768L;
    for (int s = 1; s < p.nst; ++s) {
        const int R = 1 << p.radix_log(s), P = 1 << p.p_log(s);
        for (int q = 1; q < R; ++q)
            for (int k = 0; k < P; ++k) {
                const long double ang = two_pi * (long double)(q * k) / (long double)(P * R);
                re[off + (q - 1) * P + k] = cosl(ang);
                im[off + (q - 1) * P + k] = -sinl(ang);
            }
        off += (R - 1) * P;
    }
    std::vector<unsigned char> host(size * twsize(prec));
    for (int i = 0; i < size; ++i) put_twiddle(prec, &host[i * twsize(prec)], re[i], im[i]);
    void *d = nullptr;
    int rc = dev_alloc(ctx, host.size(), &d, nullptr);
    if (rc) return rc;
    QSG_CUDA(cudaMemcpyAsync(d, host.data(), host.size(), cudaMemcpyHostToDevice, ctx->st));
    QSG_CUDA(cudaStreamSynchronize(ctx->st));
    ctx->tw_cache[key] = d;
    *out = d;
    return QSG_OK;
}

// exp(-2 pi i m / n) for m < n in long double: cosl / sinl of angles of at most
// pi / 4 only, from a table of n / 8 + 1 entries and the quarter-turn symmetries
// (exact sign changes and swaps) where 8 divides n, directly otherwise.  Long
// circles (2^22 entries for the longest four-step lines) cost an eighth of the
// trigonometric calls, which some hosts run in software for long double.
struct CircleLD {
    long n, n8;
    std::vector<long double> c, s;
    explicit CircleLD(long n_) : n(n_), n8(n_ % 8 == 0 ? n_ / 8 : 0)
    {
        const long double two_pi = 6.283185307179586476925286766559005768L;
        for (long j = 0; n8 && j <= n8; ++j) {
            const long double ang = two_pi * (long double)j / (long double)n;
            c.push_back(cosl(ang));
            s.push_back(sinl(ang));
        }
    }
    void at(long m, long double *re, long double *im) const
    {
        if (!n8) {
            const long double ang = 6.283185307179586476925286766559005768L * (long double)m / (long double)n;
            *re = cosl(ang);
            *im = -sinl(ang);
            return;
        }
        // theta = 2 pi m / n = k pi / 2 + alpha, alpha = 2 pi a / n with a in [-n/8, n/8)
        const long n4 = 2 * n8, k = (m + n8) / n4, a = m - k * n4;
        const long double ca = c[a < 0 ? -a : a], sa = a < 0 ? -s[-a] : s[a];
        long double cs, sn;
        switch (k & 3) {
        case 0: cs = ca; sn = sa; break;
        case 1: cs = -sa; sn = ca; break;
        case 2: cs = -ca; sn = -sa; break;
        default: cs = sa; sn = -ca; break;
        }
        *re = cs;
        *im = -sn;
    }
};

// exp(-2 pi i m / n), m < n
inline int get_circle(qsg_ctx *ctx, int prec, int n, const void **out)
{
    auto key = std::make_pair(prec, n);
    auto it = ctx->circle_cache.find(key);
    if (it != ctx->circle_cache.end()) {
        *out = it->second;
        return QSG_OK;
    }
    std::vector<unsigned char> host((size_t)n * twsize(prec));
    const CircleLD circle(n);
    for (int m = 0; m < n; ++m) {
        long double re, im;
        circle.at(m, &re, &im);
        put_twiddle(prec, &host[(size_t)m * twsize(prec)], re, im);
    }
    void *d = nullptr;
    int rc = dev_alloc(ctx, host.size(), &d, nullptr);
    if (rc) return rc;
    QSG_CUDA(cudaMemcpyAsync(d, host.data(), host.size(), cudaMemcpyHostToDevice, ctx->st));
    QSG_CUDA(cudaStreamSynchronize(ctx->st));
    ctx->circle_cache[key] = d;
    *out = d;
    return QSG_OK;
}

// four-step twiddles in the layout the column pass reads them: entry
// r * n1 + c = exp(-2 pi i r c / (n1 n2)), r < n2, c < n1 (the circle's entry
// m = r c, computed the same way, so the values are the circle's bit for bit)
inline int get_fs_grid(qsg_ctx *ctx, int prec, int n1, int n2, const void **out)
{
    auto key = std::make_tuple(prec + 8, n1, n2);
    auto it = ctx->tw_cache.find(key);
    if (it != ctx->tw_cache.end()) {
        *out = it->second;
        return QSG_OK;
    }
    const long n = (long)n1 * n2;
    std::vector<unsigned char> host((size_t)n * twsize(prec));
    const CircleLD circle(n);
    for (long r = 0; r < n2; ++r)
        for (long c = 0; c < n1; ++c) {
            long double re, im;
            circle.at(r * c, &re, &im);
            put_twiddle(prec, &host[(size_t)(r * n1 + c) * twsize(prec)], re, im);
        }
    void *d = nullptr;
    int rc = dev_alloc(ctx, host.size(), &d, nullptr);
    if (rc) return rc;
    QSG_CUDA(cudaMemcpyAsync(d, host.data(), host.size(), cudaMemcpyHostToDevice, ctx->st));
    QSG_CUDA(cudaStreamSynchronize(ctx->st));
    ctx->tw_cache[key] = d;
    *out = d;
    return QSG_OK;
}

// --- profiling -------------------------------------------------------------

inline cudaEvent_t take_event(qsg_ctx *ctx)
{
    if (!ctx->event_pool.empty()) {
        cudaEvent_t e = ctx->event_pool.back();
        ctx->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

struct ProfScope {
    qsg_ctx *ctx;
    const char *name;
    cudaStream_t st;
    cudaEvent_t e0 = nullptr;
    ProfScope(qsg_ctx *c, const char *n, cudaStream_t s = nullptr) : ctx(c), name(n), st(s ? s : c->st)
    {
        if (ctx->prof == 1) {
            e0 = take_event(ctx);
            cudaEventRecord(e0, st);
        } else if (ctx->prof == 2) {
            ctx->prof_stats[name].launches += 1;
        }
    }
    ~ProfScope()
    {
        if (e0) {
            cudaEvent_t e1 = take_event(ctx);
            cudaEventRecord(e1, st);
            ctx->prof_pending.emplace_back(name, e0, e1);
        }
    }
};

}  // namespace qsg_host
