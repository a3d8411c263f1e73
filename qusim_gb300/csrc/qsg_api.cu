// qsg_api.cu -- the C ABI (include/qsg.h): contexts, instances, step
// scheduling, observables.
//
// Step schedule (reference: QuUpdatePsi, src/SplittingUtils.h:14-64, with
// fold_head_tail == false, so every V factor is applied as its own multiply):
//
//   1D, n fits one CTA:  one k_evolve1d_resident launch runs all nsteps.
//   2D:  R(N->S, V)  then per step
//          O2: C(K1)  R(S->S, V V)            ... last step: R(S->N, V)
//          O4: C(KD1) R(S->S, VC2) C(KD2) R(S->S, VC2) C(KD1) R(S->S, VC1 VC1)
//                                              ... last step: R(S->N, VC1)
//        Without renormalisation the last R(S->N) is deferred: the instance
//        stays in split-k space, the next qsg_step opens with R(S->S, V V)
//        (exactly the pass a longer call would have run), and any read of the
//        state (psi, energies, reductions, a plan change) runs R(S->N) first.
//        Norm2 of a deferred state with real dt comes from sums the last C
//        pass took (the closing V factor has modulus 1).
//        R = k_row_pass, C = k_col_pass, N = natural real space, S = split-k
//        space; "V V" multiplies by the same table twice (the reference's two
//        ExpV calls at the step boundary).
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <cmath>
#include <complex>
#include <cstdio>
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/qsg.h"
#include "qsg_aux.h"
#include "qsg_host.h"
#include "qsg_launch.h"
#include "qsg_evolve3d.cuh"
#include "qsg_blue.cuh"

using namespace qsg_host;

using qsg::Geom2D;
using qsg::Plan2D;
using cd = std::complex<double>;

namespace {



// SplittingUtils.cpp:3-8
struct SplitConsts {
    double c1, c2, d1, d2;
    SplitConsts()
    {
        const double t = std::pow(2.0, 1.0 / 3.0);
        c1 = 1 / (2 * (2 - t));
        c2 = (1 - t) / (2 * (2 - t));
        d1 = 1 / (2 - t);
        d2 = -t / (2 - t);
    }
};


}  // namespace


struct qsg_inst {
    qsg_ctx *ctx = nullptr;
    int dim = 1;
    uint64_t n = 0;
    int nx = 0, ny = 0, nz = 1;
    double dx = 0, dy = 0, dz = 0, dv = 0, mass = 1, hbar = 1;
    cd dt;
    int order = 2, prec = 0, boundary = 0;
    void *psi = nullptr;
    double *V = nullptr;
    void *vtab[2] = {nullptr, nullptr};
    void *ktab[2] = {nullptr, nullptr};  // 1D kinetic tables, or 2D fp64 full tables
    void *kx[2] = {nullptr, nullptr}, *ky[2] = {nullptr, nullptr};  // 2D complex64 separable
    const void *tw = nullptr, *tw_row = nullptr, *tw_col = nullptr, *tw_nx = nullptr, *tw_kin = nullptr;
    Plan2D plan{};
    Geom2D geom{};
    cudaStream_t st = nullptr;     // launch stream of the stepping kernels (the context's unless set)
    // 1D: resident (one CTA holds the instance) or four-step (two passes per substep)
    bool fourstep = false;
    qsg_plan1d plan1d{};           // 1D: the plan in use (kind 1 = fourstep, split n1, tma)
    bool fs_tma = false;           // four-step column passes staged by tensor copies
    bool batch_member = false;     // owned by a batch, whose launches are built on its plan
    double *parts_buf = nullptr;   // four-step norm partials (allocated for every n >= 8192)
    // 1D InfiniteWall above the one-CTA sizes: the state is the odd extension
    // of psi to 2 n_out sites (psi_j, 0 at j = n_out, -psi_{2 n_out - j}
    // above), stepped as a periodic four-step instance of n = 2 n_out sites;
    // reads, reductions and writes of the state cover its first n_out sites
    bool wall_ext = false;
    uint64_t n_out = 0;
    // 1D periodic n that is not a power of two: Bluestein transforms of length
    // blue_m (qsg_blue.cuh); chirp and FFT_M(conj chirp) / M tables, K / n in ktab
    bool blue = false;
    int blue_m = 0;
    void *bw = nullptr, *bhs = nullptr;
    // 1D periodic n above the one-CTA Bluestein lengths: Bluestein's convolutions
    // on the four-step passes over a buffer of n = M sites (M >= 2 n_out - 1), the
    // user's n_out sites first and zeros above; bdesc: the passes' descriptors
    // ([0] open V / V c1, [1] K d1 / K d2, [2] V c2 / close, [3] chirp; ktab the
    // two convolution kernels in row layout), bkw: KinEn weights fold(k)^2 DT
    bool bfs = false;
    bool wall_zero = false;  // a wall extension's site 0 still holds the caller's value: zeroed
                             // before the next step (the reference's wall ExpT discards it)
    uint64_t bfs_n = 0;  // Bluestein four-step: the transform length (n, or a wall's 2n)
    qsg::FsInst *bdesc = nullptr;
    double *bkw = nullptr;
    const void *bchirp = nullptr, *bh1 = nullptr;  // chirp (column form) and first kernel, for KinEn
    // 2D grids with a side that is not a power of two: natural-layout Bluestein row
    // and column passes (qsg_blue.cuh); per side the transform length, chirp,
    // FFT_M(conj chirp) / M and twiddles, and per kinetic coefficient the factors
    // along x (with 1 / (nx ny)) and along y
    bool blue2 = false;
    int bmx = 0, bmy = 0;
    void *bwx = nullptr, *bhsx = nullptr, *bwy = nullptr, *bhsy = nullptr;
    const void *btwx = nullptr, *btwy = nullptr;
    void *bkx[2] = {nullptr, nullptr}, *bky[2] = {nullptr, nullptr};
    qsg::FsGeom fsg{};
    const void *tw_fs_col = nullptr, *tw_fs_row = nullptr, *tw_n = nullptr;
    qsg::FsInst *desc = nullptr;   // device descriptor of this instance
    void *fs_maps = nullptr;       // complex64 four-step: tensor maps of psi, V 0, V 1 (tensor-copy column pass)
    size_t fs_maps_bytes = 0;
    double *d_dv = nullptr;        // device copy of dv (resident renormalisation)
    std::vector<std::tuple<int, int, int, double, double>> shared_k;  // four-step kinetic tables in use (ctx->fs_ktabs)
    double *snorm = nullptr;       // 1D one-CTA kernels: sum |psi|^2 of the state a step call ended in
    bool snorm_valid = false;      // ... written by the last call (no renormalisation, no state change since)
    double *parts = nullptr;       // four-step norm partials (col_blocks)
    uint64_t steps = 0;
    // 2D: psi holds the split-k form of the state before the last step's closing
    // V factor (qsg_step defers that row pass; the next step merges it with its
    // own opening V factor, a read of the state runs it first)
    bool pending = false;
    double *cparts = nullptr;      // norm partials of the last column pass (one per tile)
    // 2D complex64 momentum form (QSG_FORM_MOMENTUM): psi holds the state
    // F psi / (Nx Ny) between steps (split-k order), work the split-k input of
    // the next row pass (the inverse column transform of the state)
    int form = QSG_FORM_DIRECT;
    void *work = nullptr;
    // complex64 plain-twiddle tables of the current plan (momentum form passes)
    const void *tw_row_p = nullptr, *tw_col_p = nullptr, *tw_nx_p = nullptr;
    // tensor maps of work and psi for the tensor-copy column pass (two CUtensorMap),
    // built for column blocks of tma_m rows x tma_w columns; tma_w = 0: none
    alignas(64) unsigned char tmaps[256] = {};
    int tma_m = 0, tma_w = 0;
    // 3D: per-axis kinetic factors [axis x, y, z][substep table], twiddles, kinetic partials
    void *k3[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
    const void *tw3[3] = {nullptr, nullptr, nullptr};
    double *kparts3 = nullptr;
    // ring of posted per-step norms (qsg_step_norm2_post / _get)
    static constexpr int kRing = 64;
    double *ring_dev = nullptr;    // kRing device slots
    double *ring_host = nullptr;   // pinned mirror
    cudaEvent_t ring_ev[kRing] = {};
    double ring_scale[kRing] = {};
    uint64_t ring_next = 0;
    // Bounded device-side waits that ran out: a pass whose waits give up adds
    // 1 to the counter `err` (in device memory; the members of a batched
    // four-step class share their first member's) and returns with some tiles
    // of the state updated and some not.  err_seen is the count this instance
    // has acknowledged; lost marks its state as unusable until qsg_set_psi.
    unsigned *err = nullptr;
    unsigned err_seen = 0;
    bool lost = false;
    std::vector<void *> allocs;
    size_t bytes = 0;
};

namespace {


int inst_alloc(qsg_inst *in, size_t bytes, void **p)
{
    int rc = dev_alloc(in->ctx, bytes, p, &in->bytes);
    if (rc == QSG_OK) in->allocs.push_back(*p);
    return rc;
}

int ensure_scratch(qsg_ctx *ctx, size_t bytes)
{
    if (ctx->scratch_bytes >= bytes) return QSG_OK;
    if (ctx->scratch) {
        cudaFreeAsync(ctx->scratch, ctx->st);
        ctx->in_use -= ctx->scratch_bytes;
        ctx->scratch = nullptr;
        ctx->scratch_bytes = 0;
    }
    int rc = dev_alloc(ctx, bytes, &ctx->scratch, nullptr);
    if (rc == QSG_OK) ctx->scratch_bytes = bytes;
    return rc;
}


void prof_drain(qsg_ctx *ctx)
{
    if (ctx->prof_pending.empty()) return;
    cudaDeviceSynchronize();
    for (auto &p : ctx->prof_pending) {
        float ms = 0;
        cudaEventElapsedTime(&ms, std::get<1>(p), std::get<2>(p));
        auto &s = ctx->prof_stats[std::get<0>(p)];
        s.launches += 1;
        s.total_ms += ms;
        ctx->event_pool.push_back(std::get<1>(p));
        ctx->event_pool.push_back(std::get<2>(p));
    }
    ctx->prof_pending.clear();
}

// sites of the state a caller sees (the first n_out of a wall extension)
uint64_t user_n(const qsg_inst *in) { return (in->wall_ext || in->bfs) ? in->n_out : in->n; }

// --- steps -----------------------------------------------------------------

// maps: the instances' tensor maps (3 each) for the tensor-copy pass, or null
int fs_col(qsg_inst *in, const qsg::FsInst *desc, int ninst, bool in_k, bool out_k, int vsel, bool vtwice,
           cudaStream_t st, const void *maps = nullptr)
{
    qsg::FsColArgs a{};
    a.inst = desc;
    a.tw_col = in->tw_fs_col;
    a.tw_n = in->tw_n;
    a.n1 = in->fsg.n1;
    a.vsel = vsel;
    a.vtwice = vtwice ? 1 : 0;
    a.in_k = in_k ? 1 : 0;
    a.out_k = out_k ? 1 : 0;
    a.wall = 0;  // a wall extension's site 0 is zeroed once per uploaded state (step1d)
    ProfScope ps(in->ctx, "fs_col_pass", st);
    if (maps && !in->wall_ext && in->fs_tma && qsg::fs_tma_supported(in->prec, in->fsg.n2)) {
        a.maps = maps;
        a.tiles = in->fsg.col_blocks * ninst;
        a.err = reinterpret_cast<int *>(in->err);
        QSG_CUDA(qsg::launch_fs_col_tma(in->fsg, a, st));
        return QSG_OK;
    }
    QSG_CUDA(qsg::launch_fs_col(in->prec, in->fsg, a, ninst, st));
    return QSG_OK;
}

// tensor maps (psi, V 0, V 1; V 0 stands in for an absent V 1) of
// instances, into device memory; null when a map cannot be made
void *fs_make_maps(qsg_ctx *ctx, qsg_inst *const *insts, size_t count, size_t *bytes)
{
    if (count == 0 || insts[0]->prec != 1 || !qsg::fs_tma_supported(1, insts[0]->fsg.n2)) return nullptr;
    struct alignas(64) Map { unsigned char b[128]; };
    std::vector<Map> h(3 * count);
    for (size_t k = 0; k < count; ++k) {
        qsg_inst *in = insts[k];
        const int n1 = in->fsg.n1, n2 = in->fsg.n2;
        const void *v1 = in->vtab[1] ? in->vtab[1] : in->vtab[0];
        if (!qsg::encode_fs_map(in->psi, n1, n2, h[3 * k].b) ||
            !qsg::encode_fs_map(const_cast<void *>(in->vtab[0]), n1, n2, h[3 * k + 1].b) ||
            !qsg::encode_fs_map(const_cast<void *>(v1), n1, n2, h[3 * k + 2].b))
            return nullptr;
    }
    void *d = nullptr;
    if (cudaMallocAsync(&d, sizeof(Map) * h.size(), ctx->st) != cudaSuccess) return nullptr;
    if (cudaMemcpyAsync(d, h.data(), sizeof(Map) * h.size(), cudaMemcpyHostToDevice, ctx->st) != cudaSuccess ||
        cudaStreamSynchronize(ctx->st) != cudaSuccess) {
        cudaFreeAsync(d, ctx->st);
        return nullptr;
    }
    *bytes = sizeof(Map) * h.size();
    return d;
}

int fs_row(qsg_inst *in, const qsg::FsInst *desc, int ninst, int ksel, cudaStream_t st)
{
    qsg::FsRowArgs a{};
    a.inst = desc;
    a.tw_row = in->tw_fs_row;
    a.ksel = ksel;
    a.inv_n = (float)(1.0 / (double)in->n);
    ProfScope ps(in->ctx, "fs_row_pass", st);
    QSG_CUDA(qsg::launch_fs_row(in->prec, in->fsg, a, ninst, st));
    return QSG_OK;
}

// Four-step schedule over ninst instances sharing in's geometry and tables
// layout (descriptors `desc`): like the 2D schedule with the roles of the
// passes swapped -- the column pass is the real-space one.
int step_fs(qsg_inst *in, const qsg::FsInst *desc, int ninst, uint64_t nsteps, cudaStream_t st,
            const void *maps = nullptr)
{
    int rc;
    for (uint64_t s = 0; s < nsteps; ++s) {
        const bool last = s + 1 == nsteps;
        if (s == 0 && (rc = fs_col(in, desc, ninst, false, true, 0, false, st, maps))) return rc;
        if (in->order == 2) {
            if ((rc = fs_row(in, desc, ninst, 0, st))) return rc;
        } else {
            if ((rc = fs_row(in, desc, ninst, 0, st))) return rc;
            if ((rc = fs_col(in, desc, ninst, true, true, 1, false, st, maps))) return rc;
            if ((rc = fs_row(in, desc, ninst, 1, st))) return rc;
            if ((rc = fs_col(in, desc, ninst, true, true, 1, false, st, maps))) return rc;
            if ((rc = fs_row(in, desc, ninst, 0, st))) return rc;
        }
        rc = last ? fs_col(in, desc, ninst, true, false, 0, false, st, maps)
                  : fs_col(in, desc, ninst, true, true, 0, true, st, maps);
        if (rc) return rc;
    }
    return QSG_OK;
}

// Bluestein four-step schedule (tables in build_bfs_tables): per kinetic
// substep the column pass with the diagonal before it (open / V / V c2), the
// row pass with the first kernel, the column pass with K_d, the row pass with
// the second kernel; the call ends with the column pass of the closing factor
// to natural order (its norm partials serve a renormalising call).
int step_bfs(qsg_inst *in, uint64_t nsteps, cudaStream_t st)
{
    auto row = [&](int ksel) -> int {
        qsg::FsRowArgs a{};
        a.inst = in->bdesc;
        a.tw_row = in->tw_fs_row;
        a.ksel = ksel;
        a.plain = 1;
        ProfScope ps(in->ctx, "fs_row_pass", st);
        QSG_CUDA(qsg::launch_fs_row(in->prec, in->fsg, a, 1, st));
        return QSG_OK;
    };
    const int nsub = in->order == 2 ? 1 : 3;
    int rc;
    for (uint64_t s = 0; s < nsteps; ++s) {
        for (int u = 0; u < nsub; ++u) {
            // O2: V1/2 T V1/2;  O4: VC1 TD1 VC2 TD2 VC2 TD1 VC1 (V factors at step joins merged, twice)
            if (u == 0) rc = s == 0 ? fs_col(in, in->bdesc + 0, 1, false, true, 0, false, st)
                                    : fs_col(in, in->bdesc + 0, 1, true, true, 1, true, st);
            else rc = fs_col(in, in->bdesc + 2, 1, true, true, 0, false, st);
            if (rc || (rc = row(0))) return rc;
            if ((rc = fs_col(in, in->bdesc + 1, 1, true, true, (in->order == 4 && u == 1) ? 1 : 0, false, st)))
                return rc;
            if ((rc = row(1))) return rc;
        }
    }
    return fs_col(in, in->bdesc + 2, 1, true, false, 1, false, st);
}

int step1d(qsg_inst *in, uint64_t nsteps, int renorm)
{
    qsg_ctx *ctx = in->ctx;
    if (in->wall_zero) {
        // A wall's 2n odd extension: the reference's wall ExpT discards sites 0 and n
        // before each transform (src/SplittingMethod1D.cpp:63-65) and rebuilds the odd
        // half.  Site n is 0 from the upload and the steps keep the extension odd to
        // rounding, so the caller's psi_0 is the one value to discard, once.  Zeroing
        // the two sites again before every transform feeds the rounding noise there
        // back into every mode; under a complex dt the O4 middle substep (d2 < 0)
        // multiplies the highest modes by exp(|d2| Im(dt) k^2 DT), and that loop grew
        // the error about 30x per step on fine grids.
        QSG_CUDA(cudaMemsetAsync(in->psi, 0, csize(in->prec), in->st));
        in->wall_zero = false;
    }
    if (in->blue) {
        qsg::BlueArgs a{};
        a.psi = in->psi;
        a.tw = in->tw;
        a.w = in->bw;
        a.hs = in->bhs;
        a.vtab[0] = in->vtab[0];
        a.vtab[1] = in->vtab[1];
        a.ktab[0] = in->ktab[0];
        a.ktab[1] = in->ktab[1];
        a.norm_out = renorm ? nullptr : in->snorm;
        in->snorm_valid = !renorm;
        a.dv = in->dv;
        a.nsteps = nsteps;
        a.n = (int)in->n;
        a.order = in->order;
        a.renormalize = renorm;
        a.norm_n = (int)user_n(in);
        ProfScope ps(ctx, "evolve1d_blue", in->st);
        QSG_CUDA(qsg::launch_evolve1d_blue(in->prec, in->blue_m, a, in->st));
        return QSG_OK;
    }
    if (!in->fourstep) {
        qsg::Evolve1DBatchArgs a{};
        a.inst = in->desc;
        a.tw = in->tw;
        // the kernel sums the final state's norm anyway when it renormalises;
        // otherwise one block reduction at the end of the call, which serves
        // qsg_step_norm2 / _post without a pass of their own
        a.norm_out = renorm ? nullptr : in->snorm;
        in->snorm_valid = !renorm;
        a.dv = in->d_dv;
        a.nsteps = nsteps;
        a.order = in->order;
        a.renormalize = renorm;
        a.count = 1;
        if (in->boundary == QSG_INFINITE_WALL) {
            ProfScope ps(ctx, "evolve1d_wall", in->st);
            QSG_CUDA(qsg::launch_wall1d(in->prec, (int)in->n, a, in->st));
            return QSG_OK;
        }
        ProfScope ps(ctx, "evolve1d_resident", in->st);
        QSG_CUDA(qsg::launch_evolve1d(in->prec, (int)in->n, a, in->st));
        return QSG_OK;
    }
    in->snorm_valid = false;
    int rc = in->bfs ? step_bfs(in, nsteps, in->st) : step_fs(in, in->desc, 1, nsteps, in->st, in->fs_maps);
    if (rc) return rc;
    if (renorm && in->wall_ext) {
        // Norm2 over the first n_out sites, then the whole extension scaled
        ProfScope ps(ctx, "renorm");
        int np = 0;
        QSG_CUDA(qsg::launch_reduce(in->prec, in->psi, in->V, 0, in->n_out, 0, ctx->partials, ctx->max_partials,
                                    &np, ctx->st));
        QSG_CUDA(qsg::launch_finalize(ctx->partials, np, 1, ctx->sums, ctx->st));
        QSG_CUDA(qsg::launch_renorm(in->prec, in->psi, in->n, ctx->sums, in->dv, ctx->st));
    } else if (renorm) {
        ProfScope ps(ctx, "renorm");
        QSG_CUDA(qsg::launch_finalize(in->parts, in->fsg.col_blocks, 1, ctx->sums, ctx->st));
        QSG_CUDA(qsg::launch_renorm(in->prec, in->psi, in->n, ctx->sums, in->dv, ctx->st));
    }
    return QSG_OK;
}

bool momentum(const qsg_inst *in) { return in->form == QSG_FORM_MOMENTUM; }

// real-space sum |psi|^2 / the column pass's sums: split-k scale G Ny (direct
// form) or Nx Ny (momentum form, Parseval)
double cparts_scale(const qsg_inst *in)
{
    return momentum(in) ? (double)in->nx * in->ny : (double)in->geom.g * in->ny;
}

// vdiff: the momentum form's increment pass, which runs with plain twiddles
int row_pass(qsg_inst *in, bool is, bool os, const void *v, bool vtwice, double *partials,
             const void *src = nullptr, void *dst = nullptr, bool vdiff = false)
{
    qsg::RowPassArgs a{};
    a.in = src ? src : in->psi;
    a.out = dst ? dst : in->psi;
    a.vtab = v;
    a.vtwice = vtwice ? 1 : 0;
    a.vdiff = vdiff ? 1 : 0;
    a.plain = vdiff ? 1 : 0;
    a.tw_row = vdiff ? in->tw_row_p : in->tw_row;
    a.tw_nx = vdiff ? in->tw_nx_p : in->tw_nx;
    a.partials = partials;
    a.nx = in->nx;
    a.m = in->geom.m;
    a.in_split = is ? 1 : 0;
    a.out_split = os ? 1 : 0;
    a.units = in->geom.row_blocks;
    ProfScope ps(in->ctx, "row_pass", in->st);
    QSG_CUDA(qsg::launch_row_pass(in->prec, in->geom, a, in->st));
    return QSG_OK;
}

// Momentum form: a pass whose transforms carry the whole state (the first of
// a call from natural psi, the last before a renormalising settle, the
// inverse-only pass of a settle) runs with hi + lo twiddles; the others with
// plain ones.  A plain transform's fixed operator error is harmless only where
// it is scaled by |V - 1|: on the whole state, repeated every step (a read
// after every step), it would add up coherently.
int col_pass(qsg_inst *in, int d, double *partials = nullptr, bool first = false, bool whole = false,
             bool inv_only = false, bool no_copies = false)
{
    qsg::ColPassArgs a{};
    a.partials = partials;
    a.psi = in->psi;
    a.work = momentum(in) ? in->work : nullptr;
    a.first = first ? 1 : 0;
    a.invonly = inv_only ? 1 : 0;
    a.plain = momentum(in) && !(first || whole || inv_only) ? 1 : 0;
    a.kx = in->kx[d];
    a.ky = in->ky[d];
    a.k2d = in->ktab[d];
    a.tw_col = a.plain ? in->tw_col_p : in->tw_col;
    a.nx = in->nx;
    a.ny = in->ny;
    a.g = in->geom.g;
    a.inv_n = (float)(1.0 / ((double)in->nx * in->ny));
    a.tiles = (in->ny / in->geom.col_w) * in->geom.g;
    a.err = reinterpret_cast<int *>(in->err);
    a.no_copies = no_copies ? 1 : 0;
    ProfScope ps(in->ctx, "col_pass", in->st);
    // a regular momentum-form pass: fed by tensor copies where the tile shape is compiled
    const qsg::Geom2D &g = in->geom;
    if (momentum(in) && !first && !inv_only && in->ctx->col_tma && qsg::col_tma_supported(g.m, g.col_e, g.col_w)) {
        if (in->tma_m != g.m || in->tma_w != g.col_w) {
            in->tma_m = g.m;
            in->tma_w = qsg::encode_col_tma_maps(in->work, in->psi, in->nx, in->ny, g.col_w, in->tmaps) ? g.col_w : -1;
        }
        if (in->tma_w > 0) {
            QSG_CUDA(qsg::launch_col_pass_tma(g, a, in->tmaps, in->st));
            return QSG_OK;
        }
    }
    if (no_copies) return fail(QSG_ERR_UNSUPPORTED, "no tensor-copy column pass for this instance and plan");
    QSG_CUDA(qsg::launch_col_pass(in->prec, in->geom, a, in->st));
    return QSG_OK;
}

// Momentum form of the same step.  The state P = F psi / (Nx Ny) stays in
// psi; work carries W = (column iFFT of P), the row pass's split-k input.
// An ExpV is P += F[(V - 1) F^-1 P]: the row pass turns W into the increment's
// split-k form in place (row iFFT, x (V - 1), row FFT), the next column pass
// transforms it, adds it to P, applies the kinetic factor to P, stores P and
// writes the new W.  The closing ExpV of a call is deferred as in the direct
// form; settling runs it on W into natural psi.
int step2d_momentum(qsg_inst *in, uint64_t nsteps, int renorm, double *parts)
{
    int rc;
    const void *V0 = in->vtab[0], *V1 = in->vtab[1];
    void *W = in->work;
    for (uint64_t s = 0; s < nsteps; ++s) {
        const bool last = s + 1 == nsteps;
        bool first = false;
        if (s == 0) {
            // opening ExpV: natural psi -> the split-k form of exp(V) psi
            // (transformed whole: P does not exist yet), or the increment of
            // the merged closing + opening factors
            if (in->pending)
                rc = row_pass(in, true, true, V0, true, nullptr, W, W, true);
            else
                rc = row_pass(in, false, true, V0, false, nullptr, in->psi, W), first = true;
            if (rc) return rc;
        }
        in->pending = false;
        double *cp = last && !renorm ? in->cparts : nullptr;
        const bool closing = last && renorm;  // the next pass takes W to natural psi
        if (in->order == 2) {
            if ((rc = col_pass(in, 0, cp, first, closing))) return rc;
        } else {
            if ((rc = col_pass(in, 0, nullptr, first))) return rc;
            if ((rc = row_pass(in, true, true, V1, false, nullptr, W, W, true))) return rc;
            if ((rc = col_pass(in, 1))) return rc;
            if ((rc = row_pass(in, true, true, V1, false, nullptr, W, W, true))) return rc;
            if ((rc = col_pass(in, 0, cp, false, closing))) return rc;
        }
        if (last && renorm)
            rc = row_pass(in, true, false, V0, false, parts, W, in->psi);
        else if (last)
            in->pending = true;
        else
            rc = row_pass(in, true, true, V0, true, nullptr, W, W, true);
        if (rc) return rc;
    }
    return QSG_OK;
}

// 2D step on a grid without a power-of-two plan (qsg_blue.cuh): natural layout,
// R(V, row DFT) then per substep C(column DFT, K, inverse) R(inverse row DFT, V,
// row DFT), the last row pass of the call ending in natural rows (no deferral)
int step2d_blue(qsg_inst *in, uint64_t nsteps, int renorm)
{
    qsg_ctx *ctx = in->ctx;
    auto row = [&](bool in_k, const void *v, bool twice, bool out_k) -> int {
        qsg::Blue2DArgs a{};
        a.psi = in->psi;
        a.vtab = v;
        a.vtwice = twice ? 1 : 0;
        a.in_k = in_k ? 1 : 0;
        a.out_k = out_k ? 1 : 0;
        a.tw = in->btwy;
        a.w = in->bwy;
        a.hs = in->bhsy;
        a.nx = in->nx;
        a.ny = in->ny;
        ProfScope ps(ctx, "row_pass_blue", in->st);
        QSG_CUDA(qsg::launch_row_blue(in->prec, in->bmy, a, in->st));
        return QSG_OK;
    };
    auto col = [&](int d) -> int {
        qsg::Blue2DArgs a{};
        a.psi = in->psi;
        a.tw = in->btwx;
        a.w = in->bwx;
        a.hs = in->bhsx;
        a.kx = in->bkx[d];
        a.ky = in->bky[d];
        a.nx = in->nx;
        a.ny = in->ny;
        ProfScope ps(ctx, "col_pass_blue", in->st);
        QSG_CUDA(qsg::launch_col_blue(in->prec, in->bmx, a, false, 0, 0, nullptr, in->st));
        return QSG_OK;
    };
    const int nsub = in->order == 2 ? 1 : 3;
    int rc;
    if ((rc = row(false, in->vtab[0], false, true))) return rc;
    for (uint64_t s = 0; s < nsteps; ++s) {
        for (int u = 0; u < nsub; ++u) {
            // O2: V1/2 T V1/2;  O4: VC1 TD1 VC2 TD2 VC2 TD1 VC1 (tables 0: C1 / D1, 1: C2 / D2)
            if ((rc = col(in->order == 4 && u == 1 ? 1 : 0))) return rc;
            const bool last = u == nsub - 1;
            if (last && s + 1 == nsteps)
                rc = row(true, in->vtab[0], false, false);
            else
                rc = row(true, (in->order == 4 && !last) ? in->vtab[1] : in->vtab[0], last, true);
            if (rc) return rc;
        }
    }
    if (renorm) {
        ProfScope ps(ctx, "renorm");
        int np = 0;
        QSG_CUDA(qsg::launch_reduce(in->prec, in->psi, in->V, 0, in->n, 0, ctx->partials, ctx->max_partials, &np,
                                    ctx->st));
        QSG_CUDA(qsg::launch_finalize(ctx->partials, np, 1, ctx->sums, ctx->st));
        QSG_CUDA(qsg::launch_renorm(in->prec, in->psi, in->n, ctx->sums, in->dv, ctx->st));
    }
    return QSG_OK;
}

int step2d(qsg_inst *in, uint64_t nsteps, int renorm)
{
    qsg_ctx *ctx = in->ctx;
    if (in->blue2) return step2d_blue(in, nsteps, renorm);
    double *parts = nullptr;
    if (renorm) {
        if (in->geom.row_blocks > ctx->max_partials)
            return fail(QSG_ERR_STATE, "partials buffer too small");
        parts = ctx->partials;
    }
    int rc;
    const void *V0 = in->vtab[0], *V1 = in->vtab[1];
    if (momentum(in)) {
        if ((rc = step2d_momentum(in, nsteps, renorm, parts))) return rc;
        nsteps = 0;
    }
    for (uint64_t s = 0; s < nsteps; ++s) {
        const bool last = s + 1 == nsteps;
        // opening V factor: on natural rows, or merged with the deferred closing one
        if (s == 0 && (rc = row_pass(in, in->pending, true, V0, in->pending, nullptr))) return rc;
        in->pending = false;
        // the last column pass of a deferred call also sums the norm
        double *cp = last && !renorm ? in->cparts : nullptr;
        if (in->order == 2) {
            if ((rc = col_pass(in, 0, cp))) return rc;
        } else {
            if ((rc = col_pass(in, 0))) return rc;
            if ((rc = row_pass(in, true, true, V1, false, nullptr))) return rc;
            if ((rc = col_pass(in, 1))) return rc;
            if ((rc = row_pass(in, true, true, V1, false, nullptr))) return rc;
            if ((rc = col_pass(in, 0, cp))) return rc;
        }
        if (last && renorm)
            rc = row_pass(in, true, false, V0, false, parts);
        else if (last)
            in->pending = true;  // closing V factor deferred
        else
            rc = row_pass(in, true, true, V0, true, nullptr);
        if (rc) return rc;
    }
    if (renorm) {
        ProfScope ps(ctx, "renorm");
        QSG_CUDA(qsg::launch_finalize(ctx->partials, in->geom.row_blocks, 1, ctx->sums, ctx->st));
        QSG_CUDA(qsg::launch_renorm(in->prec, in->psi, in->n, ctx->sums, in->dv, ctx->st));
    }
    return QSG_OK;
}

// 3D: one pass over the lines of an axis (0 x, 1 y, 2 z): [vpre] F^-1 K F [vpost]
template <class T>
int pass3(qsg_inst *in, int ax, int ktab, const void *vpre, bool pre2, const void *vpost, bool post2, double *kin)
{
    qsg::Pass3Args a{};
    a.psi = in->psi;
    a.vpre = vpre;
    a.vpre_twice = pre2 ? 1 : 0;
    a.vpost = vpost;
    a.vpost_twice = post2 ? 1 : 0;
    a.k = in->k3[ax][ktab];
    a.tw = in->tw3[ax];
    a.partials = kin;
    a.kinetic = kin ? 1 : 0;
    const int nx = in->nx, ny = in->ny, nz = in->nz;
    const int L[3] = {nx, ny, nz};
    a.inv_l = (float)(1.0 / L[ax]);
    if (ax == 2) {
        ProfScope ps(in->ctx, "pass3_z", in->st);
        QSG_CUDA(qsg::launch3_row<T>(nz, (size_t)nx * ny, a, in->st));
    } else if (ax == 1) {
        a.s_line = nz;
        a.s_outer = (long long)ny * nz;
        ProfScope ps(in->ctx, "pass3_y", in->st);
        QSG_CUDA(qsg::launch3_col<T>(ny, nz, nx, a, in->st));
    } else {
        a.s_line = (long long)ny * nz;
        a.s_outer = nz;
        ProfScope ps(in->ctx, "pass3_x", in->st);
        QSG_CUDA(qsg::launch3_col<T>(nx, nz, ny, a, in->st));
    }
    return QSG_OK;
}

// O2: z[V V', Kz] y[Ky] x[Kx, (V)];  O4: z[V1 V1', K1] y x[V2] z[K2] y x[V2] z[K1] y x[(V1)]
template <class T> int step3d_t(qsg_inst *in, uint64_t nsteps, int renorm)
{
    int rc;
    const void *V0 = in->vtab[0], *V1 = in->vtab[1];
    for (uint64_t s = 0; s < nsteps; ++s) {
        const bool last = s + 1 == nsteps;
        const void *close = last ? V0 : nullptr;
        if (in->order == 2) {
            if ((rc = pass3<T>(in, 2, 0, V0, s > 0, nullptr, false, nullptr))) return rc;
            if ((rc = pass3<T>(in, 1, 0, nullptr, false, nullptr, false, nullptr))) return rc;
            if ((rc = pass3<T>(in, 0, 0, nullptr, false, close, false, nullptr))) return rc;
        } else {
            if ((rc = pass3<T>(in, 2, 0, V0, s > 0, nullptr, false, nullptr))) return rc;
            if ((rc = pass3<T>(in, 1, 0, nullptr, false, nullptr, false, nullptr))) return rc;
            if ((rc = pass3<T>(in, 0, 0, nullptr, false, V1, false, nullptr))) return rc;
            if ((rc = pass3<T>(in, 2, 1, nullptr, false, nullptr, false, nullptr))) return rc;
            if ((rc = pass3<T>(in, 1, 1, nullptr, false, nullptr, false, nullptr))) return rc;
            if ((rc = pass3<T>(in, 0, 1, nullptr, false, V1, false, nullptr))) return rc;
            if ((rc = pass3<T>(in, 2, 0, nullptr, false, nullptr, false, nullptr))) return rc;
            if ((rc = pass3<T>(in, 1, 0, nullptr, false, nullptr, false, nullptr))) return rc;
            if ((rc = pass3<T>(in, 0, 0, nullptr, false, close, false, nullptr))) return rc;
        }
    }
    (void)renorm;
    return QSG_OK;
}

int step3d(qsg_inst *in, uint64_t nsteps, int renorm)
{
    int rc = in->prec == 1 ? step3d_t<float>(in, nsteps, renorm) : step3d_t<double>(in, nsteps, renorm);
    if (rc || !renorm) return rc;
    // renormalise at the end of the call, as 2D does (QuEvolverImpl::Step, src/EvolverImpl.cpp:56-68)
    qsg_ctx *ctx = in->ctx;
    int np = 0;
    QSG_CUDA(qsg::launch_reduce(in->prec, in->psi, in->V, 0, in->n, 0, ctx->partials, ctx->max_partials, &np, ctx->st));
    QSG_CUDA(qsg::launch_finalize(ctx->partials, np, 1, ctx->sums, ctx->st));
    QSG_CUDA(qsg::launch_renorm(in->prec, in->psi, in->n, ctx->sums, in->dv, ctx->st));
    return QSG_OK;
}

// <T> of a 3D state: per axis, sum |F_a psi|^2 fold^2 DT_a / sum |F_a psi|^2 (Parseval over
// the other two axes makes these the full transform's ratios), summed over the axes
int kinetic3d(qsg_inst *in, double *kin)
{
    qsg_ctx *ctx = in->ctx;
    const int L[3] = {in->nx, in->ny, in->nz};
    const double D[3] = {in->dx, in->dy, in->dz};
    double total = 0;
    for (int ax = 0; ax < 3; ++ax) {
        const int ctas = ax == 2 ? qsg::row3_ctas(in->prec, in->nz, (size_t)in->nx * in->ny)
                                 : qsg::col3_ctas(in->prec, L[ax], in->nz, ax == 1 ? in->nx : in->ny);
        int rc = in->prec == 1 ? pass3<float>(in, ax, 0, nullptr, false, nullptr, false, in->kparts3)
                               : pass3<double>(in, ax, 0, nullptr, false, nullptr, false, in->kparts3);
        if (rc) return rc;
        std::vector<double> h(2 * (size_t)ctas);
        QSG_CUDA(cudaMemcpyAsync(h.data(), in->kparts3, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, ctx->st));
        QSG_CUDA(cudaStreamSynchronize(ctx->st));
        double s1 = 0, s0 = 0;
        for (int c = 0; c < ctas; ++c) {
            s1 += h[2 * c];
            s0 += h[2 * c + 1];
        }
        const double dk = 2 * kPi / (D[ax] * L[ax]);
        total += (dk * in->hbar) * (dk * in->hbar) / (2 * in->mass) * (s1 / s0);
    }
    *kin = total;
    return QSG_OK;
}

// run the deferred closing row pass: psi back to natural real space
int settle(qsg_inst *in)
{
    if (!in->pending) return QSG_OK;
    int rc;
    if (momentum(in)) {
        // W again from the stored state, with hi + lo twiddles (the stepping
        // passes made it with plain ones), then to natural psi
        if ((rc = col_pass(in, 0, nullptr, false, false, true))) return rc;
        rc = row_pass(in, true, false, in->vtab[0], false, nullptr, in->work, in->psi);
    } else {
        rc = row_pass(in, true, false, in->vtab[0], false, nullptr);
    }
    if (rc) return rc;
    in->pending = false;
    return QSG_OK;
}

// An instance whose state a timed-out pass left half-updated refuses every
// call but qsg_set_psi (and destruction).
int lost_state(const qsg_inst *in, const char *who)
{
    if (!in->lost) return QSG_OK;
    return fail(QSG_ERR_TIMEOUT, std::string(who) +
                                     ": the instance's state was lost when a pass gave up waiting for its tensor "
                                     "copies (bounded wait); set a new state with qsg_set_psi");
}

// Queue a copy of the instance's failure counter into the pinned slot
// host_sums[7], on the stream whose synchronisation the caller waits for next.
int queue_err_copy(qsg_inst *in, cudaStream_t st)
{
    QSG_CUDA(cudaMemcpyAsync(in->ctx->host_sums + 7, in->err, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    return QSG_OK;
}

// After that synchronisation: a count above the acknowledged one means a pass
// of this instance (or of its batched launch) ran out of time since the last
// check, so its state is lost; report that (QSG_ERR_TIMEOUT) now and on every
// later call until qsg_set_psi.
int err_after_sync(qsg_inst *in, const char *who)
{
    unsigned count = 0;
    std::memcpy(&count, in->ctx->host_sums + 7, sizeof(unsigned));
    if (count != in->err_seen) {
        in->err_seen = count;
        in->lost = true;
    }
    return lost_state(in, who);
}

// pinned slot of the failure counter copied with posted norm `slot`
unsigned *ring_err(qsg_inst *in, int slot)
{
    return reinterpret_cast<unsigned *>(in->ring_host + qsg_inst::kRing) + slot;
}

// synchronise `st` and check the instance's failure counter
int sync_checked(qsg_inst *in, cudaStream_t st, const char *who)
{
    if (int rc = queue_err_copy(in, st)) return rc;
    QSG_CUDA(cudaStreamSynchronize(st));
    return err_after_sync(in, who);
}

// sum over psi[lo, hi) with the given reduction mode; synchronous

int reduce(qsg_inst *in, size_t lo, size_t hi, int mode, double *out)
{
    if (int rc = settle(in)) return rc;
    qsg_ctx *ctx = in->ctx;
    int np = 0;
    QSG_CUDA(qsg::launch_reduce(in->prec, in->psi, in->V, lo, hi, mode, ctx->partials, ctx->max_partials,
                                &np, ctx->st));
    QSG_CUDA(qsg::launch_finalize(ctx->partials, np, 1, ctx->sums, ctx->st));
    QSG_CUDA(cudaMemcpyAsync(ctx->host_sums, ctx->sums, sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
    if (int rc = sync_checked(in, ctx->st, "reduction")) return rc;
    *out = ctx->host_sums[0];
    return QSG_OK;
}

// complex factors computed on the host (long double) into a new device array of
// the instance's precision
int upload_factors(qsg_inst *in, const std::vector<std::complex<long double>> &src, void **dst)
{
    const size_t cs = csize(in->prec);
    if (int r = inst_alloc(in, src.size() * cs, dst)) return r;
    std::vector<unsigned char> h(src.size() * cs);
    for (size_t i = 0; i < src.size(); ++i) {
        if (in->prec == 0) {
            const double v[2] = {(double)src[i].real(), (double)src[i].imag()};
            std::memcpy(&h[i * cs], v, cs);
        } else {
            const float v[2] = {(float)src[i].real(), (float)src[i].imag()};
            std::memcpy(&h[i * cs], v, cs);
        }
    }
    // pageable source: the call returns once the bytes are staged
    QSG_CUDA(cudaMemcpyAsync(*dst, h.data(), h.size(), cudaMemcpyHostToDevice, in->ctx->st));
    return QSG_OK;
}

// --- 1D plans ----------------------------------------------------------------

// The timing resources of a tuner, given back on every path out: its two
// events, and the context's profiling mode (off while it times).
struct TuneGuard {
    qsg_ctx *ctx;
    int prof;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    explicit TuneGuard(qsg_ctx *c) : ctx(c), prof(c->prof) { c->prof = 0; }
    ~TuneGuard()
    {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        ctx->prof = prof;
    }
    TuneGuard(const TuneGuard &) = delete;
    TuneGuard &operator=(const TuneGuard &) = delete;
};

// four-step plans of a stepped length n: the default split first, then the
// others from the longest rows down, each with and without tensor-copy columns
void add_fs_plans(int prec, uint64_t n, bool tma_ok, std::vector<qsg_plan1d> &out)
{
    const int d = qsg::fs_default_n1(n);
    std::vector<int> n1s{d};
    for (int n1 = 4096; n1 >= 64; n1 >>= 1)
        if (n1 != d) n1s.push_back(n1);
    for (int n1 : n1s) {
        qsg::FsGeom g;
        if (!qsg::fs_geom(prec, n, &g, n1)) continue;
        out.push_back(qsg_plan1d{1, n1, 0, 0});
        if (tma_ok && qsg::fs_tma_supported(prec, g.n2)) out.push_back(qsg_plan1d{1, n1, 1, 0});
    }
}

// Bluestein on the four-step passes: the buffer length M (the smallest power of
// two >= 2 len - 1) for a transform of len sites, 0 where the passes do not reach
uint64_t bfs_len_m(int prec, uint64_t len, qsg::FsGeom *g)
{
    if (len < 2) return 0;
    uint64_t m = 1;
    while (m < 2 * len - 1) m <<= 1;
    return qsg::fs_geom(prec, m, g) ? m : 0;
}

// every plan of a 1D instance of n sites (the default first)
void plans_1d(int prec, uint64_t n, int boundary, std::vector<qsg_plan1d> &out)
{
    out.clear();
    if (prec != QSG_FP64 && prec != QSG_MIXED) return;
    const bool pow2 = n >= 1 && (n & (n - 1)) == 0;
    if (boundary == QSG_INFINITE_WALL) {
        if (!pow2 || n < 64) {
            // any other length: Bluestein transforms of the 2n odd extension, in one
            // kernel or (longer) on the four-step passes
            qsg::FsGeom g;
            if (n >= 2 && qsg::blue_m_for(prec, 2 * n)) out.push_back(qsg_plan1d{0, 0, 0, 0});
            else if (bfs_len_m(prec, 2 * n, &g)) out.push_back(qsg_plan1d{1, g.n1, 0, 0});
            return;
        }
        if (n > 4194304) return;
        if (qsg::wall1d_supported(prec, n)) out.push_back(qsg_plan1d{0, 0, 0, 0});
        else add_fs_plans(prec, 2 * n, false, out);  // the periodic 2n odd extension
        return;
    }
    if (boundary != QSG_PERIOD) return;
    if (!pow2 || n < 64) {
        qsg::FsGeom g;
        if (qsg::blue_m_for(prec, n)) out.push_back(qsg_plan1d{0, 0, 0, 0});
        else if (bfs_len_m(prec, n, &g)) out.push_back(qsg_plan1d{1, g.n1, 0, 0});
        return;
    }
    if (qsg::evolve1d_supported(prec, n)) out.push_back(qsg_plan1d{0, 0, 0, 0});
    add_fs_plans(prec, n, true, out);
}

bool same_plan1d(const qsg_plan1d &a, const qsg_plan1d &b)
{
    return a.kind == b.kind && (a.kind == 0 || (a.n1 == b.n1 && a.tma == b.tma));
}

bool plan1d_valid(int prec, uint64_t n, int boundary, const qsg_plan1d &p)
{
    std::vector<qsg_plan1d> c;
    plans_1d(prec, n, boundary, c);
    for (const auto &q : c)
        if (same_plan1d(q, p)) return true;
    return false;
}

// norm partials of the four-step passes: one per column-pass CTA, n / 4096
// (complex64) or n / 2048 (complex128) whatever the split; 0 where no
// four-step plan exists
int fs_parts_for(const qsg_inst *in)
{
    if (in->dim != 1 || in->blue) return 0;
    qsg::FsGeom g;
    if (!qsg::fs_geom(in->prec, in->n, &g)) return 0;
    return g.col_blocks;
}

// 1D periodic kinetic tables of the instance's current layout (natural for
// one-CTA kernels, row layout for four-step passes), shared across instances
int build_ktab_1d(qsg_inst *in)
{
    qsg_ctx *ctx = in->ctx;
    const SplitConsts sc;
    const int ntab = in->order == 2 ? 1 : 2;
    const double tc[2] = {in->order == 2 ? 1.0 : sc.d1, sc.d2};
    const size_t cs = csize(in->prec);
    const cd I(0, 1);
    int rc;
    // ExpT periodic: f = -i DT dt t / hbar, DT = (Dk hbar)^2/(2m), Dk = 2 pi/(dx N)
    // (SplittingMethod1D.cpp:51-53).  A wall extension of N = 2 n sites gets the
    // same table: Dk = 2 pi/(dx 2n) is the wall's Dp/hbar = pi/(dx n)
    // (SplittingMethod1D.cpp:72-74), and two inverse 2n-transforms with the
    // final -1/(2n) equal a forward and an inverse one with 1/(2n) on an odd
    // sequence, whose transform is odd as well
    const double dk = 2 * kPi / (in->dx * in->n);
    const double DT = (dk * in->hbar) * (dk * in->hbar) / (2 * in->mass);
    for (int k = 0; k < ntab; ++k) {
        const cd f = -I * DT * in->dt * tc[k] / in->hbar;
        // shared by every instance of the context with the same size and coefficient (a batch of
        // equal-dx, equal-dt instances reads one table per size from L2 instead of one each);
        // key (precision, n1, n2) for the four-step layout, (precision, n, 0) for the natural one
        const auto key = in->fourstep ? std::make_tuple(in->prec, in->fsg.n1, in->fsg.n2, f.real(), f.imag())
                                      : std::make_tuple(in->prec, (int)in->n, 0, f.real(), f.imag());
        auto it = ctx->fs_ktabs.find(key);
        const bool fresh = it == ctx->fs_ktabs.end();
        if (fresh) {
            void *p = nullptr;
            if ((rc = dev_alloc(ctx, in->n * cs, &p, nullptr))) return rc;
            it = ctx->fs_ktabs.emplace(key, qsg_ctx::SharedTable{p, in->n * cs, 0}).first;
        }
        // registered before the table is filled, so that releasing the instance
        // after a failed launch below also releases the table
        it->second.users += 1;
        in->shared_k.push_back(key);
        in->ktab[k] = it->second.p;
        if (fresh && in->fourstep) {
            QSG_CUDA(qsg::launch_ktable_fs(in->prec, it->second.p, in->fsg.n1, in->fsg.n2, f.real(), f.imag(),
                                           1.0 / (double)in->n, ctx->st));
        } else if (fresh) {
            QSG_CUDA(qsg::launch_ktable1d(in->prec, it->second.p, (int)in->n, f.real(), f.imag(),
                                          1.0 / (double)in->n, ctx->st));
        }
    }
    return QSG_OK;
}

// Tables of a Bluestein four-step instance: transforms of n = bfs_n sites (the
// user's n, or a wall's 2n odd extension) in a buffer of M = in->n sites.
// A kinetic substep x -> IDFT(K DFT x) is, with the chirp w_j =
// exp(-i pi j^2 / n) and circular convolutions C_h, C_h* by h = conj(w) and by
// w (length M), the product W* C_h* K C_h W (the chirps between the two DFTs
// cancel, 1/n goes into the second kernel).  A convolution is a forward
// transform, a product in frequency, an inverse: the column pass, the row pass
// with the kernel FFT_M(h) / M (or FFT_M(h*) / (M n)) as a plain product, the
// next column pass.  The diagonal factors meet in the column passes in natural
// layout: V w before the first convolution of a call ("open"), K_d between the
// two, V merged with w* and w between substeps (plain V), w* V at the end of a
// call ("close"); each is zero from n on, which truncates the convolutions'
// outputs and keeps the buffer zero there.  The chirp and FFT_M(h) / M come
// from double-double arithmetic; the phase factors are formed in double as the
// reference forms its own (exp(f V) and exp(f K), src/SplittingMethod1D.cpp:
// 51-53, 87), and uploaded as plain complex (complex128) or factor - 1 (complex64
// columns); the kernels are plain complex in both.
int build_bfs_tables(qsg_inst *in)
{
    const SplitConsts sc;
    const int ntab = in->order == 2 ? 1 : 2;
    const double vc[2] = {in->order == 2 ? 0.5 : sc.c1, sc.c2};
    const double tc[2] = {in->order == 2 ? 1.0 : sc.d1, sc.d2};
    using cl = std::complex<double>;
    const uint64_t n = in->bfs_n, M = in->n;
    const size_t cs = csize(in->prec);
    int rc;
    std::vector<cl> w, hs;
    qsg::blue_tables_dd(n, M, w, hs);  // chirp (zero above n), FFT_M(h) / M
    std::vector<double> Vh(n);
    QSG_CUDA(cudaMemcpyAsync(Vh.data(), in->V, n * 8, cudaMemcpyDeviceToHost, in->ctx->st));
    QSG_CUDA(cudaStreamSynchronize(in->ctx->st));
    // exp(f x) for f = a (-i dt / hbar) (ExpV: a = c, x = V; ExpT: a = d, x = fold(k)^2 DT)
    const cl mi_dt_h = cl(0, -1) * in->dt / in->hbar;
    auto phase = [&](double a, double x) { return std::exp(mi_dt_h * (a * x)); };
    // upload M natural values: complex64 as factor - 1, complex128 plain
    auto put = [&](const std::vector<cl> &v, void **dst, bool minus_one) -> int {
        if (int r = inst_alloc(in, M * cs, dst)) return r;
        std::vector<unsigned char> h(M * cs);
        for (uint64_t i = 0; i < M; ++i) {
            const cl z = (minus_one && in->prec == 1) ? v[i] - 1.0 : v[i];
            if (in->prec == 0) {
                const double d[2] = {(double)z.real(), (double)z.imag()};
                std::memcpy(&h[i * cs], d, cs);
            } else {
                const float f[2] = {(float)z.real(), (float)z.imag()};
                std::memcpy(&h[i * cs], f, cs);
            }
        }
        QSG_CUDA(cudaMemcpyAsync(*dst, h.data(), h.size(), cudaMemcpyHostToDevice, in->ctx->st));
        QSG_CUDA(cudaStreamSynchronize(in->ctx->st));  // h is pageable and goes out of scope
        return QSG_OK;
    };
    std::vector<cl> t(M);
    auto fill = [&](auto f) {
        for (uint64_t j = 0; j < M; ++j) t[j] = j < n ? f(j) : cl(0);
    };
    // a wall's 2n odd extension: KinEn transforms it with sites 0 and n / 2 zeroed
    // (src/SplittingMethod1D.cpp:112-114); the steps zero site 0 once per uploaded state
    const bool wall = in->wall_ext;
    auto mask = [&](uint64_t j) { return wall && (j == 0 || j == n / 2) ? 0.0 : 1.0; };
    void *open = nullptr, *vc1 = nullptr, *vc2 = nullptr, *close = nullptr, *k1 = nullptr, *k2 = nullptr;
    void *chirp = nullptr, *h1 = nullptr, *h2 = nullptr;
    fill([&](uint64_t j) { return w[j] * phase(vc[0], Vh[j]); });
    if ((rc = put(t, &open, true))) return rc;
    fill([&](uint64_t j) { return phase(vc[0], Vh[j]); });  // applied twice at step joins
    if ((rc = put(t, &vc1, true))) return rc;
    fill([&](uint64_t j) { return std::conj(w[j]) * phase(vc[0], Vh[j]); });
    if ((rc = put(t, &close, true))) return rc;
    if (ntab == 2) {
        fill([&](uint64_t j) { return phase(vc[1], Vh[j]); });
        if ((rc = put(t, &vc2, true))) return rc;
    }
    // ExpT periodic (SplittingMethod1D.cpp:51-53): DT = (Dk hbar)^2 / (2m), Dk = 2 pi / (dx n);
    // on a wall's 2n extension Dk = pi / (dx n_wall), the wall ExpT's (:72-74)
    const double dk = 2 * kPi / (in->dx * (double)n);
    const double DT = (dk * in->hbar) * (dk * in->hbar) / (2 * in->mass);
    auto fold2 = [&](uint64_t k) {
        const double f = (double)(k > n / 2 ? n - k : k);
        return f * f * DT;
    };
    fill([&](uint64_t k) { return phase(tc[0], fold2(k)); });
    if ((rc = put(t, &k1, true))) return rc;
    if (ntab == 2) {
        fill([&](uint64_t k) { return phase(tc[1], fold2(k)); });
        if ((rc = put(t, &k2, true))) return rc;
    }
    fill([&](uint64_t j) { return mask(j) * w[j]; });
    if ((rc = put(t, &chirp, true))) return rc;
    // the kernels in the row pass's layout: position k2 n1 + k1 holds frequency k2 + n2 k1
    const uint64_t n1 = (uint64_t)in->fsg.n1, n2 = (uint64_t)in->fsg.n2;
    for (uint64_t k2 = 0; k2 < n2; ++k2)
        for (uint64_t k1 = 0; k1 < n1; ++k1) t[k2 * n1 + k1] = hs[k2 + n2 * k1];
    if ((rc = put(t, &h1, false))) return rc;
    // FFT_M(h*)_k = conj(FFT_M(h)_{-k}), with the 1/n of the inverse DFT
    for (uint64_t k2 = 0; k2 < n2; ++k2)
        for (uint64_t k1 = 0; k1 < n1; ++k1) {
            const uint64_t k = k2 + n2 * k1;
            t[k2 * n1 + k1] = std::conj(hs[(M - k) % M]) / (double)n;
        }
    if ((rc = put(t, &h2, false))) return rc;
    // KinEn weights of the n frequencies: fold(k)^2 DT with the periodic branch's DT
    // (it omits hbar^2, src/SplittingMethod1D.cpp:101-102), the wall's with it (:117-119;
    // |F|^2 of the odd extension is even, so the ratio over the 2n frequencies is the
    // wall's over k < n)
    {
        const double DTk = wall ? DT : dk * dk / (2 * in->mass);
        std::vector<double> kw(n);
        for (uint64_t k = 0; k < n; ++k) {
            const double f = (double)(k > n / 2 ? n - k : k);
            kw[k] = f * f * DTk;
        }
        void *p = nullptr;
        if ((rc = inst_alloc(in, n * 8, &p))) return rc;
        in->bkw = static_cast<double *>(p);
        QSG_CUDA(cudaMemcpyAsync(in->bkw, kw.data(), n * 8, cudaMemcpyHostToDevice, in->ctx->st));
        QSG_CUDA(cudaStreamSynchronize(in->ctx->st));
    }
    // descriptors (the closing pass's norm partials are set in common_create)
    qsg::FsInst h[4] = {};
    for (auto &d : h) {
        d.psi = in->psi;
        d.ktab[0] = h1;
        d.ktab[1] = h2;
    }
    h[0].vtab[0] = open;
    h[0].vtab[1] = vc1;
    h[1].vtab[0] = k1;
    h[1].vtab[1] = k2;
    h[2].vtab[0] = vc2;
    h[2].vtab[1] = close;
    h[3].vtab[0] = chirp;
    in->bchirp = chirp;
    in->bh1 = h1;
    void *bd = nullptr;
    if ((rc = inst_alloc(in, sizeof(h), &bd))) return rc;
    in->bdesc = static_cast<qsg::FsInst *>(bd);
    QSG_CUDA(cudaMemcpyAsync(in->bdesc, h, sizeof(h), cudaMemcpyHostToDevice, in->ctx->st));
    QSG_CUDA(cudaStreamSynchronize(in->ctx->st));
    return QSG_OK;
}

int build_tables(qsg_inst *in)
{
    qsg_ctx *ctx = in->ctx;
    const SplitConsts sc;
    const int ntab = in->order == 2 ? 1 : 2;
    const double vc[2] = {in->order == 2 ? 0.5 : sc.c1, sc.c2};
    const double tc[2] = {in->order == 2 ? 1.0 : sc.d1, sc.d2};
    const size_t cs = csize(in->prec);
    const cd I(0, 1);
    int rc;
    if (in->bfs) return build_bfs_tables(in);
    for (int k = 0; k < ntab; ++k) {
        // ExpV coefficient -i/hbar * dt * c (SplittingMethod1D.cpp:87, SplittingMethod2D.cpp:43-50)
        const cd f = (-I / in->hbar) * in->dt * vc[k];
        if ((rc = inst_alloc(in, in->n * cs, &in->vtab[k]))) return rc;
        QSG_CUDA(qsg::launch_vtable(in->prec, in->vtab[k], in->V, in->n, f.real(), f.imag(), ctx->st));
    }
    if (in->dim == 1 && in->boundary == QSG_INFINITE_WALL && !in->wall_ext) {
        // ExpT wall: K_i = exp(f i^2), f = -i DT dt t / hbar, DT = Dp^2/(2m), Dp = hbar pi/(dx N),
        // with the final -1/(2N) folded into the complex128 table (SplittingMethod1D.cpp:72-80)
        const double dp = in->hbar * kPi / (in->dx * in->n);
        const double DT = dp * dp / (2 * in->mass);
        for (int k = 0; k < ntab; ++k) {
            const cd f = -I * DT * in->dt * tc[k] / in->hbar;
            if ((rc = inst_alloc(in, in->n * cs, &in->ktab[k]))) return rc;
            QSG_CUDA(qsg::launch_ktable_wall(in->prec, in->ktab[k], (int)in->n, f.real(), f.imag(),
                                             -1.0 / (2.0 * (double)in->n), ctx->st));
        }
    } else if (in->dim == 1 && in->blue) {
        // Bluestein: chirp, FFT_M(conj chirp) / M and K_k / n (k < n, 0 above) as plain
        // complex factors, computed in long double (K as in the periodic branch below)
        const int m = in->blue_m;
        const uint64_t n = in->n;
        std::vector<std::complex<long double>> w, hs;
        qsg::blue_tables(n, m, w, hs);
        const long double dk = 2 * (long double)kPi / ((long double)in->dx * n);
        const long double DT = (dk * in->hbar) * (dk * in->hbar) / (2 * (long double)in->mass);
        std::vector<std::vector<std::complex<long double>>> kt(ntab, std::vector<std::complex<long double>>(m, 0.0L));
        for (int k = 0; k < ntab; ++k) {
            // exp(f q), f = -i DT dt t / hbar: real part DT q t Im(dt) / hbar, imaginary -DT q t Re(dt) / hbar
            for (uint64_t i = 0; i < n; ++i) {
                const long double fo = (long double)(i > n / 2 ? n - i : i), q = fo * fo;
                const long double re = DT * q * tc[k] * (long double)in->dt.imag() / in->hbar;
                const long double im = -DT * q * tc[k] * (long double)in->dt.real() / in->hbar;
                kt[k][i] = std::exp(re) * std::complex<long double>(cosl(im), sinl(im)) / (long double)n;
            }
        }
        if ((rc = upload_factors(in, w, &in->bw))) return rc;
        if ((rc = upload_factors(in, hs, &in->bhs))) return rc;
        for (int k = 0; k < ntab; ++k)
            if ((rc = upload_factors(in, kt[k], &in->ktab[k]))) return rc;
    } else if (in->dim == 2 && in->blue2) {
        // per side: Bluestein tables; per kinetic coefficient d: exp(a d DTx fold(i)^2) / (nx ny)
        // and exp(a d DTy fold(j)^2), a = -i dt / hbar (SplittingMethod2D::InitExpT,
        // src/SplittingMethod2D.cpp:56-79, as a product of the two axes' factors)
        std::vector<std::complex<long double>> w, hs;
        qsg::blue_tables(in->nx, in->bmx, w, hs);
        if ((rc = upload_factors(in, w, &in->bwx))) return rc;
        if ((rc = upload_factors(in, hs, &in->bhsx))) return rc;
        qsg::blue_tables(in->ny, in->bmy, w, hs);
        if ((rc = upload_factors(in, w, &in->bwy))) return rc;
        if ((rc = upload_factors(in, hs, &in->bhsy))) return rc;
        const long double nn = (long double)in->nx * in->ny;
        for (int k = 0; k < ntab; ++k) {
            const long double d = in->order == 2 ? 1.0L : (long double)tc[k];
            for (int ax = 0; ax < 2; ++ax) {
                const int L = ax == 0 ? in->nx : in->ny;
                const long double D = ax == 0 ? in->dx : in->dy;
                const long double dk = 2 * (long double)kPi / (D * L);
                const long double DT = (dk * in->hbar) * (dk * in->hbar) / (2 * (long double)in->mass);
                std::vector<std::complex<long double>> f(L);
                for (int i = 0; i < L; ++i) {
                    const long double fo = (long double)(i > L / 2 ? L - i : i), q = fo * fo * DT * d;
                    const long double re = q * (long double)in->dt.imag() / in->hbar;
                    const long double im = -q * (long double)in->dt.real() / in->hbar;
                    f[i] = std::exp(re) * std::complex<long double>(cosl(im), sinl(im)) / (ax == 0 ? nn : 1.0L);
                }
                if ((rc = upload_factors(in, f, ax == 0 ? &in->bkx[k] : &in->bky[k]))) return rc;
            }
        }
    } else if (in->dim == 1) {
        if ((rc = build_ktab_1d(in))) return rc;
    } else if (in->dim == 3) {
        // SplittingMethod2D::InitExpT with a third axis, one factor per axis:
        // exp(a fold(i)^2 DT_axis) with 1/L folded in (complex128) or as factor - 1
        const int L[3] = {in->nx, in->ny, in->nz};
        const double D[3] = {in->dx, in->dy, in->dz};
        const cd alpha = -I * in->dt / in->hbar;
        for (int ax = 0; ax < 3; ++ax) {
            const double dk = 2 * kPi / (D[ax] * L[ax]);
            const double DT = (dk * in->hbar) * (dk * in->hbar) / (2 * in->mass);
            for (int k = 0; k < ntab; ++k) {
                const cd f = alpha * tc[k] * DT;
                if ((rc = inst_alloc(in, (size_t)L[ax] * cs, &in->k3[ax][k]))) return rc;
                QSG_CUDA(qsg::launch_ktable1d(in->prec, in->k3[ax][k], L[ax], f.real(), f.imag(),
                                              1.0 / (double)L[ax], ctx->st));
            }
        }
    } else if (!in->blue2) {
        // SplittingMethod2D::InitExpT (src/SplittingMethod2D.cpp:56-79)
        const double dkx = 2 * kPi / (in->dx * in->nx), dky = 2 * kPi / (in->dy * in->ny);
        const double DTx = (dkx * in->hbar) * (dkx * in->hbar) / (2 * in->mass);
        const double DTy = (dky * in->hbar) * (dky * in->hbar) / (2 * in->mass);
        const cd alpha = -I * in->dt / in->hbar;
        for (int k = 0; k < ntab; ++k) {
            const cd a = in->order == 2 ? alpha : alpha * tc[k];
            if (in->prec == 0) {
                if ((rc = inst_alloc(in, in->n * cs, &in->ktab[k]))) return rc;
                QSG_CUDA(qsg::launch_ktable2d(in->ktab[k], in->nx, in->ny, a.real(), a.imag(), DTx, DTy,
                                              1.0 / ((double)in->nx * in->ny), ctx->st));
            } else {
                const cd fx = a * DTx, fy = a * DTy;
                if ((rc = inst_alloc(in, (size_t)in->nx * cs, &in->kx[k]))) return rc;
                if ((rc = inst_alloc(in, (size_t)in->ny * cs, &in->ky[k]))) return rc;
                QSG_CUDA(qsg::launch_ktable1d(1, in->kx[k], in->nx, fx.real(), fx.imag(), 1.0, ctx->st));
                QSG_CUDA(qsg::launch_ktable1d(1, in->ky[k], in->ny, fy.real(), fy.imag(), 1.0, ctx->st));
            }
        }
    }
    return QSG_OK;
}

int upload_psi(qsg_inst *in, const double *psi)
{
    qsg_ctx *ctx = in->ctx;
    in->wall_zero = in->wall_ext;
    // the source holds the user's sites; a Bluestein buffer is zero above them
    const size_t src = (in->bfs ? in->bfs_n : in->n) * 16;
    if (in->prec == 0) {
        if (in->bfs) QSG_CUDA(cudaMemsetAsync(in->psi, 0, in->n * 16, ctx->st));
        QSG_CUDA(cudaMemcpyAsync(in->psi, psi, src, cudaMemcpyDefault, ctx->st));  // host or device source
        return QSG_OK;
    }
    int rc = ensure_scratch(ctx, in->n * 16);
    if (rc) return rc;
    if (in->bfs) QSG_CUDA(cudaMemsetAsync(ctx->scratch, 0, in->n * 16, ctx->st));
    QSG_CUDA(cudaMemcpyAsync(ctx->scratch, psi, src, cudaMemcpyDefault, ctx->st));
    QSG_CUDA(qsg::launch_c128_to_c64(in->psi, ctx->scratch, in->n, ctx->st));
    return QSG_OK;
}

// drop the instance's uses of shared kinetic tables (a table is freed, in
// stream order, when its last user lets go)
void release_shared_k(qsg_inst *in)
{
    for (const auto &key : in->shared_k) {
        auto it = in->ctx->fs_ktabs.find(key);
        if (it == in->ctx->fs_ktabs.end() || --it->second.users > 0) continue;
        cudaFreeAsync(it->second.p, in->ctx->st);
        in->ctx->in_use -= it->second.bytes;
        in->ctx->fs_ktabs.erase(it);
    }
    in->shared_k.clear();
}

void free_inst(qsg_inst *in)
{
    if (!in) return;
    if (in->ring_host) cudaFreeHost(in->ring_host);
    for (cudaEvent_t &e : in->ring_ev)
        if (e) cudaEventDestroy(e);
    if (in->ctx) {
        // ordered after everything queued on the context stream (work on other
        // streams is joined into it before an instance is released)
        for (void *p : in->allocs) cudaFreeAsync(p, in->ctx->st);
        in->ctx->in_use -= in->bytes;
        release_shared_k(in);
    }
    delete in;
}

int common_create(qsg_inst *in, const double *psi0, const double *V)
{
    qsg_ctx *ctx = in->ctx;
    int rc;
    if ((rc = inst_alloc(in, in->n * csize(in->prec), &in->psi))) return rc;
    void *v = nullptr;
    if ((rc = inst_alloc(in, 256, &v))) return rc;
    in->err = static_cast<unsigned *>(v);
    QSG_CUDA(cudaMemsetAsync(in->err, 0, sizeof(unsigned), ctx->st));
    if ((rc = inst_alloc(in, in->n * 8, &v))) return rc;
    in->V = (double *)v;
    // (a wall extension's V comes extended to all n sites; a Bluestein buffer's is zero above n_out)
    if (in->bfs) QSG_CUDA(cudaMemsetAsync(in->V, 0, in->n * 8, ctx->st));
    QSG_CUDA(cudaMemcpyAsync(in->V, V, (in->bfs ? in->bfs_n : in->n) * 8, cudaMemcpyDefault,
                             ctx->st));  // host or device source
    if ((rc = upload_psi(in, psi0))) return rc;
    if ((rc = build_tables(in))) return rc;
    if (in->dim == 1) {
        // device descriptor (+ dv, + four-step norm partials) for the 1D kernels
        // (partials for every length that has four-step plans, so that a plan switch needs none)
        const int nparts = fs_parts_for(in);
        void *blk = nullptr;
        if ((rc = inst_alloc(in, sizeof(qsg::FsInst) + sizeof(double) * (2 + nparts), &blk))) return rc;
        in->desc = static_cast<qsg::FsInst *>(blk);
        in->d_dv = reinterpret_cast<double *>(in->desc + 1);
        in->snorm = in->d_dv + 1;
        in->parts_buf = nparts ? in->d_dv + 2 : nullptr;
        in->parts = in->fourstep ? in->parts_buf : nullptr;
        qsg::FsInst h{};
        h.psi = in->psi;
        h.vtab[0] = in->vtab[0];
        h.vtab[1] = in->vtab[1];
        h.ktab[0] = in->ktab[0];
        h.ktab[1] = in->ktab[1];
        h.partials = in->parts;
        QSG_CUDA(cudaMemcpyAsync(in->desc, &h, sizeof(h), cudaMemcpyHostToDevice, ctx->st));
        QSG_CUDA(cudaMemcpyAsync(in->d_dv, &in->dv, sizeof(double), cudaMemcpyHostToDevice, ctx->st));
        if (in->bfs)  // the Bluestein closing pass (descriptor 2) sums the norm partials
            QSG_CUDA(cudaMemcpyAsync(&in->bdesc[2].partials, &in->parts, sizeof(double *), cudaMemcpyHostToDevice,
                                     ctx->st));
        if (in->fourstep && in->fs_tma) {
            size_t mb = 0;
            in->fs_maps = fs_make_maps(ctx, &in, 1, &mb);
            if (in->fs_maps) {
                in->allocs.push_back(in->fs_maps);
                in->fs_maps_bytes = mb;
                in->bytes += mb;
                ctx->in_use += mb;
            }
        }
    } else if (in->dim == 2) {
        // column-pass norm partials: at most G * Ny / W = 2 Ny tiles (G <= 4, W >= 2)
        void *cp = nullptr;
        if ((rc = inst_alloc(in, sizeof(double) * 2 * (size_t)in->ny, &cp))) return rc;
        in->cparts = static_cast<double *>(cp);
        if (in->prec == 1 && !in->blue2) {
            if ((rc = inst_alloc(in, in->n * csize(in->prec), &in->work))) return rc;
            in->form = QSG_FORM_MOMENTUM;
        }
    } else {
        // 3D: line twiddles per axis and the kinetic-energy partials (2 per CTA)
        const int L[3] = {in->nx, in->ny, in->nz};
        for (int ax = 0; ax < 3; ++ax)
            if ((rc = get_twiddles(ctx, in->prec, L[ax], in->prec == 1 ? 16 : 8, &in->tw3[ax]))) return rc;
        const size_t ctas = std::max({(size_t)qsg::row3_ctas(in->prec, in->nz, (size_t)in->nx * in->ny),
                                      (size_t)qsg::col3_ctas(in->prec, in->ny, in->nz, in->nx),
                                      (size_t)qsg::col3_ctas(in->prec, in->nx, in->nz, in->ny)});
        void *kp = nullptr;
        if ((rc = inst_alloc(in, sizeof(double) * 2 * ctas, &kp))) return rc;
        in->kparts3 = static_cast<double *>(kp);
    }
    QSG_CUDA(cudaStreamSynchronize(ctx->st));
    return QSG_OK;
}


// --- plans -----------------------------------------------------------------

std::string plan_cache_path()
{
    if (const char *p = std::getenv("QSG_PLAN_CACHE")) return p;
    const char *home = std::getenv("HOME");
    return std::string(home ? home : ".") + "/.cache/qusim_gb300/plans.tsv";
}

// 2D lines: device \t prec \t nx \t ny \t g \t row_e \t row_nt \t col_e \t col_w \t ms_per_step [\t row_kind]
// 1D lines: device \t 1d \t prec \t n \t boundary \t kind \t n1 \t tma \t ms_per_step
// (later lines win)
void load_plans(qsg_ctx *ctx)
{
    if (ctx->plans_loaded) return;
    ctx->plans_loaded = true;
    std::ifstream f(plan_cache_path());
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream is(line);
        std::string dev;
        int prec, nx, ny;
        Plan2D p;
        double ms;
        if (!std::getline(is, dev, '\t')) continue;
        if (is.peek() == '1' && line.find("\t1d\t") != std::string::npos) {
            std::string tag;
            uint64_t n = 0;
            int boundary = 0;
            qsg_plan1d q{};
            if (!(is >> tag >> prec >> n >> boundary >> q.kind >> q.n1 >> q.tma >> ms) || tag != "1d") continue;
            if (dev == ctx->device_name && plan1d_valid(prec, n, boundary, q)) {
                const bool ext = boundary == QSG_INFINITE_WALL && !qsg::wall1d_supported(prec, n);
                ctx->plans1d[std::make_tuple(prec, ext ? 2 * n : n, ext ? 1 : 0)] = q;
            }
            continue;
        }
        if (!(is >> prec >> nx >> ny >> p.g >> p.row_e >> p.row_nt >> p.col_e >> p.col_w >> ms)) continue;
        int kind = 0;
        if (is >> kind) p.row_kind = kind;
        Geom2D g;
        if (dev == ctx->device_name && qsg::geom2d(prec, nx, ny, p, &g)) ctx->plans[std::make_tuple(prec, nx, ny)] = p;
    }
}

void save_plan(qsg_ctx *ctx, int prec, int nx, int ny, const Plan2D &p, double ms)
{
    const std::string path = plan_cache_path();
    const size_t slash = path.rfind('/');
    if (slash != std::string::npos) {
        // create the directory chain (best effort)
        std::string dir = path.substr(0, slash);
        for (size_t i = 1; i <= dir.size(); ++i)
            if (i == dir.size() || dir[i] == '/') {
                std::string d = dir.substr(0, i);
                mkdir(d.c_str(), 0755);
            }
    }
    std::ofstream f(path, std::ios::app);
    if (!f) return;
    f << ctx->device_name << '\t' << prec << '\t' << nx << '\t' << ny << '\t' << p.g << '\t' << p.row_e << '\t'
      << p.row_nt << '\t' << p.col_e << '\t' << p.col_w << '\t' << ms << '\t' << p.row_kind << '\n';
}

void save_plan_1d(qsg_ctx *ctx, int prec, uint64_t n, int boundary, const qsg_plan1d &p, double ms)
{
    const std::string path = plan_cache_path();
    const size_t slash = path.rfind('/');
    if (slash != std::string::npos) {
        std::string dir = path.substr(0, slash);
        for (size_t i = 1; i <= dir.size(); ++i)
            if (i == dir.size() || dir[i] == '/') mkdir(dir.substr(0, i).c_str(), 0755);
    }
    std::ofstream f(path, std::ios::app);
    if (!f) return;
    f << ctx->device_name << "\t1d\t" << prec << '\t' << n << '\t' << boundary << '\t' << p.kind << '\t' << p.n1
      << '\t' << p.tma << '\t' << ms << '\n';
}

// give back one of the instance's own allocations (stream-ordered)
void inst_release(qsg_inst *in, void *p, size_t bytes)
{
    auto it = std::find(in->allocs.begin(), in->allocs.end(), p);
    if (it == in->allocs.end()) return;
    in->allocs.erase(it);
    cudaFreeAsync(p, in->ctx->st);
    in->bytes -= bytes;
    in->ctx->in_use -= bytes;
}

// Switch a 1D instance to plan p between steps: geometry, twiddles, kinetic
// tables in the plan's layout, descriptor and tensor maps.  The state is in
// natural order between steps in every plan, so it is kept as it is.
int apply_plan_1d(qsg_inst *in, const qsg_plan1d &p)
{
    qsg_ctx *ctx = in->ctx;
    if (!plan1d_valid(in->prec, user_n(in), in->boundary, p))
        return fail(QSG_ERR_UNSUPPORTED, "1D plan (kind " + std::to_string(p.kind) + ", n1 " + std::to_string(p.n1) +
                                             ", tma " + std::to_string(p.tma) + ") not available for this instance");
    if (same_plan1d(p, in->plan1d)) return QSG_OK;
    const bool fs = p.kind == 1;
    qsg::FsGeom g{};
    if (fs && !qsg::fs_geom(in->prec, in->n, &g, p.n1)) return fail(QSG_ERR_UNSUPPORTED, "four-step split not built");
    int rc;
    const void *tfc = nullptr, *tfr = nullptr, *tn = nullptr, *tw = nullptr;
    if (fs) {
        if ((rc = get_twiddles(ctx, in->prec, g.n2, g.col_e, &tfc))) return rc;
        if ((rc = get_twiddles(ctx, in->prec, g.n1, g.row_e, &tfr))) return rc;
        if ((rc = get_fs_grid(ctx, in->prec, g.n1, g.n2, &tn))) return rc;
        if ((rc = get_twiddles(ctx, in->prec, g.n1, qsg::elems_per_thread(in->prec), &tw))) return rc;
    } else {
        if ((rc = get_twiddles(ctx, in->prec, (int)in->n, qsg::elems_per_thread(in->prec), &tw))) return rc;
    }
    // launches already queued read the old tables
    QSG_CUDA(cudaStreamSynchronize(in->st));
    QSG_CUDA(cudaStreamSynchronize(ctx->st));
    // The new kinetic tables and descriptor are made first; the old tables are
    // released only once the descriptor points at the new ones, so a failure
    // on the way puts the old plan back as it was.
    struct Saved {
        bool fourstep, fs_tma;
        qsg::FsGeom fsg;
        const void *tfc, *tfr, *tn, *tw;
        qsg_plan1d plan;
        double *parts;
        void *ktab[2];
        std::vector<std::tuple<int, int, int, double, double>> keys;
    } old{in->fourstep, in->fs_tma, in->fsg, in->tw_fs_col, in->tw_fs_row, in->tw_n, in->tw, in->plan1d, in->parts,
          {in->ktab[0], in->ktab[1]}, in->shared_k};
    auto restore = [&](int code) {
        release_shared_k(in);  // the new plan's tables, if any were made
        in->fourstep = old.fourstep;
        in->fs_tma = old.fs_tma;
        in->fsg = old.fsg;
        in->tw_fs_col = old.tfc;
        in->tw_fs_row = old.tfr;
        in->tw_n = old.tn;
        in->tw = old.tw;
        in->plan1d = old.plan;
        in->parts = old.parts;
        in->ktab[0] = old.ktab[0];
        in->ktab[1] = old.ktab[1];
        in->shared_k = old.keys;
        return code;
    };
    in->shared_k.clear();
    in->ktab[0] = in->ktab[1] = nullptr;
    in->fourstep = fs;
    in->fsg = g;
    in->tw_fs_col = tfc;
    in->tw_fs_row = tfr;
    in->tw_n = tn;
    in->tw = tw;
    in->fs_tma = p.tma != 0;
    in->plan1d = p;
    in->parts = fs ? in->parts_buf : nullptr;
    if ((rc = build_ktab_1d(in))) return restore(rc);
    if (std::getenv("QSG_FAIL_PLAN_SWITCH"))  // host-side failure injection for the tests of this path
        return restore(fail(QSG_ERR_CUDA, "injected plan-switch failure (QSG_FAIL_PLAN_SWITCH)"));
    qsg::FsInst h{};
    h.psi = in->psi;
    h.vtab[0] = in->vtab[0];
    h.vtab[1] = in->vtab[1];
    h.ktab[0] = in->ktab[0];
    h.ktab[1] = in->ktab[1];
    h.partials = in->parts;
    cudaError_t e = cudaMemcpyAsync(in->desc, &h, sizeof(h), cudaMemcpyHostToDevice, ctx->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return restore(fail(QSG_ERR_CUDA, std::string("1D plan switch: ") + cudaGetErrorString(e)));
    }
    // committed: the old tables go, the tensor maps follow the split
    {
        std::vector<std::tuple<int, int, int, double, double>> now = in->shared_k;
        in->shared_k = old.keys;
        release_shared_k(in);
        in->shared_k = now;
    }
    in->snorm_valid = false;
    if (in->fs_maps) {
        inst_release(in, in->fs_maps, in->fs_maps_bytes);
        in->fs_maps = nullptr;
        in->fs_maps_bytes = 0;
    }
    if (fs && in->fs_tma) {
        size_t mb = 0;
        in->fs_maps = fs_make_maps(ctx, &in, 1, &mb);  // none: the column pass loads with instructions
        if (in->fs_maps) {
            in->allocs.push_back(in->fs_maps);
            in->fs_maps_bytes = mb;
            in->bytes += mb;
            ctx->in_use += mb;
        }
    }
    QSG_CUDA(cudaStreamSynchronize(ctx->st));
    return QSG_OK;
}

// point the instance at a plan: geometry + the twiddle tables it needs
int apply_plan(qsg_inst *in, const Plan2D &p)
{
    Geom2D g;
    if (!qsg::geom2d(in->prec, in->nx, in->ny, p, &g))
        return fail(QSG_ERR_UNSUPPORTED, "plan not available for this grid");
    const void *tr, *tc, *tn, *tk;
    int rc;
    if ((rc = get_twiddles(in->ctx, in->prec, in->ny, p.row_e, &tr))) return rc;
    if ((rc = get_twiddles(in->ctx, in->prec, g.m, p.col_e, &tc))) return rc;
    if ((rc = get_circle(in->ctx, in->prec, in->nx, &tn))) return rc;
    if ((rc = get_twiddles(in->ctx, in->prec, g.m, g.kin_e, &tk))) return rc;
    if (in->prec == 1) {
        const void *pr, *pc, *pn;
        if ((rc = get_twiddles(in->ctx, 2, in->ny, p.row_e, &pr))) return rc;
        if ((rc = get_twiddles(in->ctx, 2, g.m, p.col_e, &pc))) return rc;
        if ((rc = get_circle(in->ctx, 2, in->nx, &pn))) return rc;
        in->tw_row_p = pr;
        in->tw_col_p = pc;
        in->tw_nx_p = pn;
    }
    in->plan = p;
    in->geom = g;
    in->tw_row = tr;
    in->tw_col = tc;
    in->tw_nx = tn;
    in->tw_kin = tk;
    return QSG_OK;
}

bool finite_pos(double v) { return std::isfinite(v) && v > 0; }

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================

extern "C" {

const char *qsg_version(void) { return "qsg 0.1 (sm_103a)"; }

const char *qsg_last_error(void) { return g_last_error.c_str(); }

int qsg_init(int device_ordinal, size_t hbm_budget_bytes, qsg_ctx **out)
{
    if (!out) return fail(QSG_ERR_ARG, "qsg_init: out is null");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess) return fail(QSG_ERR_CUDA, std::string("cudaGetDeviceCount: ") + cudaGetErrorString(e));
    if (device_ordinal < 0 || device_ordinal >= ndev)
        return fail(QSG_ERR_ARG, "qsg_init: no CUDA device " + std::to_string(device_ordinal));
    QSG_CUDA(cudaSetDevice(device_ordinal));
    cudaDeviceProp prop;
    QSG_CUDA(cudaGetDeviceProperties(&prop, device_ordinal));
    if (prop.major * 10 + prop.minor < 100)
        return fail(QSG_ERR_UNSUPPORTED, std::string("qsg_init: device ") + prop.name +
                                             " is not a Blackwell (sm_10x) GPU");
    qsg_ctx *ctx = new qsg_ctx();
    ctx->dev = device_ordinal;
    ctx->device_name = prop.name;
    if (const char *g = std::getenv("QSG_BATCH_GRAPHS")) ctx->graphs = std::atoi(g) != 0;
    if (const char *g = std::getenv("QSG_COL_TMA")) ctx->col_tma = std::atoi(g) != 0;
    if (const char *g = std::getenv("QSG_FS_TMA")) ctx->fs_tma = std::atoi(g) != 0;
    if (const char *g = std::getenv("QSG_BATCH_QUEUE")) ctx->batch_queue = std::atoi(g) != 0;
    ctx->budget = hbm_budget_bytes;
    e = cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete ctx;
        return fail(QSG_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    }
    {
        // keep freed blocks in the device pool for reuse instead of returning them
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device_ordinal) == cudaSuccess) {
            uint64_t thr = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
    }
    ctx->max_partials = 65536;
    void *p = nullptr;
    int rc = dev_alloc(ctx, sizeof(double) * 2 * ctx->max_partials, &p, nullptr, false);
    if (rc) {
        qsg_ctx_destroy(ctx);
        return rc;
    }
    ctx->partials = (double *)p;
    if ((rc = dev_alloc(ctx, sizeof(double) * 8, &p, nullptr, false))) {
        qsg_ctx_destroy(ctx);
        return rc;
    }
    ctx->sums = (double *)p;
    e = cudaMallocHost(&p, sizeof(double) * 8);
    if (e != cudaSuccess) {
        qsg_ctx_destroy(ctx);
        return fail(QSG_ERR_CUDA, std::string("cudaMallocHost: ") + cudaGetErrorString(e));
    }
    ctx->host_sums = (double *)p;
    *out = ctx;
    return QSG_OK;
}

void qsg_ctx_destroy(qsg_ctx *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->dev);
    if (ctx->st) cudaStreamSynchronize(ctx->st);
    for (auto &kv : ctx->tw_cache) cudaFreeAsync(kv.second, ctx->st);
    for (auto &kv : ctx->circle_cache) cudaFreeAsync(kv.second, ctx->st);
    if (ctx->scratch) cudaFreeAsync(ctx->scratch, ctx->st);
    if (ctx->partials) cudaFreeAsync(ctx->partials, ctx->st);
    if (ctx->sums) cudaFreeAsync(ctx->sums, ctx->st);
    if (ctx->st) cudaStreamSynchronize(ctx->st);
    if (ctx->host_sums) cudaFreeHost(ctx->host_sums);
    for (auto &p : ctx->prof_pending) {
        cudaEventDestroy(std::get<1>(p));
        cudaEventDestroy(std::get<2>(p));
    }
    for (auto e : ctx->event_pool) cudaEventDestroy(e);
    if (ctx->st) cudaStreamDestroy(ctx->st);
    delete ctx;
}

void *qsg_ctx_stream(qsg_ctx *ctx) { return ctx ? (void *)ctx->st : nullptr; }

size_t qsg_ctx_bytes_in_use(qsg_ctx *ctx) { return ctx ? ctx->in_use : 0; }

static int create_1d_locked(qsg_ctx *ctx, uint64_t n, double dx, double mass, double hbar, double dt_re,
                            double dt_im, int order, int precision, int boundary, const double *psi0,
                            const double *V, qsg_inst **out);

namespace {

// The 2n-site odd extension of a wall state (host or device source, n
// complex): ext_j = psi_j (j < n), 0 at j = n, ext_{2n-j} = -psi_j (0 < j < n).
// Site 0 keeps psi_0 as given: the reference discards it (and site n) only when
// a kinetic factor is applied; step1d zeroes it before the first step.
int wall_odd_extension(const double *psi, uint64_t n, std::vector<double> &ext)
{
    std::vector<double> h(2 * n);
    QSG_CUDA(cudaMemcpy(h.data(), psi, sizeof(double) * 2 * n, cudaMemcpyDefault));
    ext.assign(4 * n, 0.0);
    std::memcpy(ext.data(), h.data(), sizeof(double) * 2 * n);
    for (uint64_t j = 1; j < n; ++j) {
        ext[2 * (2 * n - j)] = -h[2 * j];
        ext[2 * (2 * n - j) + 1] = -h[2 * j + 1];
    }
    return QSG_OK;
}

// V on the extension: even (V_{2n-j} = V_j), 0 at j = n (where the state is 0)
int wall_even_extension(const double *V, uint64_t n, std::vector<double> &ext)
{
    std::vector<double> h(n);
    QSG_CUDA(cudaMemcpy(h.data(), V, sizeof(double) * n, cudaMemcpyDefault));
    ext.assign(2 * n, 0.0);
    std::memcpy(ext.data(), h.data(), sizeof(double) * n);
    for (uint64_t j = 1; j < n; ++j) ext[2 * n - j] = h[j];
    return QSG_OK;
}

}  // namespace

int qsg_create_1d(qsg_ctx *ctx, uint64_t n, double dx, double mass, double hbar, double dt_re,
                  double dt_im, int order, int precision, int boundary, const double *psi0,
                  const double *V, qsg_inst **out)
{
    if (!ctx) return fail(QSG_ERR_ARG, "qsg_create_1d: null argument");
    std::lock_guard<std::mutex> lk(ctx->mu);
    return create_1d_locked(ctx, n, dx, mass, hbar, dt_re, dt_im, order, precision, boundary, psi0, V, out);
}

static int create_1d_locked(qsg_ctx *ctx, uint64_t n, double dx, double mass, double hbar, double dt_re,
                            double dt_im, int order, int precision, int boundary, const double *psi0,
                            const double *V, qsg_inst **out)
{
    if (!ctx || !out || !psi0 || !V) return fail(QSG_ERR_ARG, "qsg_create_1d: null argument");
    *out = nullptr;
    if (order != 2 && order != 4) return fail(QSG_ERR_ARG, "qsg_create_1d: order must be 2 or 4");
    if (precision != QSG_FP64 && precision != QSG_MIXED)
        return fail(QSG_ERR_ARG, "qsg_create_1d: precision must be QSG_FP64 or QSG_MIXED");
    if (!finite_pos(dx) || !finite_pos(mass) || !finite_pos(hbar) || !std::isfinite(dt_re) ||
        !std::isfinite(dt_im))
        return fail(QSG_ERR_ARG, "qsg_create_1d: dx, mass, hbar must be finite and > 0, dt finite");
    if (boundary != QSG_PERIOD && boundary != QSG_INFINITE_WALL)
        return fail(QSG_ERR_ARG, "qsg_create_1d: unknown boundary");
    const bool wall = boundary == QSG_INFINITE_WALL;
    const bool pow2 = n >= 1 && (n & (n - 1)) == 0;
    qsg::FsGeom fsg{};
    // lengths that are not powers of two (and powers of two below 64): Bluestein
    // transforms of n sites (a wall: of its 2n odd extension), in one kernel where
    // M >= 2 len - 1 fits one CTA, else two convolutions on the four-step passes
    // over a buffer of bfs_m >= 2 len - 1 sites
    const bool any_len = !pow2 || n < 64;
    const uint64_t blue_len = wall ? 2 * n : n;
    const int one_cta_m = any_len && n >= 2 ? qsg::blue_m_for(precision, blue_len) : 0;
    const uint64_t bfs_m = any_len && !one_cta_m ? bfs_len_m(precision, blue_len, &fsg) : 0;
    const bool wall_blue = wall && one_cta_m > 0;
    const std::string wall_limits = " (supported: any n from 2 to 2097152, and powers of two up to 4194304)";
    if (wall && any_len && !one_cta_m && !bfs_m)
        return fail(QSG_ERR_UNSUPPORTED, "qsg_create_1d: InfiniteWall n=" + std::to_string(n) + wall_limits);
    // walls above one CTA: a four-step periodic instance of the 2n odd extension
    const bool wall_ext = wall && (any_len || !qsg::wall1d_supported(precision, n));
    const int blue_m = one_cta_m;
    const bool resident = wall ? (wall_blue || !wall_ext) : (blue_m > 0 || qsg::evolve1d_supported(precision, n));
    if (wall_ext && !any_len && (n < 64 || !qsg::fs_geom(precision, 2 * n, &fsg)))
        return fail(QSG_ERR_UNSUPPORTED, "qsg_create_1d: InfiniteWall n=" + std::to_string(n) + wall_limits);
    if (!wall && any_len && !blue_m && !bfs_m)
        return fail(QSG_ERR_UNSUPPORTED, "qsg_create_1d: n=" + std::to_string(n) +
                                             " (lengths that are not powers of two: 2 .. 4194304)");
    if (!wall && pow2 && !resident && !qsg::fs_geom(precision, n, &fsg))
        return fail(QSG_ERR_UNSUPPORTED, "qsg_create_1d: n=" + std::to_string(n) +
                                             " (supported: powers of two, 64 .. 8388608)");
    // the plan: the one tuned for this shape (in this context or the plan cache),
    // else the default (one CTA where it fits, else four-step, default split)
    qsg_plan1d plan{resident ? 0 : 1, resident ? 0 : fsg.n1, 0, 0};
    if (!resident && !wall_ext && !bfs_m && ctx->fs_tma && qsg::fs_tma_supported(precision, fsg.n2)) plan.tma = 1;
    if (!blue_m && !bfs_m && !(wall && !wall_ext)) {
        load_plans(ctx);
        auto it = ctx->plans1d.find(std::make_tuple(precision, wall_ext ? 2 * n : n, wall_ext ? 1 : 0));
        if (it != ctx->plans1d.end() && plan1d_valid(precision, n, boundary, it->second)) plan = it->second;
    }
    if (plan.kind == 1 && !qsg::fs_geom(precision, bfs_m ? bfs_m : (wall_ext ? 2 * n : n), &fsg, plan.n1))
        return fail(QSG_ERR_STATE, "qsg_create_1d: plan cache entry does not fit n=" + std::to_string(n));
    QSG_CUDA(cudaSetDevice(ctx->dev));
    qsg_inst *in = new qsg_inst();
    in->ctx = ctx;
    in->dim = 1;
    in->n = bfs_m ? bfs_m : (wall_ext ? 2 * n : n);
    in->n_out = n;
    in->bfs = bfs_m > 0;
    in->bfs_n = bfs_m ? blue_len : 0;
    in->wall_ext = wall_ext;
    in->nx = (int)n;
    in->dx = dx;
    in->dv = dx;
    in->mass = mass;
    in->hbar = hbar;
    in->dt = cd(dt_re, dt_im);
    in->order = order;
    in->prec = precision;
    in->boundary = boundary;
    in->st = ctx->st;
    in->fourstep = plan.kind == 1;
    in->fsg = in->fourstep ? fsg : qsg::FsGeom{};
    in->plan1d = plan;
    in->fs_tma = plan.tma != 0;
    in->blue = blue_m > 0;
    in->blue_m = blue_m;
    int rc = QSG_OK;
    if (in->blue) {
        rc = get_twiddles(ctx, precision, blue_m, qsg::blue_elems(precision), &in->tw);
    } else if (!in->fourstep) {
        // the wall transforms run on the 2n odd extension
        rc = get_twiddles(ctx, precision, (int)(wall ? 2 * n : n), qsg::elems_per_thread(precision), &in->tw);
    } else {
        rc = get_twiddles(ctx, precision, fsg.n2, fsg.col_e, &in->tw_fs_col);
        if (!rc) rc = get_twiddles(ctx, precision, fsg.n1, fsg.row_e, &in->tw_fs_row);
        if (!rc) rc = get_fs_grid(ctx, precision, fsg.n1, fsg.n2, &in->tw_n);
        if (!rc) rc = get_twiddles(ctx, precision, (int)fsg.n1, qsg::elems_per_thread(precision), &in->tw);
    }
    if (!rc && wall_ext) {
        std::vector<double> pe, ve;
        rc = wall_odd_extension(psi0, n, pe);
        if (!rc) rc = wall_even_extension(V, n, ve);
        if (!rc) rc = common_create(in, pe.data(), ve.data());
    } else if (!rc) {
        rc = common_create(in, psi0, V);
    }
    if (rc) {
        std::string msg = g_last_error;
        free_inst(in);
        return fail(rc, msg);
    }
    *out = in;
    return QSG_OK;
}

}  // extern "C"

namespace {

int check_spec(const qsg_spec *sp, const char *who)
{
    if (!sp) return fail(QSG_ERR_ARG, std::string(who) + ": null spec");
    if (!(sp->s > 0) || !std::isfinite(sp->s) || sp->nbumps < 0 || sp->nbumps > QSG_SPEC_MAX_BUMPS)
        return fail(QSG_ERR_ARG, std::string(who) + ": spec needs s > 0 and 0 <= nbumps <= " +
                                     std::to_string(QSG_SPEC_MAX_BUMPS));
    for (int b = 0; b < sp->nbumps; ++b)
        if (!(sp->bumps[b][3] > 0)) return fail(QSG_ERR_ARG, std::string(who) + ": bump widths must be > 0");
    return QSG_OK;
}

// psi0 (complex128, normalised if asked) and V sampled from the spec into one
// temporary device buffer of 24 bytes per site on the context stream; the
// buffer counts against the budget until the caller releases it
int sample_spec(qsg_ctx *ctx, int dim, uint64_t nx, uint64_t ny, double dx, double dy, const qsg_spec &sp,
                void **buf)
{
    const size_t n = (size_t)nx * ny;
    const size_t bytes = n * 24;
    if (ctx->budget && ctx->in_use + bytes > ctx->budget)
        return fail(QSG_ERR_BUDGET, "spec sampling needs " + std::to_string(bytes) + " bytes of the HBM budget");
    QSG_CUDA(cudaSetDevice(ctx->dev));
    QSG_CUDA(cudaMallocAsync(buf, bytes, ctx->st));
    ctx->in_use += bytes;
    qsg::SpecArgs a{};
    a.x0 = sp.x0;
    a.y0 = sp.y0;
    a.dx = dx;
    a.dy = dy;
    a.kx = sp.kx;
    a.ky = sp.ky;
    a.cx = sp.cx;
    a.cy = sp.cy;
    a.s = sp.s;
    a.v0 = sp.v0;
    a.dim = dim;
    a.nbumps = sp.nbumps;
    for (int b = 0; b < sp.nbumps; ++b)
        for (int k = 0; k < 4; ++k) a.bumps[b][k] = sp.bumps[b][k];
    double *psi = static_cast<double *>(*buf);
    cudaError_t e = qsg::launch_sample_spec(a, (int)nx, (int)ny, psi, psi + 2 * n, ctx->st);
    if (e == cudaSuccess && sp.normalize) {
        // psi *= 1 / sqrt(sum |psi|^2 dv), the reference's host normalisation
        int np = 0;
        e = qsg::launch_reduce(0, psi, nullptr, 0, n, 0, ctx->partials, ctx->max_partials, &np, ctx->st);
        if (e == cudaSuccess) e = qsg::launch_finalize(ctx->partials, np, 1, ctx->sums, ctx->st);
        if (e == cudaSuccess) e = qsg::launch_renorm(0, psi, n, ctx->sums, dim == 2 ? dx * dy : dx, ctx->st);
    }
    if (e != cudaSuccess) {
        cudaFreeAsync(*buf, ctx->st);
        ctx->in_use -= bytes;
        *buf = nullptr;
        return fail(QSG_ERR_CUDA, std::string("spec sampling: ") + cudaGetErrorString(e));
    }
    return QSG_OK;
}

void release_spec(qsg_ctx *ctx, void *buf, size_t n)
{
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaFreeAsync(buf, ctx->st);
    ctx->in_use -= n * 24;
}

}  // namespace

extern "C" {

// psi0 and V sampled from expressions into a temporary device buffer of 24
// bytes per site (counted against the budget while it lives), psi0 normalised
// if asked; the buffer then feeds the array creation path
static int sample_expr_buf(qsg_ctx *ctx, int dim, uint64_t nx, uint64_t ny, double x0, double y0, double dx, double dy,
                           const char *psi_expr, const char *v_expr, int normalize, void **buf)
{
    const size_t n = (size_t)nx * ny;
    const size_t bytes = n * 24;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (ctx->budget && ctx->in_use + bytes > ctx->budget)
        return fail(QSG_ERR_BUDGET, "expression sampling needs " + std::to_string(bytes) + " bytes of the HBM budget");
    QSG_CUDA(cudaSetDevice(ctx->dev));
    QSG_CUDA(cudaMallocAsync(buf, bytes, ctx->st));
    ctx->in_use += bytes;
    double *psi = static_cast<double *>(*buf);
    std::string err;
    int rc = qsg::sample_expr(dim, psi_expr, v_expr, (int)nx, (int)ny, x0, y0, dx, dy, psi, psi + 2 * n, ctx->st, err);
    cudaError_t e = cudaSuccess;
    if (!rc && normalize) {
        // psi *= 1 / sqrt(sum |psi|^2 dv), the reference's force_normalization (src/EvolverImpl1D.cpp:64-69)
        int np = 0;
        e = qsg::launch_reduce(0, psi, nullptr, 0, n, 0, ctx->partials, ctx->max_partials, &np, ctx->st);
        if (e == cudaSuccess) e = qsg::launch_finalize(ctx->partials, np, 1, ctx->sums, ctx->st);
        if (e == cudaSuccess) e = qsg::launch_renorm(0, psi, n, ctx->sums, dim == 2 ? dx * dy : dx, ctx->st);
        if (e != cudaSuccess) {
            rc = QSG_ERR_CUDA;
            err = std::string("expression sampling: ") + cudaGetErrorString(e);
        }
    }
    if (rc) {
        cudaFreeAsync(*buf, ctx->st);
        ctx->in_use -= bytes;
        *buf = nullptr;
        return fail(rc, err);
    }
    return QSG_OK;
}

int qsg_create_1d_expr(qsg_ctx *ctx, uint64_t n, double x0, double dx, double mass, double hbar, double dt_re,
                       double dt_im, int order, int precision, int boundary, const char *psi_expr, const char *v_expr,
                       int normalize, qsg_inst **out)
{
    if (!ctx || !out || !psi_expr || !v_expr) return fail(QSG_ERR_ARG, "qsg_create_1d_expr: null argument");
    if (n == 0 || n > 8388608 || !(dx > 0) || !std::isfinite(x0))
        return fail(QSG_ERR_ARG, "qsg_create_1d_expr: bad n, x0 or dx");
    void *buf = nullptr;
    int rc = sample_expr_buf(ctx, 1, n, 1, x0, 0.0, dx, 0.0, psi_expr, v_expr, normalize, &buf);
    if (rc) return rc;
    const double *psi = static_cast<const double *>(buf);
    rc = qsg_create_1d(ctx, n, dx, mass, hbar, dt_re, dt_im, order, precision, boundary, psi, psi + 2 * n, out);
    const std::string msg = rc ? std::string(g_last_error) : std::string();
    release_spec(ctx, buf, n);
    return rc ? fail(rc, msg) : QSG_OK;
}

int qsg_create_2d_expr(qsg_ctx *ctx, uint64_t nx, uint64_t ny, double x0, double y0, double dx, double dy,
                       double mass, double hbar, double dt_re, double dt_im, int order, int precision,
                       const char *psi_expr, const char *v_expr, int normalize, qsg_inst **out)
{
    if (!ctx || !out || !psi_expr || !v_expr) return fail(QSG_ERR_ARG, "qsg_create_2d_expr: null argument");
    if (nx == 0 || ny == 0 || nx * ny > ((uint64_t)1 << 26) || !(dx > 0) || !(dy > 0) || !std::isfinite(x0) ||
        !std::isfinite(y0))
        return fail(QSG_ERR_ARG, "qsg_create_2d_expr: bad sizes, origin or spacing");
    void *buf = nullptr;
    int rc = sample_expr_buf(ctx, 2, nx, ny, x0, y0, dx, dy, psi_expr, v_expr, normalize, &buf);
    if (rc) return rc;
    const double *psi = static_cast<const double *>(buf);
    const size_t n = (size_t)nx * ny;
    rc = qsg_create_2d(ctx, nx, ny, dx, dy, mass, hbar, dt_re, dt_im, order, precision, psi, psi + 2 * n, out);
    const std::string msg = rc ? std::string(g_last_error) : std::string();
    release_spec(ctx, buf, n);
    return rc ? fail(rc, msg) : QSG_OK;
}

int qsg_create_1d_spec(qsg_ctx *ctx, uint64_t n, double dx, double mass, double hbar, double dt_re,
                       double dt_im, int order, int precision, int boundary, const qsg_spec *spec,
                       qsg_inst **out)
{
    if (!ctx || !out) return fail(QSG_ERR_ARG, "qsg_create_1d_spec: null argument");
    int rc = check_spec(spec, "qsg_create_1d_spec");
    if (rc) return rc;
    if (n == 0 || n > 8388608 || !(dx > 0)) return fail(QSG_ERR_ARG, "qsg_create_1d_spec: bad n or dx");
    void *buf = nullptr;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        if ((rc = sample_spec(ctx, 1, n, 1, dx, 0.0, *spec, &buf))) return rc;
    }
    const double *psi = static_cast<const double *>(buf);
    rc = qsg_create_1d(ctx, n, dx, mass, hbar, dt_re, dt_im, order, precision, boundary, psi, psi + 2 * n, out);
    const std::string msg = rc ? std::string(g_last_error) : std::string();
    release_spec(ctx, buf, n);
    return rc ? fail(rc, msg) : QSG_OK;
}

int qsg_create_2d_spec(qsg_ctx *ctx, uint64_t nx, uint64_t ny, double dx, double dy, double mass,
                       double hbar, double dt_re, double dt_im, int order, int precision,
                       const qsg_spec *spec, qsg_inst **out)
{
    if (!ctx || !out) return fail(QSG_ERR_ARG, "qsg_create_2d_spec: null argument");
    int rc = check_spec(spec, "qsg_create_2d_spec");
    if (rc) return rc;
    if (nx == 0 || ny == 0 || nx > 8192 || ny > 8192 || !(dx > 0) || !(dy > 0))
        return fail(QSG_ERR_ARG, "qsg_create_2d_spec: bad sizes or spacing");
    void *buf = nullptr;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        if ((rc = sample_spec(ctx, 2, nx, ny, dx, dy, *spec, &buf))) return rc;
    }
    const size_t n = (size_t)nx * ny;
    const double *psi = static_cast<const double *>(buf);
    rc = qsg_create_2d(ctx, nx, ny, dx, dy, mass, hbar, dt_re, dt_im, order, precision, psi, psi + 2 * n, out);
    const std::string msg = rc ? std::string(g_last_error) : std::string();
    release_spec(ctx, buf, n);
    return rc ? fail(rc, msg) : QSG_OK;
}

int qsg_create_2d(qsg_ctx *ctx, uint64_t nx, uint64_t ny, double dx, double dy, double mass,
                  double hbar, double dt_re, double dt_im, int order, int precision,
                  const double *psi0, const double *V, qsg_inst **out)
{
    if (!ctx || !out || !psi0 || !V) return fail(QSG_ERR_ARG, "qsg_create_2d: null argument");
    *out = nullptr;
    if (order != 2 && order != 4) return fail(QSG_ERR_ARG, "qsg_create_2d: order must be 2 or 4");
    if (precision != QSG_FP64 && precision != QSG_MIXED)
        return fail(QSG_ERR_ARG, "qsg_create_2d: precision must be QSG_FP64 or QSG_MIXED");
    if (!finite_pos(dx) || !finite_pos(dy) || !finite_pos(mass) || !finite_pos(hbar) ||
        !std::isfinite(dt_re) || !std::isfinite(dt_im))
        return fail(QSG_ERR_ARG, "qsg_create_2d: dx, dy, mass, hbar must be finite and > 0, dt finite");
    Plan2D plan{};
    // grids without a power-of-two plan: Bluestein passes on sides up to 4096
    const bool pow2_plan = nx <= 8192 && ny <= 8192 && qsg::default_plan(precision, (int)nx, (int)ny, &plan);
    const int bmx = pow2_plan ? 0 : qsg::blue_m_for(precision, nx), bmy = pow2_plan ? 0 : qsg::blue_m_for(precision, ny);
    if (!pow2_plan && (!bmx || !bmy))
        return fail(QSG_ERR_UNSUPPORTED, "qsg_create_2d: grid " + std::to_string(nx) + "x" + std::to_string(ny) +
                                             " (supported: sides 2 .. 4096, and powers of two 128 .. 4096 with one side up to 8192)");
    std::lock_guard<std::mutex> lk(ctx->mu);
    QSG_CUDA(cudaSetDevice(ctx->dev));
    qsg_inst *in = new qsg_inst();
    in->ctx = ctx;
    in->dim = 2;
    in->nx = (int)nx;
    in->ny = (int)ny;
    in->n = nx * ny;
    in->dx = dx;
    in->dy = dy;
    in->dv = dx * dy;
    in->mass = mass;
    in->hbar = hbar;
    in->dt = cd(dt_re, dt_im);
    in->order = order;
    in->prec = precision;
    in->st = ctx->st;
    int rc = QSG_OK;
    if (pow2_plan) {
        load_plans(ctx);
        auto it = ctx->plans.find(std::make_tuple(precision, (int)nx, (int)ny));
        if (it != ctx->plans.end()) plan = it->second;
        rc = apply_plan(in, plan);
    } else {
        in->blue2 = true;
        in->bmx = bmx;
        in->bmy = bmy;
        rc = get_twiddles(ctx, precision, bmx, qsg::blue_elems(precision), &in->btwx);
        if (!rc) rc = get_twiddles(ctx, precision, bmy, qsg::blue_elems(precision), &in->btwy);
    }
    if (!rc) rc = common_create(in, psi0, V);
    if (rc) {
        std::string msg = g_last_error;
        free_inst(in);
        return fail(rc, msg);
    }
    *out = in;
    return QSG_OK;
}

int qsg_create_3d(qsg_ctx *ctx, uint64_t nx, uint64_t ny, uint64_t nz, double dx, double dy, double dz,
                  double mass, double hbar, double dt_re, double dt_im, int order, int precision,
                  const double *psi0, const double *V, qsg_inst **out)
{
    if (!ctx || !out || !psi0 || !V) return fail(QSG_ERR_ARG, "qsg_create_3d: null argument");
    *out = nullptr;
    if (order != 2 && order != 4) return fail(QSG_ERR_ARG, "qsg_create_3d: order must be 2 or 4");
    if (precision != QSG_FP64 && precision != QSG_MIXED)
        return fail(QSG_ERR_ARG, "qsg_create_3d: precision must be QSG_FP64 or QSG_MIXED");
    if (!finite_pos(dx) || !finite_pos(dy) || !finite_pos(dz) || !finite_pos(mass) || !finite_pos(hbar) ||
        !std::isfinite(dt_re) || !std::isfinite(dt_im))
        return fail(QSG_ERR_ARG, "qsg_create_3d: dx, dy, dz, mass, hbar must be finite and > 0, dt finite");
    if (!qsg::evolve3d_supported(precision, nx, ny, nz))
        return fail(QSG_ERR_UNSUPPORTED, "qsg_create_3d: grid " + std::to_string(nx) + "x" + std::to_string(ny) +
                                             "x" + std::to_string(nz) +
                                             " (supported: powers of two, 16 .. 1024 per side, nz a multiple of "
                                             "the strided passes' tile width, at most 2^30 sites)");
    std::lock_guard<std::mutex> lk(ctx->mu);
    QSG_CUDA(cudaSetDevice(ctx->dev));
    qsg_inst *in = new qsg_inst();
    in->ctx = ctx;
    in->dim = 3;
    in->nx = (int)nx;
    in->ny = (int)ny;
    in->nz = (int)nz;
    in->n = nx * ny * nz;
    in->dx = dx;
    in->dy = dy;
    in->dz = dz;
    in->dv = dx * dy * dz;
    in->mass = mass;
    in->hbar = hbar;
    in->dt = cd(dt_re, dt_im);
    in->order = order;
    in->prec = precision;
    in->st = ctx->st;
    int rc = common_create(in, psi0, V);
    if (rc) {
        std::string msg = g_last_error;
        free_inst(in);
        return fail(rc, msg);
    }
    *out = in;
    return QSG_OK;
}

int qsg_step(qsg_inst *in, uint64_t nsteps, int renormalize)
{
    if (!in) return fail(QSG_ERR_ARG, "qsg_step: null instance");
    if (nsteps == 0 && !renormalize) return QSG_OK;
    std::lock_guard<std::mutex> lk(in->ctx->mu);
    if (int rc = lost_state(in, "qsg_step")) return rc;
    QSG_CUDA(cudaSetDevice(in->ctx->dev));
    int rc;
    if (nsteps == 0) {
        // renormalise only
        in->snorm_valid = false;
        double s = 0;
        if ((rc = reduce(in, 0, user_n(in), 0, &s))) return rc;
        QSG_CUDA(qsg::launch_renorm(in->prec, in->psi, in->n, in->ctx->sums, in->dv, in->ctx->st));
        return QSG_OK;
    }
    rc = in->dim == 1 ? step1d(in, nsteps, renormalize)
         : in->dim == 2 ? step2d(in, nsteps, renormalize) : step3d(in, nsteps, renormalize);
    if (rc) return rc;
    in->steps += nsteps;
    return QSG_OK;
}

int qsg_sync(qsg_inst *in)
{
    if (!in) return fail(QSG_ERR_ARG, "qsg_sync: null instance");
    qsg_ctx *ctx = in->ctx;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (int rc = lost_state(in, "qsg_sync")) return rc;
    return sync_checked(in, in->st, "qsg_sync");
}

int qsg_norm2(qsg_inst *in, double *out)
{
    if (!in || !out) return fail(QSG_ERR_ARG, "qsg_norm2: null argument");
    std::lock_guard<std::mutex> lk(in->ctx->mu);
    if (int rc = lost_state(in, "qsg_norm2")) return rc;
    double s = 0;
    int rc = reduce(in, 0, user_n(in), 0, &s);
    if (rc) return rc;
    *out = s * in->dv;
    return QSG_OK;
}

int qsg_step_norm2(qsg_inst *in, double *out)
{
    if (!in || !out) return fail(QSG_ERR_ARG, "qsg_step_norm2: null argument");
    std::lock_guard<std::mutex> lk(in->ctx->mu);
    if (int rc = lost_state(in, "qsg_step_norm2")) return rc;
    if (in->dim == 2 && in->pending && in->dt.imag() == 0) {
        // the deferred closing V factor has modulus 1: the sums the last
        // column pass took, times G Ny (split-k scale), are the norm
        qsg_ctx *ctx = in->ctx;
        const int tiles = (in->ny / in->geom.col_w) * in->geom.g;
        QSG_CUDA(qsg::launch_finalize(in->cparts, tiles, 1, ctx->sums, ctx->st));
        QSG_CUDA(cudaMemcpyAsync(ctx->host_sums, ctx->sums, sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
        if (int rc = sync_checked(in, ctx->st, "qsg_step_norm2")) return rc;
        *out = ctx->host_sums[0] * cparts_scale(in) * in->dv;
        return QSG_OK;
    }
    if (in->dim == 1 && in->snorm_valid) {
        // the one-CTA 1D kernel summed the state it ended in
        QSG_CUDA(cudaMemcpyAsync(in->ctx->host_sums, in->snorm, sizeof(double), cudaMemcpyDeviceToHost, in->st));
        if (int rc = sync_checked(in, in->st, "qsg_step_norm2")) return rc;
        *out = in->ctx->host_sums[0] * in->dv;
        return QSG_OK;
    }
    double s = 0;
    int rc = reduce(in, 0, user_n(in), 0, &s);
    if (rc) return rc;
    *out = s * in->dv;
    return QSG_OK;
}

int qsg_step_norm2_post(qsg_inst *in, uint64_t *ticket)
{
    if (!in || !ticket) return fail(QSG_ERR_ARG, "qsg_step_norm2_post: null argument");
    std::lock_guard<std::mutex> lk(in->ctx->mu);
    if (int rc = lost_state(in, "qsg_step_norm2_post")) return rc;
    qsg_ctx *ctx = in->ctx;
    int rc;
    if (!in->ring_dev) {
        void *p = nullptr;
        if ((rc = inst_alloc(in, sizeof(double) * qsg_inst::kRing, &p))) return rc;
        in->ring_dev = static_cast<double *>(p);
        // kRing values, then kRing copies of the failure counter (one per post)
        QSG_CUDA(cudaMallocHost(&in->ring_host, (sizeof(double) + sizeof(unsigned)) * qsg_inst::kRing));
        for (cudaEvent_t &e : in->ring_ev) QSG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    const int slot = (int)(in->ring_next % qsg_inst::kRing);
    double *dst = in->ring_dev + slot;
    if (in->dim == 1 && in->snorm_valid) {
        // the one-CTA 1D kernel's own sum of its final state: one copy, no kernel
        QSG_CUDA(cudaMemcpyAsync(in->ring_host + slot, in->snorm, sizeof(double), cudaMemcpyDeviceToHost, in->st));
        QSG_CUDA(cudaMemcpyAsync(ring_err(in, slot), in->err, sizeof(unsigned), cudaMemcpyDeviceToHost, in->st));
        QSG_CUDA(cudaEventRecord(in->ring_ev[slot], in->st));
        in->ring_scale[slot] = in->dv;
        *ticket = in->ring_next++;
        return QSG_OK;
    }
    if (in->dim == 2 && in->pending && in->dt.imag() == 0) {
        // as qsg_step_norm2: the last column pass's split-k sums
        const int tiles = (in->ny / in->geom.col_w) * in->geom.g;
        QSG_CUDA(qsg::launch_finalize(in->cparts, tiles, 1, dst, ctx->st));
        in->ring_scale[slot] = cparts_scale(in) * in->dv;
    } else {
        if ((rc = settle(in))) return rc;
        int np = 0;
        QSG_CUDA(qsg::launch_reduce(in->prec, in->psi, in->V, 0, user_n(in), 0, ctx->partials, ctx->max_partials,
                                    &np, ctx->st));
        QSG_CUDA(qsg::launch_finalize(ctx->partials, np, 1, dst, ctx->st));
        in->ring_scale[slot] = in->dv;
    }
    QSG_CUDA(cudaMemcpyAsync(in->ring_host + slot, dst, sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
    QSG_CUDA(cudaMemcpyAsync(ring_err(in, slot), in->err, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->st));
    QSG_CUDA(cudaEventRecord(in->ring_ev[slot], ctx->st));
    *ticket = in->ring_next++;
    return QSG_OK;
}

int qsg_step_norm2_get(qsg_inst *in, uint64_t ticket, double *out)
{
    if (!in || !out) return fail(QSG_ERR_ARG, "qsg_step_norm2_get: null argument");
    std::lock_guard<std::mutex> lk(in->ctx->mu);
    if (ticket >= in->ring_next) return fail(QSG_ERR_ARG, "qsg_step_norm2_get: ticket not posted");
    if (in->ring_next - ticket > (uint64_t)qsg_inst::kRing)
        return fail(QSG_ERR_STATE, "qsg_step_norm2_get: ticket overwritten (more than 64 posts since)");
    if (int rc = lost_state(in, "qsg_step_norm2_get")) return rc;
    const int slot = (int)(ticket % qsg_inst::kRing);
    QSG_CUDA(cudaEventSynchronize(in->ring_ev[slot]));  // that copy only, not the work queued after it
    std::memcpy(in->ctx->host_sums + 7, ring_err(in, slot), sizeof(unsigned));
    if (int rc = err_after_sync(in, "qsg_step_norm2_get")) return rc;
    *out = in->ring_host[slot] * in->ring_scale[slot];
    return QSG_OK;
}

int qsg_energies(qsg_inst *in, double *kin, double *pot)
{
    if (!in) return fail(QSG_ERR_ARG, "qsg_energies: null instance");
    std::lock_guard<std::mutex> lk(in->ctx->mu);
    qsg_ctx *ctx = in->ctx;
    int rc;
    if ((rc = lost_state(in, "qsg_energies"))) return rc;
    if ((rc = settle(in))) return rc;
    if (pot) {
        // Abs2Mul(psi, V) dv / Norm2 (src/EvolverImpl.cpp:45-49)
        double s1 = 0, s0 = 0;
        if ((rc = reduce(in, 0, user_n(in), 1, &s1))) return rc;
        if ((rc = reduce(in, 0, user_n(in), 0, &s0))) return rc;
        *pot = (s1 * in->dv) / (s0 * in->dv);
    }
    if (kin && in->dim == 3) {
        if ((rc = kinetic3d(in, kin))) return rc;
    } else if (kin) {
        if (in->dim == 1) {
            // periodic branch omits hbar^2 (src/SplittingMethod1D.cpp:101-102); a wall
            // extension of 2n sites keeps it, with Dk = 2 pi/(dx 2n) = pi/(dx n) the wall's
            // Dk (:117-119): |F|^2 of the odd extension is even, so the 2n-periodic ratio
            // sum |F_k|^2 fold(k)^2 / sum |F_k|^2 is the wall's ratio over k < n
            const double dk = 2 * kPi / (in->dx * in->n);
            const double DT = in->wall_ext ? (dk * in->hbar) * (dk * in->hbar) / (2 * in->mass)
                                           : dk * dk / (2 * in->mass);
            if (in->blue) {
                qsg::BlueArgs ba{};
                ba.psi = in->psi;
                ba.tw = in->tw;
                ba.w = in->bw;
                ba.hs = in->bhs;
                ba.n = (int)in->n;
                ba.wall_n = in->wall_ext ? (int)in->n_out : 0;
                QSG_CUDA(qsg::launch_kinetic1d_blue(in->prec, in->blue_m, ba, DT, ctx->sums, ctx->st));
            } else if (in->boundary == QSG_INFINITE_WALL && !in->wall_ext) {
                // wall branch: Dk = pi/(dx N), DT = (Dk hbar)^2/(2m) (src/SplittingMethod1D.cpp:117-119)
                const double dkw = kPi / (in->dx * in->n);
                const double DTw = (dkw * in->hbar) * (dkw * in->hbar) / (2 * in->mass);
                QSG_CUDA(qsg::launch_kinetic1d_wall(in->prec, (int)in->n, in->psi, in->tw, DTw, ctx->sums, ctx->st));
            } else if (!in->fourstep) {
                QSG_CUDA(qsg::launch_kinetic1d(in->prec, (int)in->n, in->psi, in->tw, DT, ctx->sums, ctx->st));
            } else if (in->bfs) {
                // |DFT_n(psi)_k| = |C_h(w psi)_k| for k < n: on a copy, the column pass
                // with the chirp, the row pass with FFT_M(h) / M, the column pass back
                // to natural order; then sum |.|^2 fold(k)^2 DT / sum |.|^2 over k < n
                const size_t bytes = in->n * csize(in->prec);
                if ((rc = ensure_scratch(ctx, bytes + sizeof(qsg::FsInst)))) return rc;
                qsg::FsInst h{};
                h.psi = ctx->scratch;
                h.vtab[0] = in->bchirp;
                h.ktab[0] = in->bh1;
                qsg::FsInst *dd = reinterpret_cast<qsg::FsInst *>(static_cast<char *>(ctx->scratch) + bytes);
                QSG_CUDA(cudaMemcpyAsync(dd, &h, sizeof(h), cudaMemcpyHostToDevice, ctx->st));
                QSG_CUDA(cudaMemcpyAsync(ctx->scratch, in->psi, bytes, cudaMemcpyDeviceToDevice, ctx->st));
                qsg::FsColArgs ca{};
                ca.inst = dd;
                ca.tw_col = in->tw_fs_col;
                ca.tw_n = in->tw_n;
                ca.n1 = in->fsg.n1;
                ca.vsel = 0;
                ca.in_k = 0;
                ca.out_k = 1;
                QSG_CUDA(qsg::launch_fs_col(in->prec, in->fsg, ca, 1, ctx->st));
                qsg::FsRowArgs ra{};
                ra.inst = dd;
                ra.tw_row = in->tw_fs_row;
                ra.ksel = 0;
                ra.plain = 1;
                QSG_CUDA(qsg::launch_fs_row(in->prec, in->fsg, ra, 1, ctx->st));
                ca.vsel = 1;  // no table: the descriptor's second V entry is null
                ca.in_k = 1;
                ca.out_k = 0;
                QSG_CUDA(qsg::launch_fs_col(in->prec, in->fsg, ca, 1, ctx->st));
                double sk[2];
                for (int mode = 1; mode >= 0; --mode) {
                    int np = 0;
                    QSG_CUDA(qsg::launch_reduce(in->prec, ctx->scratch, in->bkw, 0, in->bfs_n, mode, ctx->partials,
                                                ctx->max_partials, &np, ctx->st));
                    QSG_CUDA(qsg::launch_finalize(ctx->partials, np, 1, ctx->sums, ctx->st));
                    QSG_CUDA(cudaMemcpyAsync(ctx->host_sums, ctx->sums, sizeof(double), cudaMemcpyDeviceToHost,
                                             ctx->st));
                    if ((rc = sync_checked(in, ctx->st, "qsg_energies"))) return rc;
                    sk[mode] = ctx->host_sums[0];
                }
                *kin = sk[1] / sk[0];
                return QSG_OK;
            } else {
                // forward transform of a copy: column pass (natural -> k layout), then row
                // FFTs with the reductions
                const size_t bytes = in->n * csize(in->prec);
                if ((rc = ensure_scratch(ctx, bytes + 2 * sizeof(qsg::FsInst)))) return rc;
                qsg::FsInst h{};
                h.psi = ctx->scratch;
                qsg::FsInst *dd = reinterpret_cast<qsg::FsInst *>(static_cast<char *>(ctx->scratch) + bytes);
                QSG_CUDA(cudaMemcpyAsync(dd, &h, sizeof(h), cudaMemcpyHostToDevice, ctx->st));
                QSG_CUDA(cudaMemcpyAsync(ctx->scratch, in->psi, bytes, cudaMemcpyDeviceToDevice, ctx->st));
                qsg::FsColArgs ca{};
                ca.inst = dd;
                ca.tw_col = in->tw_fs_col;
                ca.tw_n = in->tw_n;
                ca.n1 = in->fsg.n1;
                ca.vsel = 0;
                ca.in_k = 0;
                ca.out_k = 1;
                ca.wall = in->wall_ext ? 1 : 0;  // the wall KinEn transforms psi with sites 0 and n zeroed
                QSG_CUDA(qsg::launch_fs_col(in->prec, in->fsg, ca, 1, ctx->st));
                qsg::FsRowArgs ra{};
                ra.inst = dd;
                ra.tw_row = in->tw_fs_row;
                if (2 * in->fsg.row_blocks > 2 * ctx->max_partials) return fail(QSG_ERR_STATE, "partials buffer too small");
                QSG_CUDA(qsg::launch_fs_row_kinetic(in->prec, in->fsg, ra, DT, ctx->partials, ctx->st));
                QSG_CUDA(qsg::launch_finalize(ctx->partials, in->fsg.row_blocks, 2, ctx->sums, ctx->st));
            }
            QSG_CUDA(cudaMemcpyAsync(ctx->host_sums, ctx->sums, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                                     ctx->st));
            if ((rc = sync_checked(in, ctx->st, "qsg_energies"))) return rc;
            *kin = ctx->host_sums[0] / ctx->host_sums[1];
        } else {
            const double dkx = 2 * kPi / (in->dx * in->nx), dky = 2 * kPi / (in->dy * in->ny);
            const double DTx = (dkx * in->hbar) * (dkx * in->hbar) / (2 * in->mass);
            const double DTy = (dky * in->hbar) * (dky * in->hbar) / (2 * in->mass);
            if ((rc = ensure_scratch(ctx, in->n * csize(in->prec)))) return rc;
            if (in->blue2) {
                // SplittingMethod2D::CalKinEn on a copy: row DFTs, then the column DFTs with the sums
                QSG_CUDA(cudaMemcpyAsync(ctx->scratch, in->psi, in->n * csize(in->prec), cudaMemcpyDeviceToDevice,
                                         ctx->st));
                qsg::Blue2DArgs a{};
                a.psi = ctx->scratch;
                a.out_k = 1;
                a.tw = in->btwy;
                a.w = in->bwy;
                a.hs = in->bhsy;
                a.nx = in->nx;
                a.ny = in->ny;
                QSG_CUDA(qsg::launch_row_blue(in->prec, in->bmy, a, ctx->st));
                a.out_k = 0;
                a.tw = in->btwx;
                a.w = in->bwx;
                a.hs = in->bhsx;
                const int w = qsg::blue_cols_per_cta(in->prec, in->bmx);
                const int nblk = (in->ny + w - 1) / w;
                if (nblk > ctx->max_partials) return fail(QSG_ERR_STATE, "partials buffer too small");
                QSG_CUDA(qsg::launch_col_blue(in->prec, in->bmx, a, true, DTx, DTy, ctx->partials, ctx->st));
                QSG_CUDA(qsg::launch_finalize(ctx->partials, nblk, 2, ctx->sums, ctx->st));
                QSG_CUDA(cudaMemcpyAsync(ctx->host_sums, ctx->sums, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                                         ctx->st));
                if ((rc = sync_checked(in, ctx->st, "qsg_energies"))) return rc;
                *kin = ctx->host_sums[0] / ctx->host_sums[1];
                return QSG_OK;
            }
            if ((rc = row_pass(in, false, true, nullptr, false, nullptr, in->psi, ctx->scratch))) return rc;
            qsg::ColPassArgs a{};
            a.psi = ctx->scratch;
            a.tw_col = in->tw_kin;
            a.nx = in->nx;
            a.ny = in->ny;
            a.g = in->geom.g;
            const int nblk = (in->ny / in->geom.kin_w) * in->geom.g;
            if (nblk > ctx->max_partials) return fail(QSG_ERR_STATE, "partials buffer too small");
            QSG_CUDA(qsg::launch_col_kinetic(in->prec, in->geom, a, DTx, DTy, ctx->partials, ctx->st));
            QSG_CUDA(qsg::launch_finalize(ctx->partials, nblk, 2, ctx->sums, ctx->st));
            QSG_CUDA(cudaMemcpyAsync(ctx->host_sums, ctx->sums, 2 * sizeof(double), cudaMemcpyDeviceToHost,
                                     ctx->st));
            if ((rc = sync_checked(in, ctx->st, "qsg_energies"))) return rc;
            *kin = ctx->host_sums[0] / ctx->host_sums[1];
        }
    }
    return QSG_OK;
}

int qsg_xavg(qsg_inst *in, double x0, double *out)
{
    if (!in || !out) return fail(QSG_ERR_ARG, "qsg_xavg: null argument");
    if (in->dim != 1) return fail(QSG_ERR_ARG, "qsg_xavg: 1D instances only");
    std::lock_guard<std::mutex> lk(in->ctx->mu);
    double s2 = 0, s0 = 0;
    int rc;
    if ((rc = lost_state(in, "qsg_xavg"))) return rc;
    if ((rc = reduce(in, 0, user_n(in), 2, &s2))) return rc;
    if ((rc = reduce(in, 0, user_n(in), 0, &s0))) return rc;
    *out = x0 + in->dx * (s2 / s0);
    return QSG_OK;
}

int qsg_norm2_range(qsg_inst *in, double x0, double xa, double xb, double *out)
{
    if (!in || !out) return fail(QSG_ERR_ARG, "qsg_norm2_range: null argument");
    if (in->dim != 1) return fail(QSG_ERR_ARG, "qsg_norm2_range: 1D instances only");
    std::lock_guard<std::mutex> lk(in->ctx->mu);
    if (int rc = lost_state(in, "qsg_norm2_range")) return rc;
    int64_t i1 = (int64_t)((xa - x0) / in->dx), i2 = (int64_t)((xb - x0) / in->dx);
    if (i1 <= 0) i1 = 0;
    if (i2 >= (int64_t)user_n(in)) i2 = (int64_t)user_n(in);
    if (i1 >= i2) {
        *out = 0;
        return QSG_OK;
    }
    double s = 0;
    int rc = reduce(in, (size_t)i1, (size_t)i2, 0, &s);
    if (rc) return rc;
    *out = s * in->dx;
    return QSG_OK;
}

int qsg_get_psi(qsg_inst *in, double *out)
{
    if (!in || !out) return fail(QSG_ERR_ARG, "qsg_get_psi: null argument");
    std::lock_guard<std::mutex> lk(in->ctx->mu);
    qsg_ctx *ctx = in->ctx;
    if (int rc = lost_state(in, "qsg_get_psi")) return rc;
    if (int rc = settle(in)) return rc;
    const uint64_t n = user_n(in);
    if (in->prec == 0) {
        QSG_CUDA(cudaMemcpyAsync(out, in->psi, n * 16, cudaMemcpyDeviceToHost, ctx->st));
    } else {
        int rc = ensure_scratch(ctx, n * 16);
        if (rc) return rc;
        QSG_CUDA(qsg::launch_c64_to_c128(ctx->scratch, in->psi, n, ctx->st));
        QSG_CUDA(cudaMemcpyAsync(out, ctx->scratch, n * 16, cudaMemcpyDeviceToHost, ctx->st));
    }
    // a pass that timed out before this read leaves out holding a half-updated state: reported here
    return sync_checked(in, ctx->st, "qsg_get_psi");
}

int qsg_set_psi(qsg_inst *in, const double *psi)
{
    if (!in || !psi) return fail(QSG_ERR_ARG, "qsg_set_psi: null argument");
    std::lock_guard<std::mutex> lk(in->ctx->mu);
    int rc;
    if (in->wall_ext) {
        std::vector<double> pe;
        if ((rc = wall_odd_extension(psi, in->n_out, pe))) return rc;
        rc = upload_psi(in, pe.data());
        if (!rc) QSG_CUDA(cudaStreamSynchronize(in->ctx->st));  // pe is pageable and goes out of scope
    } else {
        rc = upload_psi(in, psi);
    }
    if (rc) return rc;
    in->pending = false;  // the state is replaced, with it any deferred row pass
    in->snorm_valid = false;
    // the new state makes an earlier timed-out pass irrelevant: acknowledge its count
    if ((rc = queue_err_copy(in, in->ctx->st))) return rc;
    QSG_CUDA(cudaStreamSynchronize(in->ctx->st));
    std::memcpy(&in->err_seen, in->ctx->host_sums + 7, sizeof(unsigned));
    in->lost = false;
    return QSG_OK;
}

int qsg_steps_taken(qsg_inst *in, uint64_t *out)
{
    if (!in || !out) return fail(QSG_ERR_ARG, "qsg_steps_taken: null argument");
    *out = in->steps;
    return QSG_OK;
}

void qsg_destroy(qsg_inst *in)
{
    if (!in) return;
    std::lock_guard<std::mutex> lk(in->ctx->mu);
    free_inst(in);
}

int qsg_candidate_plans(int precision, uint64_t nx, uint64_t ny, qsg_plan2d *out, int cap)
{
    if ((precision != QSG_FP64 && precision != QSG_MIXED) || nx > 8192 || ny > 8192) return 0;
    std::vector<Plan2D> v(256);
    const int n = qsg::candidate_plans(precision, (int)nx, (int)ny, v.data(), (int)v.size());
    for (int i = 0; i < n && i < cap && out; ++i)
        out[i] = qsg_plan2d{v[i].g, v[i].row_e, v[i].row_nt, v[i].col_e, v[i].col_w, v[i].row_kind};
    return n;
}

int qsg_get_plan(qsg_inst *in, qsg_plan2d *out)
{
    if (!in || !out) return fail(QSG_ERR_ARG, "qsg_get_plan: null argument");
    if (in->dim != 2) return fail(QSG_ERR_ARG, "qsg_get_plan: 2D instances only");
    *out = qsg_plan2d{in->plan.g, in->plan.row_e, in->plan.row_nt, in->plan.col_e, in->plan.col_w, in->plan.row_kind};
    return QSG_OK;
}

int qsg_set_plan(qsg_inst *in, const qsg_plan2d *p)
{
    if (!in || !p) return fail(QSG_ERR_ARG, "qsg_set_plan: null argument");
    if (in->dim != 2) return fail(QSG_ERR_ARG, "qsg_set_plan: 2D instances only");
    if (in->blue2) return fail(QSG_ERR_UNSUPPORTED, "qsg_set_plan: no plans for a grid with a side that is not a power of two");
    std::lock_guard<std::mutex> lk(in->ctx->mu);
    if (int rc = lost_state(in, "qsg_set_plan")) return rc;
    QSG_CUDA(cudaSetDevice(in->ctx->dev));
    if (int rc = settle(in)) return rc;  // the split-k layout belongs to the current plan
    QSG_CUDA(cudaStreamSynchronize(in->ctx->st));
    return apply_plan(in, Plan2D{p->g, p->row_e, p->row_nt, p->col_e, p->col_w, p->row_kind});
}

int qsg_check_wait_timeout(qsg_inst *in)
{
    if (!in) return fail(QSG_ERR_ARG, "qsg_check_wait_timeout: null instance");
    if (!(in->dim == 2 && in->prec == 1 && momentum(in)))
        return fail(QSG_ERR_UNSUPPORTED, "qsg_check_wait_timeout: needs a complex64 2D momentum-form instance");
    qsg_ctx *ctx = in->ctx;
    std::lock_guard<std::mutex> lk(ctx->mu);
    QSG_CUDA(cudaSetDevice(ctx->dev));
    if (int rc = lost_state(in, "qsg_check_wait_timeout")) return rc;
    // The withheld pass returns before any store, but it is reported as any
    // pass that ran out of time is: the instance's state counts as lost.
    if (int rc = col_pass(in, 0, nullptr, false, false, false, true)) return rc;
    return sync_checked(in, in->st, "qsg_check_wait_timeout");
}

int qsg_set_form(qsg_inst *in, int form)
{
    if (!in) return fail(QSG_ERR_ARG, "qsg_set_form: null instance");
    if (form != QSG_FORM_MOMENTUM && form != QSG_FORM_DIRECT) return fail(QSG_ERR_ARG, "qsg_set_form: unknown form");
    std::lock_guard<std::mutex> lk(in->ctx->mu);
    if (form == QSG_FORM_MOMENTUM && !(in->dim == 2 && in->prec == 1 && in->work))
        return fail(QSG_ERR_UNSUPPORTED, "qsg_set_form: the momentum form is for complex64 2D instances");
    if (int rc = lost_state(in, "qsg_set_form")) return rc;
    QSG_CUDA(cudaSetDevice(in->ctx->dev));
    if (int rc = settle(in)) return rc;  // the deferred pass belongs to the current form
    in->form = form;
    return QSG_OK;
}

int qsg_get_form(qsg_inst *in, int *form)
{
    if (!in || !form) return fail(QSG_ERR_ARG, "qsg_get_form: null argument");
    *form = in->form;
    return QSG_OK;
}

int qsg_autotune(qsg_inst *in, int trial_steps, int persist, qsg_plan2d *best, double *best_ms_per_step)
{
    if (!in) return fail(QSG_ERR_ARG, "qsg_autotune: null instance");
    if (in->dim != 2) return fail(QSG_ERR_ARG, "qsg_autotune: 2D instances only");
    if (in->blue2) return fail(QSG_ERR_UNSUPPORTED, "qsg_autotune: no plans for a grid with a side that is not a power of two");
    if (trial_steps < 1) trial_steps = 4;
    std::lock_guard<std::mutex> lk(in->ctx->mu);
    qsg_ctx *ctx = in->ctx;
    if (int rc = lost_state(in, "qsg_autotune")) return rc;
    QSG_CUDA(cudaSetDevice(ctx->dev));
    std::vector<Plan2D> cands(256);
    const int n = qsg::candidate_plans(in->prec, in->nx, in->ny, cands.data(), (int)cands.size());
    if (n <= 0) return fail(QSG_ERR_UNSUPPORTED, "qsg_autotune: no plan for this grid");
    cands.resize(n);
    // the trials evolve a copy; psi and the step count are restored afterwards
    const size_t bytes = in->n * csize(in->prec);
    int rc = settle(in);
    if (rc) return rc;
    if ((rc = ensure_scratch(ctx, bytes))) return rc;
    QSG_CUDA(cudaMemcpyAsync(ctx->scratch, in->psi, bytes, cudaMemcpyDeviceToDevice, ctx->st));
    const Plan2D keep = in->plan;
    TuneGuard g(ctx);
    QSG_CUDA(cudaEventCreate(&g.e0));
    QSG_CUDA(cudaEventCreate(&g.e1));
    cudaEvent_t e0 = g.e0, e1 = g.e1;
    double best_ms = 1e30;
    Plan2D best_p = keep;
    for (const Plan2D &p : cands) {
        if (apply_plan(in, p)) continue;
        if (step2d(in, 1, 0)) continue;  // warm-up (also loads the module)
        cudaEventRecord(e0, ctx->st);
        if (step2d(in, (uint64_t)trial_steps, 0)) continue;
        cudaEventRecord(e1, ctx->st);
        if (cudaEventSynchronize(e1) != cudaSuccess) break;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        const double per = ms / trial_steps;
        if (per < best_ms) {
            best_ms = per;
            best_p = p;
        }
    }
    cudaError_t err = cudaGetLastError();
    QSG_CUDA(cudaMemcpyAsync(in->psi, ctx->scratch, bytes, cudaMemcpyDeviceToDevice, ctx->st));
    in->pending = false;  // the restored copy is the settled state
    // a trial pass that ran out of time worked on the copy: acknowledge its count
    if ((rc = queue_err_copy(in, ctx->st))) return rc;
    QSG_CUDA(cudaStreamSynchronize(ctx->st));
    std::memcpy(&in->err_seen, ctx->host_sums + 7, sizeof(unsigned));
    if (err != cudaSuccess) return fail(QSG_ERR_CUDA, std::string("qsg_autotune: ") + cudaGetErrorString(err));
    if ((rc = apply_plan(in, best_p))) return rc;
    ctx->plans[std::make_tuple(in->prec, in->nx, in->ny)] = best_p;
    if (persist) save_plan(ctx, in->prec, in->nx, in->ny, best_p, best_ms);
    if (best) *best = qsg_plan2d{best_p.g, best_p.row_e, best_p.row_nt, best_p.col_e, best_p.col_w, best_p.row_kind};
    if (best_ms_per_step) *best_ms_per_step = best_ms;
    return QSG_OK;
}

int qsg_candidate_plans_1d(int precision, uint64_t n, int boundary, qsg_plan1d *out, int cap)
{
    std::vector<qsg_plan1d> v;
    plans_1d(precision, n, boundary, v);
    for (int i = 0; out && i < (int)v.size() && i < cap; ++i) out[i] = v[i];
    return (int)v.size();
}

int qsg_get_plan_1d(qsg_inst *in, qsg_plan1d *out)
{
    if (!in || !out) return fail(QSG_ERR_ARG, "qsg_get_plan_1d: null argument");
    if (in->dim != 1) return fail(QSG_ERR_ARG, "qsg_get_plan_1d: 1D instances only");
    *out = in->plan1d;
    return QSG_OK;
}

int qsg_set_plan_1d(qsg_inst *in, const qsg_plan1d *p)
{
    if (!in || !p) return fail(QSG_ERR_ARG, "qsg_set_plan_1d: null argument");
    if (in->dim != 1) return fail(QSG_ERR_ARG, "qsg_set_plan_1d: 1D instances only");
    if (in->batch_member) return fail(QSG_ERR_STATE, "qsg_set_plan_1d: a batch member keeps its batch's plan");
    std::lock_guard<std::mutex> lk(in->ctx->mu);
    if (int rc = lost_state(in, "qsg_set_plan_1d")) return rc;
    QSG_CUDA(cudaSetDevice(in->ctx->dev));
    return apply_plan_1d(in, *p);
}

int qsg_autotune_1d(qsg_inst *in, int trial_steps, int persist, qsg_plan1d *best, double *best_ms_per_step)
{
    if (!in) return fail(QSG_ERR_ARG, "qsg_autotune_1d: null instance");
    if (in->dim != 1) return fail(QSG_ERR_ARG, "qsg_autotune_1d: 1D instances only");
    if (in->batch_member) return fail(QSG_ERR_STATE, "qsg_autotune_1d: a batch member keeps its batch's plan");
    if (trial_steps < 1) trial_steps = 4;
    qsg_ctx *ctx = in->ctx;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (int rc = lost_state(in, "qsg_autotune_1d")) return rc;
    QSG_CUDA(cudaSetDevice(ctx->dev));
    std::vector<qsg_plan1d> cands;
    plans_1d(in->prec, user_n(in), in->boundary, cands);
    if (cands.empty()) return fail(QSG_ERR_UNSUPPORTED, "qsg_autotune_1d: no plan for this instance");
    // each trial long enough to time: at least 2^22 site-steps
    const uint64_t steps = std::max<uint64_t>((uint64_t)trial_steps, ((uint64_t)1 << 22) / in->n);
    // the trials evolve a copy; psi is restored afterwards
    const size_t bytes = in->n * csize(in->prec);
    QSG_CUDA(cudaStreamSynchronize(in->st));
    int rc = ensure_scratch(ctx, bytes);
    if (rc) return rc;
    QSG_CUDA(cudaMemcpyAsync(ctx->scratch, in->psi, bytes, cudaMemcpyDeviceToDevice, ctx->st));
    QSG_CUDA(cudaStreamSynchronize(ctx->st));
    const qsg_plan1d keep = in->plan1d;
    const bool wall_zero = in->wall_zero;  // the trials step a copy: the state's zeroing is still due
    TuneGuard g(ctx);
    QSG_CUDA(cudaEventCreate(&g.e0));
    QSG_CUDA(cudaEventCreate(&g.e1));
    cudaEvent_t e0 = g.e0, e1 = g.e1;
    double best_ms = 1e30;
    qsg_plan1d best_p = keep;
    for (const qsg_plan1d &p : cands) {
        if (apply_plan_1d(in, p)) continue;  // the instance keeps its plan
        if (step1d(in, 1, 0)) continue;  // warm-up (also loads the module)
        cudaEventRecord(e0, in->st);
        if (step1d(in, steps, 0)) continue;
        cudaEventRecord(e1, in->st);
        if (cudaEventSynchronize(e1) != cudaSuccess) break;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        const double per = ms / (double)steps;
        if (per < best_ms) {
            best_ms = per;
            best_p = p;
        }
    }
    cudaError_t err = cudaGetLastError();
    QSG_CUDA(cudaStreamSynchronize(in->st));
    QSG_CUDA(cudaMemcpyAsync(in->psi, ctx->scratch, bytes, cudaMemcpyDeviceToDevice, ctx->st));
    in->snorm_valid = false;
    in->wall_zero = wall_zero;
    // a trial pass that ran out of time worked on the copy: acknowledge its count
    if ((rc = queue_err_copy(in, ctx->st))) return rc;
    QSG_CUDA(cudaStreamSynchronize(ctx->st));
    std::memcpy(&in->err_seen, ctx->host_sums + 7, sizeof(unsigned));
    if (err != cudaSuccess) return fail(QSG_ERR_CUDA, std::string("qsg_autotune_1d: ") + cudaGetErrorString(err));
    if ((rc = apply_plan_1d(in, best_p))) return rc;
    // a Bluestein four-step length has its one plan: nothing to remember
    const bool ext = in->wall_ext;
    if (!in->bfs) ctx->plans1d[std::make_tuple(in->prec, in->n, ext ? 1 : 0)] = best_p;
    if (persist && !in->bfs) save_plan_1d(ctx, in->prec, user_n(in), in->boundary, best_p, best_ms);
    if (best) *best = best_p;
    if (best_ms_per_step) *best_ms_per_step = best_ms;
    return QSG_OK;
}

// ---------------------------------------------------------------------------
// Batches of 1D instances: grouped by size; each size class is advanced by
// launches over all its instances (resident: one launch per qsg_batch_step;
// four-step: one launch per pass), on a stream of its own so classes overlap.
// ---------------------------------------------------------------------------

}  // extern "C"

struct qsg_batch {
    qsg_ctx *ctx = nullptr;
    std::vector<qsg_inst *> insts;
    struct Class {
        uint64_t n = 0;
        std::vector<int> members;
        qsg::FsInst *d_desc = nullptr;
        void *d_maps = nullptr;     // complex64 four-step: the members' tensor maps (3 each)
        double *d_dv = nullptr;
        cudaStream_t st = nullptr;
        cudaEvent_t done = nullptr;
        bool queued = false;        // stepped by the tile-queue launch, not a launch of its own
    };
    std::vector<Class> classes;
    // the tile queue over the queued classes (complex64 resident lengths 1024 .. 8192):
    // descriptors and dv of their members in class order, the tiles, the queue counter
    qsg::FsInst *q_desc = nullptr;
    double *q_dv = nullptr;
    qsg::QueueTile *q_tiles = nullptr;
    unsigned *q_counter = nullptr;
    int q_ntiles = 0;
    const void *q_tw = nullptr;     // any queued class's twiddles (the tiles carry their own)
    cudaStream_t q_st = nullptr;
    cudaEvent_t q_done = nullptr;
    uint64_t sites = 0;
    // the launches of one qsg_batch_step(nsteps) captured as a CUDA graph
    // (every class's launches for all nsteps, forked from and joined to the
    // context stream); replayed while nsteps repeats
    cudaGraphExec_t gexec = nullptr;
    uint64_t gsteps = 0;
    std::map<std::string, uint64_t> glaunches;  // launches per kernel name in the graph
    bool broken = false;  // a plan switch failed half-way: the descriptors cannot be trusted
};

static void batch_free(qsg_batch *b)
{
    if (!b) return;
    if (b->ctx) cudaSetDevice(b->ctx->dev);
    if (b->gexec) {
        if (b->ctx) cudaStreamSynchronize(b->ctx->st);
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    if (b->q_st) cudaStreamSynchronize(b->q_st);
    if (b->q_desc) cudaFreeAsync(b->q_desc, b->ctx->st);
    if (b->q_done) cudaEventDestroy(b->q_done);
    if (b->q_st) cudaStreamDestroy(b->q_st);
    for (auto &c : b->classes) {
        if (c.st) cudaStreamSynchronize(c.st);
        if (c.d_desc) cudaFreeAsync(c.d_desc, b->ctx->st);
        if (c.d_maps) cudaFreeAsync(c.d_maps, b->ctx->st);
        if (c.done) cudaEventDestroy(c.done);
        if (c.st) cudaStreamDestroy(c.st);
    }
    for (qsg_inst *in : b->insts) free_inst(in);
    delete b;
}

// Gather the complex64 resident classes of length 1024 .. 8192 into one tile
// queue: tiles of 8192 sites (8192 / n instances of one class each), the
// members' descriptors and dv in class order, a zeroed queue counter.
static int batch_make_queue(qsg_batch *b)
{
    qsg_ctx *ctx = b->ctx;
    const int qt = qsg::queue_tile_sites(b->insts.empty() ? 0 : b->insts[0]->prec);
    if (!ctx->batch_queue || qt == 0) return QSG_OK;
    std::vector<qsg::FsInst> desc;
    std::vector<double> dv;
    std::vector<qsg::QueueTile> tiles;
    for (auto &c : b->classes) {
        qsg_inst *proto = b->insts[c.members[0]];
        if (proto->fourstep || c.n < 1024 || c.n > (uint64_t)qt) continue;
        c.queued = true;
        const int per = qt / (int)c.n;
        const int first = (int)desc.size();
        for (size_t k = 0; k < c.members.size(); ++k) {
            qsg_inst *in = b->insts[c.members[k]];
            qsg::FsInst h{};
            h.psi = in->psi;
            h.vtab[0] = in->vtab[0];
            h.vtab[1] = in->vtab[1];
            h.ktab[0] = in->ktab[0];
            h.ktab[1] = in->ktab[1];
            desc.push_back(h);
            dv.push_back(in->dv);
        }
        for (int k = 0; k < (int)c.members.size(); k += per)
            tiles.push_back(qsg::QueueTile{proto->tw, (int)c.n, first + k, std::min(per, (int)c.members.size() - k), 0});
        b->q_tw = proto->tw;
    }
    if (tiles.empty()) return QSG_OK;
    // biggest lengths first: their tiles are the longest
    std::stable_sort(tiles.begin(), tiles.end(),
                     [](const qsg::QueueTile &x, const qsg::QueueTile &y) { return x.L > y.L; });
    const size_t bd = sizeof(qsg::FsInst) * desc.size(), bv = sizeof(double) * dv.size();
    const size_t bt = sizeof(qsg::QueueTile) * tiles.size();
    void *p = nullptr;
    QSG_CUDA(cudaMallocAsync(&p, bd + bv + bt + 256, ctx->st));
    b->q_desc = static_cast<qsg::FsInst *>(p);
    b->q_dv = reinterpret_cast<double *>(static_cast<char *>(p) + bd);
    b->q_tiles = reinterpret_cast<qsg::QueueTile *>(static_cast<char *>(p) + bd + bv);
    b->q_counter = reinterpret_cast<unsigned *>(static_cast<char *>(p) + bd + bv + bt);
    b->q_ntiles = (int)tiles.size();
    QSG_CUDA(cudaMemcpyAsync(b->q_desc, desc.data(), bd, cudaMemcpyHostToDevice, ctx->st));
    QSG_CUDA(cudaMemcpyAsync(b->q_dv, dv.data(), bv, cudaMemcpyHostToDevice, ctx->st));
    QSG_CUDA(cudaMemcpyAsync(b->q_tiles, tiles.data(), bt, cudaMemcpyHostToDevice, ctx->st));
    QSG_CUDA(cudaMemsetAsync(b->q_counter, 0, 2 * sizeof(unsigned), ctx->st));
    QSG_CUDA(cudaStreamSynchronize(ctx->st));
    QSG_CUDA(cudaStreamCreateWithFlags(&b->q_st, cudaStreamNonBlocking));
    QSG_CUDA(cudaEventCreateWithFlags(&b->q_done, cudaEventDisableTiming));
    return QSG_OK;
}

extern "C" {

int qsg_batch_create_1d(qsg_ctx *ctx, int count, const uint64_t *n, const double *dx, const double *dt_re,
                        const double *dt_im, double mass, double hbar, int order, int precision,
                        const double *const *psi0, const double *const *V, qsg_batch **out)
{
    if (!ctx || !out || !n || !dx || !dt_re || !psi0 || !V || count <= 0)
        return fail(QSG_ERR_ARG, "qsg_batch_create_1d: null argument or empty batch");
    *out = nullptr;
    std::lock_guard<std::mutex> lk(ctx->mu);
    QSG_CUDA(cudaSetDevice(ctx->dev));
    qsg_batch *b = new qsg_batch();
    b->ctx = ctx;
    std::map<uint64_t, int> cls;
    for (int i = 0; i < count; ++i) {
        qsg_inst *in = nullptr;
        int rc = create_1d_locked(ctx, n[i], dx[i], mass, hbar, dt_re[i], dt_im ? dt_im[i] : 0.0, order, precision,
                                  QSG_PERIOD, psi0[i], V[i], &in);
        if (!rc && (in->blue || in->bfs)) {
            free_inst(in);
            rc = fail(QSG_ERR_UNSUPPORTED, "n=" + std::to_string(n[i]) + ": batches take powers of two");
        }
        if (rc) {
            std::string msg = g_last_error;
            batch_free(b);
            return fail(rc, "qsg_batch_create_1d: instance " + std::to_string(i) + ": " + msg);
        }
        in->batch_member = true;
        b->insts.push_back(in);
        b->sites += n[i];
        auto it = cls.find(n[i]);
        if (it == cls.end()) {
            cls[n[i]] = (int)b->classes.size();
            b->classes.emplace_back();
            b->classes.back().n = n[i];
            it = cls.find(n[i]);
        }
        b->classes[it->second].members.push_back(i);
    }
    for (auto &c : b->classes) {
        std::vector<qsg::FsInst> h(c.members.size());
        std::vector<double> dv(c.members.size());
        for (size_t k = 0; k < c.members.size(); ++k) {
            qsg_inst *in = b->insts[c.members[k]];
            h[k].psi = in->psi;
            h[k].vtab[0] = in->vtab[0];
            h[k].vtab[1] = in->vtab[1];
            h[k].ktab[0] = in->ktab[0];
            h[k].ktab[1] = in->ktab[1];
            h[k].partials = nullptr;
            dv[k] = in->dv;
        }
        void *p = nullptr;
        const size_t bytes = sizeof(qsg::FsInst) * h.size() + sizeof(double) * dv.size();
        cudaError_t e = cudaMallocAsync(&p, bytes, ctx->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
        if (e == cudaSuccess) {
            c.d_desc = static_cast<qsg::FsInst *>(p);
            c.d_dv = reinterpret_cast<double *>(c.d_desc + h.size());
            e = cudaMemcpy(c.d_desc, h.data(), sizeof(qsg::FsInst) * h.size(), cudaMemcpyHostToDevice);
        }
        if (e == cudaSuccess) e = cudaMemcpy(c.d_dv, dv.data(), sizeof(double) * dv.size(), cudaMemcpyHostToDevice);
        // a four-step class's launches report bounded-wait failures in its first member's counter
        for (size_t k = 1; k < c.members.size(); ++k) b->insts[c.members[k]]->err = b->insts[c.members[0]]->err;
        if (e == cudaSuccess && b->insts[c.members[0]]->fourstep) {
            std::vector<qsg_inst *> mi(c.members.size());
            for (size_t k = 0; k < mi.size(); ++k) mi[k] = b->insts[c.members[k]];
            size_t mb = 0;
            c.d_maps = fs_make_maps(ctx, mi.data(), mi.size(), &mb);
        }
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c.done, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            batch_free(b);
            return fail(QSG_ERR_CUDA, std::string("qsg_batch_create_1d: ") + cudaGetErrorString(e));
        }
    }
    if (int rc = batch_make_queue(b)) {
        const std::string msg = g_last_error;
        batch_free(b);
        return fail(rc, "qsg_batch_create_1d: " + msg);
    }
    *out = b;
    return QSG_OK;
}

}  // extern "C"

namespace {

// queue every class's launches for nsteps: each class on its own stream,
// forked from the context stream and joined back to it
int batch_enqueue(qsg_batch *b, uint64_t nsteps)
{
    qsg_ctx *ctx = b->ctx;
    // classes start after everything already queued on the context stream
    cudaEvent_t start;
    QSG_CUDA(cudaEventCreateWithFlags(&start, cudaEventDisableTiming));
    QSG_CUDA(cudaEventRecord(start, ctx->st));
    // biggest classes first, so their long launches start earliest
    std::vector<int> order(b->classes.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::sort(order.begin(), order.end(), [&](int x, int y) {
        return b->classes[x].n * b->classes[x].members.size() > b->classes[y].n * b->classes[y].members.size();
    });
    int rc = QSG_OK;
    if (b->q_ntiles > 0) {
        // every queued class in one persistent launch
        qsg::Evolve1DQueueArgs qa{};
        qa.b.inst = b->q_desc;
        qa.b.tw = b->q_tw;
        qa.b.dv = b->q_dv;
        qa.b.nsteps = nsteps;
        qa.b.order = b->insts[0]->order;
        qa.tiles = b->q_tiles;
        qa.ntiles = b->q_ntiles;
        qa.counter = b->q_counter;
        cudaError_t e = cudaStreamWaitEvent(b->q_st, start, 0);
        if (e == cudaSuccess) {
            ProfScope ps(ctx, "evolve1d_queue", b->q_st);
            e = qsg::launch_evolve1d_queue(b->insts[0]->prec, qa, b->q_st);
        }
        if (e == cudaSuccess) e = cudaEventRecord(b->q_done, b->q_st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->st, b->q_done, 0);
        if (e != cudaSuccess) rc = fail(QSG_ERR_CUDA, std::string("qsg_batch_step: tile queue: ") + cudaGetErrorString(e));
    }
    for (int ci : order) {
        if (rc) break;
        auto &c = b->classes[ci];
        if (c.queued) continue;
        qsg_inst *proto = b->insts[c.members[0]];
        cudaStreamWaitEvent(c.st, start, 0);
        if (!proto->fourstep) {
            qsg::Evolve1DBatchArgs a{};
            a.inst = c.d_desc;
            a.tw = proto->tw;
            a.dv = c.d_dv;
            a.nsteps = nsteps;
            a.order = proto->order;
            a.count = (int)c.members.size();
            ProfScope ps(ctx, "evolve1d_resident", c.st);
            cudaError_t e = qsg::launch_evolve1d(proto->prec, (int)proto->n, a, c.st);
            if (e != cudaSuccess) {
                rc = fail(QSG_ERR_CUDA, std::string("qsg_batch_step: ") + cudaGetErrorString(e));
                break;
            }
        } else if ((rc = step_fs(proto, c.d_desc, (int)c.members.size(), nsteps, c.st, c.d_maps))) {
            break;
        }
        cudaEventRecord(c.done, c.st);
        cudaStreamWaitEvent(ctx->st, c.done, 0);
    }
    cudaEventDestroy(start);
    return rc;
}

// capture batch_enqueue(nsteps) into b->gexec
int batch_capture(qsg_batch *b, uint64_t nsteps)
{
    qsg_ctx *ctx = b->ctx;
    // count the captured launches (launch-count profiling mode during the
    // capture, the context's own counts put back afterwards)
    const auto saved = ctx->prof_stats;
    const int prof = ctx->prof;
    ctx->prof_stats.clear();
    ctx->prof = 2;
    cudaError_t e = cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal);
    const int rc = e == cudaSuccess ? batch_enqueue(b, nsteps) : QSG_OK;
    cudaGraph_t g = nullptr;
    if (e == cudaSuccess) e = cudaStreamEndCapture(ctx->st, &g);
    std::map<std::string, uint64_t> counts;
    for (auto &kv : ctx->prof_stats) counts[kv.first] = kv.second.launches;
    ctx->prof_stats = saved;
    ctx->prof = prof;
    if (rc || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return rc ? rc : fail(QSG_ERR_CUDA, std::string("qsg_batch_step: graph capture: ") + cudaGetErrorString(e));
    }
    cudaGraphExec_t x = nullptr;
    const cudaError_t ei = cudaGraphInstantiate(&x, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) return fail(QSG_ERR_CUDA, std::string("qsg_batch_step: graph: ") + cudaGetErrorString(ei));
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    b->gexec = x;
    b->gsteps = nsteps;
    b->glaunches = counts;
    return QSG_OK;
}

}  // namespace

extern "C" {

// With graphs on (QSG_BATCH_GRAPHS=1), a step call is replayed from a graph
// captured on the first call with this nsteps; with per-launch event profiling
// on, or graphs off (the default), the launches are queued directly.
int qsg_batch_step(qsg_batch *b, uint64_t nsteps)
{
    if (!b) return fail(QSG_ERR_ARG, "qsg_batch_step: null batch");
    if (b->broken) return fail(QSG_ERR_STATE, "qsg_batch_step: a failed plan switch left the batch unusable");
    if (nsteps == 0) return QSG_OK;
    qsg_ctx *ctx = b->ctx;
    std::lock_guard<std::mutex> lk(ctx->mu);
    QSG_CUDA(cudaSetDevice(ctx->dev));
    int rc;
    if (ctx->prof == 1 || !ctx->graphs) {
        rc = batch_enqueue(b, nsteps);
    } else {
        rc = b->gexec && b->gsteps == nsteps ? QSG_OK : batch_capture(b, nsteps);
        if (!rc) QSG_CUDA(cudaGraphLaunch(b->gexec, ctx->st));
        if (!rc && ctx->prof == 2)
            for (auto &kv : b->glaunches) ctx->prof_stats[kv.first].launches += kv.second;
    }
    if (rc) return rc;
    for (qsg_inst *in : b->insts) {
        in->steps += nsteps;
        in->snorm_valid = false;  // batch launches do not write the per-instance sum
    }
    return QSG_OK;
}

int qsg_batch_size(qsg_batch *b, int *count, uint64_t *sites)
{
    if (!b) return fail(QSG_ERR_ARG, "qsg_batch_size: null batch");
    if (count) *count = (int)b->insts.size();
    if (sites) *sites = b->sites;
    return QSG_OK;
}

int qsg_batch_instance(qsg_batch *b, int i, qsg_inst **out)
{
    if (!b || !out || i < 0 || i >= (int)b->insts.size()) return fail(QSG_ERR_ARG, "qsg_batch_instance: bad index");
    *out = b->insts[i];
    return QSG_OK;
}

int qsg_batch_sync(qsg_batch *b)
{
    if (!b) return fail(QSG_ERR_ARG, "qsg_batch_sync: null batch");
    QSG_CUDA(cudaStreamSynchronize(b->ctx->st));
    return QSG_OK;
}

void qsg_batch_destroy(qsg_batch *b)
{
    if (!b) return;
    std::lock_guard<std::mutex> lk(b->ctx->mu);
    batch_free(b);
}

}  // extern "C"

namespace {

qsg_batch::Class *batch_class(qsg_batch *b, uint64_t n)
{
    for (auto &c : b->classes)
        if (c.n == n) return &c;
    return nullptr;
}

// Switch every member of a four-step class to plan p, then rebuild the class's
// descriptors (the kinetic tables move with the split) and tensor maps; a
// captured batch graph is dropped (it holds the old launches).
int batch_class_plan(qsg_batch *b, qsg_batch::Class &c, const qsg_plan1d &p)
{
    qsg_ctx *ctx = b->ctx;
    if (p.kind != 1 || !b->insts[c.members[0]]->fourstep)
        return fail(QSG_ERR_UNSUPPORTED, "batch plans: four-step plans of four-step classes only");
    QSG_CUDA(cudaStreamSynchronize(c.st));
    QSG_CUDA(cudaStreamSynchronize(ctx->st));
    int rc;
    const qsg_plan1d was = b->insts[c.members[0]]->plan1d;
    for (size_t k = 0; k < c.members.size(); ++k) {
        if ((rc = apply_plan_1d(b->insts[c.members[k]], p))) {
            // put the members switched so far back, so that the class's descriptors stay right
            const std::string msg = g_last_error;
            for (size_t j = 0; j < k; ++j) apply_plan_1d(b->insts[c.members[j]], was);
            return fail(rc, msg);
        }
    }
    std::vector<qsg::FsInst> h(c.members.size());
    std::vector<qsg_inst *> mi(c.members.size());
    for (size_t k = 0; k < c.members.size(); ++k) {
        qsg_inst *in = b->insts[c.members[k]];
        mi[k] = in;
        h[k] = qsg::FsInst{};
        h[k].psi = in->psi;
        h[k].vtab[0] = in->vtab[0];
        h[k].vtab[1] = in->vtab[1];
        h[k].ktab[0] = in->ktab[0];
        h[k].ktab[1] = in->ktab[1];
    }
    const cudaError_t e = cudaMemcpy(c.d_desc, h.data(), sizeof(qsg::FsInst) * h.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        // the class's descriptors may name released tables: the batch cannot step any more
        cudaGetLastError();
        b->broken = true;
        return fail(QSG_ERR_CUDA, std::string("batch plan switch: ") + cudaGetErrorString(e));
    }
    if (c.d_maps) cudaFreeAsync(c.d_maps, ctx->st);
    size_t mb = 0;
    c.d_maps = fs_make_maps(ctx, mi.data(), mi.size(), &mb);
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
        b->gsteps = 0;
    }
    QSG_CUDA(cudaStreamSynchronize(ctx->st));
    return QSG_OK;
}

}  // namespace

extern "C" {

int qsg_batch_get_plan_1d(qsg_batch *b, uint64_t n, qsg_plan1d *out)
{
    if (!b || !out) return fail(QSG_ERR_ARG, "qsg_batch_get_plan_1d: null argument");
    qsg_batch::Class *c = batch_class(b, n);
    if (!c) return fail(QSG_ERR_ARG, "qsg_batch_get_plan_1d: no member of length " + std::to_string(n));
    *out = b->insts[c->members[0]]->plan1d;
    return QSG_OK;
}

int qsg_batch_set_plan_1d(qsg_batch *b, uint64_t n, const qsg_plan1d *p)
{
    if (!b || !p) return fail(QSG_ERR_ARG, "qsg_batch_set_plan_1d: null argument");
    if (b->broken) return fail(QSG_ERR_STATE, "qsg_batch_set_plan_1d: a failed plan switch left the batch unusable");
    std::lock_guard<std::mutex> lk(b->ctx->mu);
    QSG_CUDA(cudaSetDevice(b->ctx->dev));
    qsg_batch::Class *c = batch_class(b, n);
    if (!c) return fail(QSG_ERR_ARG, "qsg_batch_set_plan_1d: no member of length " + std::to_string(n));
    qsg_inst *proto = b->insts[c->members[0]];
    if (same_plan1d(*p, proto->plan1d)) return QSG_OK;
    if (!plan1d_valid(proto->prec, n, QSG_PERIOD, *p))
        return fail(QSG_ERR_UNSUPPORTED, "qsg_batch_set_plan_1d: plan not available for length " + std::to_string(n));
    return batch_class_plan(b, *c, *p);
}

int qsg_batch_autotune(qsg_batch *b, int trial_steps, double *ms_per_step)
{
    if (!b) return fail(QSG_ERR_ARG, "qsg_batch_autotune: null batch");
    if (b->broken) return fail(QSG_ERR_STATE, "qsg_batch_autotune: a failed plan switch left the batch unusable");
    if (trial_steps < 1) trial_steps = 4;
    qsg_ctx *ctx = b->ctx;
    std::lock_guard<std::mutex> lk(ctx->mu);
    QSG_CUDA(cudaSetDevice(ctx->dev));
    QSG_CUDA(cudaStreamSynchronize(ctx->st));
    TuneGuard g(ctx);
    QSG_CUDA(cudaEventCreate(&g.e0));
    QSG_CUDA(cudaEventCreate(&g.e1));
    auto check = [](cudaError_t e, const char *what) -> int {
        if (e == cudaSuccess) return QSG_OK;
        cudaGetLastError();
        return fail(QSG_ERR_CUDA, std::string("qsg_batch_autotune: ") + what + ": " + cudaGetErrorString(e));
    };
    double total = 0;
    for (auto &c : b->classes) {
        qsg_inst *proto = b->insts[c.members[0]];
        if (!proto->fourstep) continue;
        std::vector<qsg_plan1d> cands;
        plans_1d(proto->prec, c.n, QSG_PERIOD, cands);
        cands.erase(std::remove_if(cands.begin(), cands.end(), [](const qsg_plan1d &q) { return q.kind != 1; }),
                    cands.end());
        if (cands.size() < 2) continue;
        const int ninst = (int)c.members.size();
        const uint64_t steps =
            std::max<uint64_t>((uint64_t)trial_steps, ((uint64_t)1 << 22) / (c.n * (uint64_t)ninst));
        // the trials evolve the members' states: keep copies
        const size_t bytes = proto->n * csize(proto->prec);
        int rc = ensure_scratch(ctx, bytes * ninst);
        if (rc) return rc;
        unsigned char *keep = static_cast<unsigned char *>(ctx->scratch);
        for (int k = 0; k < ninst && !rc; ++k)
            rc = check(cudaMemcpyAsync(keep + k * bytes, b->insts[c.members[k]]->psi, bytes, cudaMemcpyDeviceToDevice,
                                       ctx->st), "copy of a state");
        if (!rc) rc = check(cudaStreamSynchronize(ctx->st), "copy of the states");
        if (rc) return rc;
        qsg_plan1d best_p = proto->plan1d;
        double best_ms = 1e30;
        for (const qsg_plan1d &p : cands) {
            if (!same_plan1d(p, proto->plan1d) && (rc = batch_class_plan(b, c, p))) break;
            if ((rc = step_fs(proto, c.d_desc, ninst, 1, c.st, c.d_maps))) break;  // warm-up
            cudaEventRecord(g.e0, c.st);
            if ((rc = step_fs(proto, c.d_desc, ninst, steps, c.st, c.d_maps))) break;
            cudaEventRecord(g.e1, c.st);
            if ((rc = check(cudaEventSynchronize(g.e1), "trial"))) break;
            float ms = 0;
            cudaEventElapsedTime(&ms, g.e0, g.e1);
            if (ms / steps < best_ms) {
                best_ms = ms / steps;
                best_p = p;
            }
        }
        if (!rc && !same_plan1d(best_p, proto->plan1d)) rc = batch_class_plan(b, c, best_p);
        // the states go back whatever happened above
        const std::string msg = rc ? g_last_error : std::string();
        int rc2 = check(cudaStreamSynchronize(c.st), "trial stream");
        for (int k = 0; k < ninst && !rc2; ++k)
            rc2 = check(cudaMemcpyAsync(b->insts[c.members[k]]->psi, keep + k * bytes, bytes, cudaMemcpyDeviceToDevice,
                                        ctx->st), "restore of a state");
        if (!rc2) rc2 = check(cudaStreamSynchronize(ctx->st), "restore of the states");
        if (rc) return fail(rc, msg);
        if (rc2) return rc2;
        total += best_ms;
    }
    if (ms_per_step) *ms_per_step = total;
    return QSG_OK;
}

// ---------------------------------------------------------------------------
// Serving: a scheduler thread with continuous batching.
//
//   submit -> queued (host copies of psi0 / V)
//   admission (FIFO, while the server context's HBM budget allows): the
//     instance is created on the device and stays resident until done
//   each scheduler round, every running request whose previous chunk has
//     finished gets its next chunk:
//       resident 1D: requests of one (n, order, precision) advance together by
//                    the same step count in one batched launch
//       four-step 1D and 2D: a chunk of steps (about 1e8 site-steps) on the
//                    request's stream
//     launches go to a pool of streams, so work of different requests
//     overlaps on the device
//   done: psi copied back, device memory released, latency recorded
//
// Splitting a request's steps into chunks does not change its result: a
// chunk boundary performs the same multiplies as the fused step boundary
// inside a chunk, and every kernel is deterministic -- a request's result is
// the same alone or in any mix.
// ---------------------------------------------------------------------------

}  // extern "C"

#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>
#include <unordered_map>

namespace {

using clk = std::chrono::steady_clock;

struct SrvRequest {
    uint64_t id = 0;
    qsg_request req{};
    std::vector<double> psi0, V, result;
    qsg_spec spec{};
    bool has_spec = false;  // psi0 / V from spec
    int state = 0;  // 0 queued, 1 running, 2 done, 3 failed
    int error = 0;
    std::string message;
    clk::time_point submit, admit, first_dispatch, finish;
    qsg_inst *inst = nullptr;
    uint64_t dispatched = 0, chunks = 0;
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;  // recorded after this request's latest queued work (whichever stream ran it)
    bool in_flight = false;
    bool admitted_mid_flight = false;  // admitted while another request had work on the device
    int fail_rc = 0;                   // a dispatch failed: finish with this status once nothing is in flight
    std::string fail_msg;
};

}  // namespace

struct qsg_server {
    qsg_ctx *ctx = nullptr;
    int max_running = 64;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<std::shared_ptr<SrvRequest>> incoming;
    std::unordered_map<uint64_t, std::shared_ptr<SrvRequest>> all;
    uint64_t next_id = 1;
    bool stop = false;
    std::thread th;
    std::vector<cudaStream_t> streams;
    // device descriptor ring for batched resident launches
    qsg::FsInst *ring = nullptr, *ring_host = nullptr;  // device ring + pinned staging
    int ring_size = 4096, ring_pos = 0;
    // statistics
    uint64_t done_site_steps = 0, completed = 0, failed = 0;
    uint64_t admitted_mid_flight = 0;  // admissions while other requests had work on the device
    uint32_t max_in_flight = 0;        // most requests with device work queued at one time
    size_t peak_bytes = 0;
    clk::time_point t0 = clk::now();
    // host-side fault injection for tests (QSG_SERVER_FAIL_REQUEST=<id>): the
    // dispatches of that request fail with QSG_ERR_CUDA instead of launching
    uint64_t inject_fail_id = 0;
};

namespace {

size_t request_bytes(const qsg_request &r)
{
    const size_t n = (size_t)r.nx * (r.dim == 2 ? r.ny : 1);
    const size_t cs = r.precision == QSG_MIXED ? 8 : 16;
    const int ntab = r.order == 2 ? 1 : 2;
    if (r.dim == 1 && (n & (n - 1)) && n > 4096) {
        // Bluestein on the four-step passes: a buffer of M >= 2n - 1 sites with its
        // state, V, 7 (O2) or 9 (O4) tables and the upload staging, KinEn weights of n
        size_t m = 1;
        while (m < 2 * n - 1) m <<= 1;
        return m * (cs + 8 + (r.order == 2 ? 7 : 9) * cs + 16) + n * 8 + (r.spec ? n * 24 : 0);
    }
    const size_t work = r.dim == 2 && r.precision == QSG_MIXED ? n * cs : 0;  // momentum form
    return n * (cs + 8 + ntab * cs * 2) + n * 16 + work + (r.spec ? n * 24 : 0);  // psi, V, tables, staging, spec buffer
}

int srv_create(qsg_server *S, SrvRequest &q)
{
    const qsg_request &r = q.req;
    qsg_ctx *ctx = S->ctx;
    if (q.has_spec) {
        // the spec entry points take the context lock themselves
        ctx->mu.unlock();
        int rc = r.dim == 1 ? qsg_create_1d_spec(ctx, r.nx, r.dx, r.mass, r.hbar, r.dt_re, r.dt_im, r.order,
                                                 r.precision, QSG_PERIOD, &q.spec, &q.inst)
                            : qsg_create_2d_spec(ctx, r.nx, r.ny, r.dx, r.dy, r.mass, r.hbar, r.dt_re, r.dt_im,
                                                 r.order, r.precision, &q.spec, &q.inst);
        ctx->mu.lock();
        return rc;
    }
    if (r.dim == 1)
        return create_1d_locked(ctx, r.nx, r.dx, r.mass, r.hbar, r.dt_re, r.dt_im, r.order, r.precision, QSG_PERIOD,
                                q.psi0.data(), q.V.data(), &q.inst);
    ctx->mu.unlock();  // qsg_create_2d takes the context lock itself
    int rc = qsg_create_2d(ctx, r.nx, r.ny, r.dx, r.dy, r.mass, r.hbar, r.dt_re, r.dt_im, r.order, r.precision,
                           q.psi0.data(), q.V.data(), &q.inst);
    ctx->mu.lock();
    return rc;
}

void srv_finish(qsg_server *S, SrvRequest &q, int err, const std::string &msg)
{
    if (q.inst) {
        // the read back and the release run on the context stream, after the
        // request's last queued work (also on the failure paths: a dispatch
        // that failed part-way may have queued launches)
        if (q.ev) {
            const cudaError_t e = cudaStreamWaitEvent(S->ctx->st, q.ev, 0);
            if (e != cudaSuccess) {
                cudaStreamSynchronize(q.st);  // fall back to waiting on the host
                if (!err) {
                    err = QSG_ERR_CUDA;
                    q.message = std::string("cudaStreamWaitEvent: ") + cudaGetErrorString(e);
                }
            }
        }
        if (!err) {
            q.result.resize(2 * (size_t)user_n(q.inst));  // the caller's sites (a Bluestein buffer holds more)
            q.inst->st = S->ctx->st;
            S->ctx->mu.unlock();
            int rc = qsg_get_psi(q.inst, q.result.data());
            S->ctx->mu.lock();
            if (rc) {
                err = rc;
                q.message = g_last_error;
            }
        }
        free_inst(q.inst);
        q.inst = nullptr;
    }
    if (q.ev) {
        cudaEventDestroy(q.ev);
        q.ev = nullptr;
    }
    std::lock_guard<std::mutex> lk(S->mu);
    q.finish = clk::now();
    q.error = err;
    if (err && q.message.empty()) q.message = msg;
    q.state = err ? 3 : 2;
    q.psi0.clear();
    q.psi0.shrink_to_fit();
    q.V.clear();
    q.V.shrink_to_fit();
    if (err) {
        ++S->failed;
    } else {
        ++S->completed;
        S->done_site_steps += q.req.nx * (q.req.dim == 2 ? q.req.ny : 1) * q.req.nsteps;
    }
    S->cv.notify_all();
}

// A dispatch of q failed: its work so far is marked by q.ev (recorded on st
// where possible) and the request finishes with rc once nothing is in flight.
void srv_mark_failed(SrvRequest &q, cudaStream_t st, int rc, const std::string &msg)
{
    if (q.fail_rc) return;
    q.fail_rc = rc;
    q.fail_msg = msg;
    if (q.ev && st && cudaEventRecord(q.ev, st) != cudaSuccess) cudaStreamSynchronize(st);
    q.in_flight = false;
}

void srv_loop(qsg_server *S)
{
    qsg_ctx *ctx = S->ctx;
    cudaSetDevice(ctx->dev);
    std::deque<std::shared_ptr<SrvRequest>> pending;
    std::vector<std::shared_ptr<SrvRequest>> running;
    uint64_t rr = 0;
    // Uses of the descriptor ring, in launch order: slots [pos, pos + cnt) (device
    // ring and pinned staging) stay taken until the server-owned event `ev`,
    // recorded after the launch that reads them, has completed.  (Requests' own
    // events cannot mark the slots: a request that finishes destroys its event.)
    struct RingUse {
        int pos, cnt;
        cudaEvent_t ev;
    };
    std::deque<RingUse> ring_uses;
    std::vector<cudaEvent_t> ring_ev_pool;
    // true when [pos, pos + cnt) is free; retires the completed uses it overlaps
    auto ring_range_free = [&](int pos, int cnt) {
        bool free = true;
        for (auto it = ring_uses.begin(); it != ring_uses.end();) {
            if (!(it->pos < pos + cnt && pos < it->pos + it->cnt)) {
                ++it;
                continue;
            }
            const cudaError_t q = cudaEventQuery(it->ev);
            if (q == cudaErrorNotReady) {
                free = false;
                ++it;
                continue;
            }
            if (q != cudaSuccess) cudaGetLastError();  // a failed context: nothing is running any more
            ring_ev_pool.push_back(it->ev);
            it = ring_uses.erase(it);
        }
        return free;
    };
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(S->mu);
            if (S->stop) break;
            if (S->incoming.empty() && pending.empty() && running.empty())
                S->cv.wait_for(lk, std::chrono::milliseconds(5));
            while (!S->incoming.empty()) {
                pending.push_back(S->incoming.front());
                S->incoming.pop_front();
            }
        }
        std::unique_lock<std::mutex> clk_ctx(ctx->mu);
        bool progress = false;
        // admission, FIFO while memory allows
        while (!pending.empty() && (int)running.size() < S->max_running) {
            auto q = pending.front();
            const int rc = srv_create(S, *q);
            if (rc == QSG_ERR_BUDGET) {
                if (running.empty()) {  // can never fit
                    pending.pop_front();
                    srv_finish(S, *q, rc, "request does not fit the server's HBM budget");
                    progress = true;
                    continue;
                }
                break;  // wait for running requests to release memory
            }
            pending.pop_front();
            progress = true;
            if (rc) {
                srv_finish(S, *q, rc, g_last_error);
                continue;
            }
            q->st = S->streams[rr++ % S->streams.size()];
            q->inst->st = q->st;
            const cudaError_t ee = cudaEventCreateWithFlags(&q->ev, cudaEventDisableTiming);
            if (ee != cudaSuccess) {
                q->ev = nullptr;
                srv_finish(S, *q, QSG_ERR_CUDA, std::string("cudaEventCreateWithFlags: ") + cudaGetErrorString(ee));
                continue;
            }
            bool busy = false;
            for (auto &r : running) busy = busy || r->in_flight;
            {
                std::lock_guard<std::mutex> lk(S->mu);
                q->state = 1;
                q->admit = clk::now();
                q->admitted_mid_flight = busy;
                if (busy) ++S->admitted_mid_flight;
            }
            running.push_back(q);
        }
        S->peak_bytes = std::max(S->peak_bytes, ctx->in_use);
        // completions
        uint32_t in_flight_now = 0;
        for (size_t i = 0; i < running.size();) {
            auto &q = running[i];
            if (q->in_flight) {
                const cudaError_t eq = cudaEventQuery(q->ev);
                if (eq == cudaSuccess) {
                    q->in_flight = false;
                } else if (eq != cudaErrorNotReady) {
                    cudaGetLastError();
                    srv_mark_failed(*q, nullptr, QSG_ERR_CUDA, std::string("cudaEventQuery: ") + cudaGetErrorString(eq));
                }
            }
            if (!q->in_flight && (q->fail_rc || q->dispatched >= q->req.nsteps)) {
                srv_finish(S, *q, q->fail_rc, q->fail_msg);
                running.erase(running.begin() + i);
                progress = true;
                continue;
            }
            in_flight_now += q->in_flight ? 1 : 0;
            ++i;
        }
        // dispatch: batched resident groups
        std::map<std::tuple<uint64_t, int, int>, std::vector<SrvRequest *>> groups;
        for (auto &q : running)
            if (!q->in_flight && !q->fail_rc && q->dispatched < q->req.nsteps && q->req.dim == 1 &&
                !q->inst->fourstep && !q->inst->blue)
                groups[std::make_tuple(q->req.nx, q->req.order, q->req.precision)].push_back(q.get());
        for (auto &kv : groups) {
            auto &g = kv.second;
            uint64_t chunk = 1024;
            for (auto *q : g) chunk = std::min(chunk, q->req.nsteps - q->dispatched);
            const int cnt = (int)g.size();
            if (cnt > S->ring_size) continue;
            if (S->ring_pos + cnt > S->ring_size) S->ring_pos = 0;
            // the slots must not be in use by a launch still running
            if (!ring_range_free(S->ring_pos, cnt)) continue;
            cudaEvent_t done = nullptr;
            if (!ring_ev_pool.empty()) {
                done = ring_ev_pool.back();
                ring_ev_pool.pop_back();
            } else if (cudaEventCreateWithFlags(&done, cudaEventDisableTiming) != cudaSuccess) {
                cudaGetLastError();
                continue;  // retried on a later pass
            }
            qsg::FsInst *h = S->ring_host + S->ring_pos;
            for (int k = 0; k < cnt; ++k) {
                qsg_inst *in = g[k]->inst;
                in->snorm_valid = false;  // grouped launches do not write the per-instance sum
                h[k] = qsg::FsInst{};
                h[k].psi = in->psi;
                h[k].vtab[0] = in->vtab[0];
                h[k].vtab[1] = in->vtab[1];
                h[k].ktab[0] = in->ktab[0];
                h[k].ktab[1] = in->ktab[1];
            }
            qsg::FsInst *d = S->ring + S->ring_pos;
            cudaStream_t st = g[0]->st;
            cudaError_t e = cudaSuccess;
            const char *what = "";
            for (int k = 1; k < cnt && e == cudaSuccess; ++k) {
                e = cudaStreamWaitEvent(st, g[k]->ev, 0);
                what = "cudaStreamWaitEvent";
            }
            if (e == cudaSuccess) {
                e = cudaMemcpyAsync(d, h, sizeof(qsg::FsInst) * cnt, cudaMemcpyHostToDevice, st);
                what = "cudaMemcpyAsync";
            }
            bool injected = false;
            for (int k = 0; k < cnt; ++k) injected = injected || g[k]->id == S->inject_fail_id;
            if (e == cudaSuccess && !injected) {
                qsg::Evolve1DBatchArgs a{};
                a.inst = d;
                a.tw = g[0]->inst->tw;
                a.nsteps = chunk;
                a.order = g[0]->req.order;
                a.count = cnt;
                e = qsg::launch_evolve1d(g[0]->req.precision, (int)g[0]->req.nx, a, st);
                what = "resident 1D launch";
            }
            // ring slots (device and pinned staging) stay busy until this event
            const cudaError_t er = cudaEventRecord(done, st);
            if (er == cudaSuccess) {
                ring_uses.push_back(RingUse{S->ring_pos, cnt, done});
            } else {
                cudaStreamSynchronize(st);  // no event to wait on: the slots are free after this
                ring_ev_pool.push_back(done);
            }
            S->ring_pos += cnt;
            progress = true;
            if (e != cudaSuccess || injected) {
                // the group's launch failed: every member fails with it
                cudaGetLastError();
                const std::string msg = injected ? std::string("injected dispatch failure (QSG_SERVER_FAIL_REQUEST)")
                                                 : std::string(what) + ": " + cudaGetErrorString(e);
                for (int k = 0; k < cnt; ++k) srv_mark_failed(*g[k], st, QSG_ERR_CUDA, msg);
                continue;
            }
            for (int k = 0; k < cnt; ++k) {
                if (cudaEventRecord(g[k]->ev, st) != cudaSuccess) {
                    srv_mark_failed(*g[k], st, QSG_ERR_CUDA, "cudaEventRecord failed after a resident 1D launch");
                    continue;
                }
                if (!g[k]->chunks++) g[k]->first_dispatch = clk::now();
                g[k]->dispatched += chunk;
                g[k]->in_flight = true;
                ++in_flight_now;
            }
        }
        // dispatch: stepped requests (four-step 1D, 2D), one chunk each
        for (auto &q : running) {
            if (q->in_flight || q->fail_rc || q->dispatched >= q->req.nsteps) continue;
            if (q->req.dim == 1 && !q->inst->fourstep && !q->inst->blue) continue;
            const double sites = (double)q->inst->n;
            uint64_t chunk = (uint64_t)std::max(1.0, 1e8 / (sites * (q->req.order == 4 ? 3 : 1)));
            chunk = std::min(chunk, q->req.nsteps - q->dispatched);
            progress = true;
            int rc = q->id == S->inject_fail_id
                         ? fail(QSG_ERR_CUDA, "injected dispatch failure (QSG_SERVER_FAIL_REQUEST)")
                         : q->req.dim == 1 ? step1d(q->inst, chunk, 0) : step2d(q->inst, chunk, 0);
            if (rc) {
                srv_mark_failed(*q, q->st, rc, g_last_error);
                continue;
            }
            const cudaError_t er = cudaEventRecord(q->ev, q->st);
            if (er != cudaSuccess) {
                srv_mark_failed(*q, q->st, QSG_ERR_CUDA, std::string("cudaEventRecord: ") + cudaGetErrorString(er));
                continue;
            }
            if (!q->chunks++) q->first_dispatch = clk::now();
            q->dispatched += chunk;
            q->inst->steps += chunk;
            q->in_flight = true;
            ++in_flight_now;
        }
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->max_in_flight = std::max(S->max_in_flight, in_flight_now);
        }
        clk_ctx.unlock();
        if (!progress) std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
    // shut down: wait for the device, release everything still held
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaDeviceSynchronize();
    for (auto &q : running) srv_finish(S, *q, QSG_ERR_STATE, "server stopped");
    for (auto &q : pending) srv_finish(S, *q, QSG_ERR_STATE, "server stopped");
    for (auto &u : ring_uses) cudaEventDestroy(u.ev);
    for (cudaEvent_t e : ring_ev_pool) cudaEventDestroy(e);
}

}  // namespace

extern "C" {

int qsg_server_create(int device_ordinal, size_t hbm_budget_bytes, int max_running, qsg_server **out)
{
    if (!out) return fail(QSG_ERR_ARG, "qsg_server_create: out is null");
    *out = nullptr;
    qsg_ctx *ctx = nullptr;
    int rc = qsg_init(device_ordinal, hbm_budget_bytes, &ctx);
    if (rc) return rc;
    qsg_server *S = new qsg_server();
    S->ctx = ctx;
    if (max_running > 0) S->max_running = max_running;
    if (const char *rs = std::getenv("QSG_SERVER_RING")) {
        const long v = std::strtol(rs, nullptr, 10);
        if (v >= 1 && v <= (1 << 20)) S->ring_size = (int)v;
    }
    // a resident group (at most max_running requests) must fit the ring
    S->ring_size = std::max(S->ring_size, S->max_running);
    for (int i = 0; i < 8; ++i) {
        cudaStream_t st;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) break;
        S->streams.push_back(st);
    }
    void *p = nullptr, *ph = nullptr;
    if (S->streams.empty() || cudaMalloc(&p, sizeof(qsg::FsInst) * S->ring_size) != cudaSuccess ||
        cudaMallocHost(&ph, sizeof(qsg::FsInst) * S->ring_size) != cudaSuccess) {
        for (auto st : S->streams) cudaStreamDestroy(st);
        qsg_ctx_destroy(ctx);
        delete S;
        return fail(QSG_ERR_CUDA, "qsg_server_create: stream / descriptor allocation failed");
    }
    S->ring = static_cast<qsg::FsInst *>(p);
    S->ring_host = static_cast<qsg::FsInst *>(ph);
    if (const char *inj = std::getenv("QSG_SERVER_FAIL_REQUEST")) S->inject_fail_id = std::strtoull(inj, nullptr, 10);
    S->th = std::thread(srv_loop, S);
    *out = S;
    return QSG_OK;
}

int qsg_server_submit(qsg_server *S, const qsg_request *r, uint64_t *id)
{
    if (!S || !r || (!r->spec && (!r->psi0 || !r->V))) return fail(QSG_ERR_ARG, "qsg_server_submit: null argument");
    if (r->spec) {
        const int rc = check_spec(r->spec, "qsg_server_submit");
        if (rc) return rc;
    }
    if ((r->dim != 1 && r->dim != 2) || (r->order != 2 && r->order != 4) || r->nx == 0 ||
        (r->dim == 2 && r->ny == 0) || r->nsteps == 0)
        return fail(QSG_ERR_ARG, "qsg_server_submit: bad request (dim, order, sizes or steps)");
    if (S->ctx->budget && request_bytes(*r) > S->ctx->budget)
        return fail(QSG_ERR_BUDGET, "qsg_server_submit: request larger than the server's HBM budget");
    auto q = std::make_shared<SrvRequest>();
    q->req = *r;
    const size_t n = (size_t)r->nx * (r->dim == 2 ? r->ny : 1);
    if (r->spec) {
        q->spec = *r->spec;
        q->has_spec = true;
    } else {
        q->psi0.assign(r->psi0, r->psi0 + 2 * n);
        q->V.assign(r->V, r->V + n);
    }
    q->req.psi0 = nullptr;
    q->req.V = nullptr;
    q->req.spec = nullptr;
    q->submit = clk::now();
    std::lock_guard<std::mutex> lk(S->mu);
    q->id = S->next_id++;
    S->all[q->id] = q;
    S->incoming.push_back(q);
    if (id) *id = q->id;
    S->cv.notify_all();
    return QSG_OK;
}

int qsg_server_poll(qsg_server *S, uint64_t id, int *state)
{
    if (!S || !state) return fail(QSG_ERR_ARG, "qsg_server_poll: null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->all.find(id);
    if (it == S->all.end()) return fail(QSG_ERR_ARG, "qsg_server_poll: unknown request id");
    *state = it->second->state;
    return QSG_OK;
}

int qsg_server_wait(qsg_server *S, uint64_t id, double timeout_s, int *state)
{
    if (!S) return fail(QSG_ERR_ARG, "qsg_server_wait: null server");
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->all.find(id);
    if (it == S->all.end()) return fail(QSG_ERR_ARG, "qsg_server_wait: unknown request id");
    auto q = it->second;
    const auto until = clk::now() + std::chrono::duration_cast<clk::duration>(std::chrono::duration<double>(timeout_s));
    while (q->state < 2) {
        if (S->cv.wait_until(lk, until) == std::cv_status::timeout && q->state < 2) {
            if (state) *state = q->state;
            return fail(QSG_ERR_TIMEOUT, "qsg_server_wait: timed out");
        }
    }
    if (state) *state = q->state;
    return QSG_OK;
}

int qsg_server_take(qsg_server *S, uint64_t id, double *psi_out, double *latency_s)
{
    if (!S) return fail(QSG_ERR_ARG, "qsg_server_take: null server");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->all.find(id);
    if (it == S->all.end()) return fail(QSG_ERR_ARG, "qsg_server_take: unknown request id");
    auto q = it->second;
    if (q->state < 2) return fail(QSG_ERR_STATE, "qsg_server_take: request not finished");
    if (latency_s) *latency_s = std::chrono::duration<double>(q->finish - q->submit).count();
    const int err = q->error;
    const std::string msg = q->message;
    if (!err && psi_out) std::memcpy(psi_out, q->result.data(), q->result.size() * sizeof(double));
    S->all.erase(it);
    if (err) return fail(err, msg);
    return QSG_OK;
}

int qsg_server_stats(qsg_server *S, qsg_server_info *out)
{
    if (!S || !out) return fail(QSG_ERR_ARG, "qsg_server_stats: null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    out->completed = S->completed;
    out->failed = S->failed;
    out->site_steps = S->done_site_steps;
    out->peak_device_bytes = S->peak_bytes;
    out->budget_bytes = S->ctx->budget;
    out->admitted_mid_flight = S->admitted_mid_flight;
    out->max_in_flight = S->max_in_flight;
    return QSG_OK;
}

int qsg_server_request_info(qsg_server *S, uint64_t id, qsg_request_info *out)
{
    if (!S || !out) return fail(QSG_ERR_ARG, "qsg_server_request_info: null argument");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->all.find(id);
    if (it == S->all.end()) return fail(QSG_ERR_ARG, "qsg_server_request_info: unknown request id");
    const SrvRequest &q = *it->second;
    auto since = [&](clk::time_point t) { return std::chrono::duration<double>(t - S->t0).count(); };
    *out = qsg_request_info{};
    out->state = q.state;
    out->admitted_mid_flight = q.admitted_mid_flight ? 1 : 0;
    out->chunks = q.chunks;
    out->steps_dispatched = q.dispatched;
    out->t_submit = since(q.submit);
    out->t_admit = q.state >= 1 && q.admit != clk::time_point{} ? since(q.admit) : -1;
    out->t_first_dispatch = q.chunks ? since(q.first_dispatch) : -1;
    out->t_finish = q.state >= 2 ? since(q.finish) : -1;
    return QSG_OK;
}

void qsg_server_destroy(qsg_server *S)
{
    if (!S) return;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
        S->cv.notify_all();
    }
    if (S->th.joinable()) S->th.join();
    cudaSetDevice(S->ctx->dev);
    cudaDeviceSynchronize();
    for (auto st : S->streams) cudaStreamDestroy(st);
    cudaFree(S->ring);
    cudaFreeHost(S->ring_host);
    qsg_ctx_destroy(S->ctx);
    delete S;
}

int qsg_profile_enable(qsg_ctx *ctx, int on)
{
    if (!ctx) return fail(QSG_ERR_ARG, "qsg_profile_enable: null context");
    std::lock_guard<std::mutex> lk(ctx->mu);
    prof_drain(ctx);
    ctx->prof_stats.clear();
    ctx->prof = on == 2 ? 2 : (on != 0 ? 1 : 0);
    return QSG_OK;
}

int qsg_profile_read(qsg_ctx *ctx, int cap, const char **names, uint64_t *launches, double *total_ms)
{
    if (!ctx) return fail(QSG_ERR_ARG, "qsg_profile_read: null context");
    std::lock_guard<std::mutex> lk(ctx->mu);
    prof_drain(ctx);
    ctx->prof_names.clear();
    for (auto &kv : ctx->prof_stats) ctx->prof_names.push_back(kv.first);
    int i = 0;
    for (auto &kv : ctx->prof_stats) {
        if (i < cap) {
            if (names) names[i] = ctx->prof_names[i].c_str();
            if (launches) launches[i] = kv.second.launches;
            if (total_ms) total_ms[i] = kv.second.total_ms;
        }
        ++i;
    }
    return i;
}

}  // extern "C"

namespace qsg {

PlanRT::PlanRT(int L_, int E_) : L(L_), E(E_)
{
    auto lg = [](int v) {
        int r = 0;
        while ((1 << r) < v) ++r;
        return r;
    };
    const int logl = lg(L), le = lg(E);
    loge = le;
    nst = (logl + le - 1) / le;
    logr0 = logl - (nst - 1) * le;
}

int PlanRT::tw_size() const
{
    int off = 0;
    for (int s = 1; s < nst; ++s) off += ((1 << radix_log(s)) - 1) * (1 << p_log(s));
    return off;
}

}  // namespace qsg

int qsg::set_last_error(int code, const std::string &msg) { return fail(code, msg); }
