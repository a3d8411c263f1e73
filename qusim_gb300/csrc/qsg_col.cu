// 2D column passes: instantiations, launchers, planner.
#include "qsg_dispatch.cuh"

namespace qsg {

template <class T, int M>
static cudaError_t run_colkin(const Geom2D &g, const ColPassArgs &a, double dtx, double dty,
                              double *partials, cudaStream_t st)
{
    constexpr int P = sizeof(T) == 4 ? 1 : 0;
    constexpr int E = kin_e_for(P);
    constexpr int W = kin_w_for(P, M);
    auto k = k_col_kinetic<T, M, E, W>;
    cudaError_t e = prepare_smem(k, g.kin_smem);
    if (e != cudaSuccess) return e;
    dim3 grid(g.ny / W, g.g);
    k<<<grid, W * (M / E), g.kin_smem, st>>>(a, dtx, dty, partials);
    return cudaGetLastError();
}

static bool col_variant_exists(int prec, int m, int e, int w)
{
#define C(T, M, E, W) \
    if (m == M && e == E && w == W) return true;
    if (prec == 1) {
        QSG_COL_VARIANTS_F32(C)
    } else {
        QSG_COL_VARIANTS_F64(C)
    }
#undef C
    return false;
}

template <bool PL> cudaError_t launch_col_pass_f32_t(const Geom2D &, const ColPassArgs &, cudaStream_t);
extern template cudaError_t launch_col_pass_f32_t<false>(const Geom2D &, const ColPassArgs &, cudaStream_t);
extern template cudaError_t launch_col_pass_f32_t<true>(const Geom2D &, const ColPassArgs &, cudaStream_t);
cudaError_t launch_col_pass_f64(const Geom2D &, const ColPassArgs &, cudaStream_t);

cudaError_t launch_col_pass(int prec, const Geom2D &g, const ColPassArgs &a, cudaStream_t st)
{
    if (prec != 1) return launch_col_pass_f64(g, a, st);
    return a.plain ? launch_col_pass_f32_t<true>(g, a, st) : launch_col_pass_f32_t<false>(g, a, st);
}

#define QSG_M_CASES(X, T) X(T, 128) X(T, 256) X(T, 512) X(T, 1024) X(T, 2048)

cudaError_t launch_col_kinetic(int prec, const Geom2D &g, const ColPassArgs &a, double dtx,
                               double dty, double *partials, cudaStream_t st)
{
#define X(T, M) case M: return run_colkin<T, M>(g, a, dtx, dty, partials, st);
    if (prec == 1) {
        switch (g.m) { QSG_M_CASES(X, float) default: break; }
    } else {
        switch (g.m) { QSG_M_CASES(X, double) default: break; }
    }
#undef X
    return cudaErrorNotSupported;
}

template <bool PL> cudaError_t launch_row_pass_f32a_t(const Geom2D &, const RowPassArgs &, cudaStream_t);
template <bool PL> cudaError_t launch_row_pass_f32b_t(const Geom2D &, const RowPassArgs &, cudaStream_t);
extern template cudaError_t launch_row_pass_f32a_t<false>(const Geom2D &, const RowPassArgs &, cudaStream_t);
extern template cudaError_t launch_row_pass_f32a_t<true>(const Geom2D &, const RowPassArgs &, cudaStream_t);
extern template cudaError_t launch_row_pass_f32b_t<false>(const Geom2D &, const RowPassArgs &, cudaStream_t);
extern template cudaError_t launch_row_pass_f32b_t<true>(const Geom2D &, const RowPassArgs &, cudaStream_t);
cudaError_t launch_row_pass_f64(const Geom2D &, const RowPassArgs &, cudaStream_t);
bool row_variant_exists_f32a(int ny, int e, int g, int nt);
bool row_variant_exists_f32b(int ny, int e, int g, int nt);
bool row_variant_exists_f64(int ny, int e, int g, int nt);

cudaError_t launch_row_pass(int prec, const Geom2D &g, const RowPassArgs &a, cudaStream_t st)
{
    if (g.row_kind == 1) return launch_row_pass_tm(g, a, st);
    if (prec == 0) return launch_row_pass_f64(g, a, st);
    if (g.row_e == 16) return a.plain ? launch_row_pass_f32a_t<true>(g, a, st) : launch_row_pass_f32a_t<false>(g, a, st);
    return a.plain ? launch_row_pass_f32b_t<true>(g, a, st) : launch_row_pass_f32b_t<false>(g, a, st);
}

bool geom2d(int prec, int nx, int ny, const Plan2D &p, Geom2D *g)
{
    auto pow2 = [](int v) { return v > 0 && (v & (v - 1)) == 0; };
    if (!pow2(nx) || !pow2(ny) || ny < 128 || ny > 8192 || nx < 128 || nx > 8192) return false;
    if (!pow2(p.g) || p.g > 4 || nx % p.g) return false;
    const int csz = prec == 1 ? 8 : 16;
    if (p.row_kind != 0 && p.row_kind != 1) return false;
    const bool tm = p.row_kind == 1;
    const bool row_ok = tm ? (prec == 1 && row_tm_supported(ny, p.g) && p.row_e == 16 && p.row_nt == 512)
                      : prec == 1 ? (row_variant_exists_f32a(ny, p.row_e, p.g, p.row_nt) ||
                                     row_variant_exists_f32b(ny, p.row_e, p.g, p.row_nt))
                                  : row_variant_exists_f64(ny, p.row_e, p.g, p.row_nt);
    if (!row_ok) return false;
    g->row_kind = p.row_kind;
    g->nx = nx;
    g->ny = ny;
    g->g = p.g;
    g->m = nx / p.g;
    if (!col_variant_exists(prec, g->m, p.col_e, p.col_w)) return false;
    g->row_e = p.row_e;
    g->row_b = tm ? 1 : row_b_for(ny, p.row_e, p.g);
    g->row_threads = p.row_nt;
    g->row_rs = tm ? p.g : row_work_for(ny, p.row_e, p.g) / p.row_nt;
    if (g->m % g->row_b) return false;
    g->row_blocks = g->m / g->row_b;
    // the TMEM pass sizes its own shared memory (one line per thread group)
    g->row_smem = tm ? 0 : row_smem_for(csz, ny, p.row_e, p.g);
    g->col_e = p.col_e;
    g->col_w = p.col_w;
    if (ny % p.col_w) return false;
    g->col_threads = p.col_w * (g->m / p.col_e);
    g->col_smem = (size_t)csz * col_tile_elems(csz, g->m, p.col_w, p.col_e);
    g->kin_e = kin_e_for(prec);
    g->kin_w = kin_w_for(prec, g->m);
    if (ny % g->kin_w) return false;
    g->kin_threads = g->kin_w * (g->m / g->kin_e);
    g->kin_smem = (size_t)csz * col_tile_elems(csz, g->m, g->kin_w);
    const size_t smem_max = 227 * 1024 - 1024;
    return g->row_threads <= 1024 && g->col_threads <= 512 && g->kin_threads <= 512 &&
           g->row_smem <= smem_max && g->col_smem <= smem_max && g->kin_smem <= smem_max &&
           g->m >= 128 && g->m <= 2048;
}

int candidate_plans(int prec, int nx, int ny, Plan2D *out, int cap)
{
    int n = 0;
    const int es[2] = {16, 8};
    const int ces[3] = {16, 8, 32};
    const int ws[5] = {4, 8, 16, 32, 2};
    const int nts[3] = {512, 256, 1024};
    for (int g = 1; g <= 4; g *= 2)
        for (int re : es)
            for (int nt : nts)
                for (int ce : ces)
                    for (int w : ws) {
                        Plan2D p{g, re, nt, ce, w};
                        Geom2D gm;
                        if (!geom2d(prec, nx, ny, p, &gm)) continue;
                        if (n < cap) out[n] = p;
                        ++n;
                    }
    // TMEM row pass (one row per thread group in flight, the others parked in tensor memory)
    for (int ce : ces)
        for (int w : ws) {
            Plan2D p{4, 16, 512, ce, w, 1};
            Geom2D gm;
            if (!geom2d(prec, nx, ny, p, &gm)) continue;
            if (n < cap) out[n] = p;
            ++n;
        }
    return n;
}

bool default_plan(int prec, int nx, int ny, Plan2D *p)
{
    // complex64: column blocks of <= 1024 rows with 64-byte column segments
    // (radix 16); complex128: blocks of <= 2048 rows (radix 8)
    Plan2D c;
    if (prec == 1) {
        c.g = nx > 1024 ? nx / 1024 : 1;
        c.row_e = 16;
        c.row_nt = (ny >= 4096 && c.g >= 2) || (ny >= 2048 && c.g >= 4) ? 512 : 256;
        c.col_e = 16;
        const int m = nx / c.g;
        c.col_w = m >= 512 ? 8 : (m == 256 ? 16 : 32);
        // radix 32: two stages (one exchange) for 512- and 1024-point columns
        if (m == 1024) c.col_e = 32;
        if (m == 512) {
            c.col_e = 32;
            c.col_w = 16;
        }
        // rows of 2048 / 4096 points in 4-row units: waiting rows parked in TMEM
        if (c.g == 4 && row_tm_supported(ny, c.g)) {
            c.row_nt = 512;
            c.row_kind = 1;
        }
    } else {
        c.g = nx > 2048 ? nx / 2048 : 1;
        c.row_e = 8;
        c.row_nt = row_work_for(ny, 8, c.g) >= 512 ? 512 : 256;
        c.col_e = 8;
        const int m = nx / c.g;
        c.col_w = m >= 2048 ? 2 : (m >= 512 ? 4 : (m == 256 ? 8 : 16));
    }
    Geom2D g;
    if (geom2d(prec, nx, ny, c, &g)) {
        *p = c;
        return true;
    }
    Plan2D cands[64];
    const int n = candidate_plans(prec, nx, ny, cands, 64);
    if (n <= 0) return false;
    *p = cands[0];
    return true;
}

}  // namespace qsg
