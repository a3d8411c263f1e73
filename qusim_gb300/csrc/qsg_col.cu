// 2D column passes: instantiations + launchers.
#include "qsg_dispatch.cuh"

namespace qsg {

template <class T, int M>
static cudaError_t run_col(const Geom2D &g, const ColPassArgs &a, cudaStream_t st)
{
    constexpr int E = sizeof(T) == 4 ? 16 : 8;
    constexpr int W = col_w_for(M, E, sizeof(T) == 4 ? 1 : 0);
    auto k = k_col_pass<T, M, E, W>;
    cudaError_t e = prepare_smem(k, g.col_smem);
    if (e != cudaSuccess) return e;
    dim3 grid(g.ny / W, g.g);
    k<<<grid, W * (M / E), g.col_smem, st>>>(a);
    return cudaGetLastError();
}

template <class T, int M>
static cudaError_t run_colkin(const Geom2D &g, const ColPassArgs &a, double dtx, double dty,
                              double *partials, cudaStream_t st)
{
    constexpr int E = sizeof(T) == 4 ? 16 : 8;
    constexpr int W = col_w_for(M, E, sizeof(T) == 4 ? 1 : 0);
    auto k = k_col_kinetic<T, M, E, W>;
    cudaError_t e = prepare_smem(k, g.col_smem);
    if (e != cudaSuccess) return e;
    dim3 grid(g.ny / W, g.g);
    k<<<grid, W * (M / E), g.col_smem, st>>>(a, dtx, dty, partials);
    return cudaGetLastError();
}

#define QSG_M_CASES(X, T) X(T, 128) X(T, 256) X(T, 512) X(T, 1024)

cudaError_t launch_col_pass(int prec, const Geom2D &g, const ColPassArgs &a, cudaStream_t st)
{
#define X(T, M) case M: return run_col<T, M>(g, a, st);
    if (prec == 1) {
        switch (g.m) { QSG_M_CASES(X, float) default: break; }
    } else {
        switch (g.m) { QSG_M_CASES(X, double) X(double, 2048) default: break; }
    }
#undef X
    return cudaErrorNotSupported;
}

cudaError_t launch_col_kinetic(int prec, const Geom2D &g, const ColPassArgs &a, double dtx,
                               double dty, double *partials, cudaStream_t st)
{
#define X(T, M) case M: return run_colkin<T, M>(g, a, dtx, dty, partials, st);
    if (prec == 1) {
        switch (g.m) { QSG_M_CASES(X, float) default: break; }
    } else {
        switch (g.m) { QSG_M_CASES(X, double) X(double, 2048) default: break; }
    }
#undef X
    return cudaErrorNotSupported;
}

cudaError_t launch_row_pass_f32(const Geom2D &, bool, bool, const RowPassArgs &, cudaStream_t);
cudaError_t launch_row_pass_f64(const Geom2D &, bool, bool, const RowPassArgs &, cudaStream_t);

cudaError_t launch_row_pass(int prec, const Geom2D &g, bool in_split, bool out_split,
                            const RowPassArgs &a, cudaStream_t st)
{
    return prec == 1 ? launch_row_pass_f32(g, in_split, out_split, a, st)
                     : launch_row_pass_f64(g, in_split, out_split, a, st);
}

bool geom2d(int prec, int nx, int ny, Geom2D *g)
{
    auto pow2 = [](int v) { return v > 0 && (v & (v - 1)) == 0; };
    if (!pow2(nx) || !pow2(ny) || ny < 128 || ny > 4096 || nx < 128 || nx > 4096) return false;
    const int E = elems_per_thread(prec);
    const int csz = prec == 1 ? 8 : 16;
    const int pads = prec == 1 ? 4 : 3;
    g->nx = nx;
    g->ny = ny;
    g->g = split_g_for(prec, nx);
    g->m = nx / g->g;
    g->row_b = row_b_for(ny, E, g->g);
    const int rs = row_rs_for(ny, E, g->g);
    g->row_threads = g->row_b * g->g * (ny / E) / rs;
    if (g->m % g->row_b) return false;
    g->row_blocks = g->m / g->row_b;
    g->row_smem = (size_t)csz * g->row_b * g->g * (ny + (ny >> pads));
    g->col_w = col_w_for(g->m, E, prec);
    if (ny % g->col_w) return false;
    g->col_threads = g->col_w * (g->m / E);
    g->col_smem = (size_t)csz * col_tile_elems(csz, g->m, g->col_w);
    return g->row_threads <= 512 && g->col_threads <= 512 && g->row_smem <= 200 * 1024 &&
           g->col_smem <= 200 * 1024;
}

}  // namespace qsg
