// 1D evolution: batched resident kernel, four-step passes, kinetic transforms.
#include "qsg_dispatch.cuh"

namespace qsg {

// Resident: n <= 8192 (complex64) / 4096 (complex128); several instances per
// CTA while a line has fewer than 256 threads.
bool evolve1d_supported(int prec, uint64_t n)
{
    if (n < 64 || (n & (n - 1))) return false;
    return prec == 1 ? n <= 8192 : n <= 4096;
}
constexpr int res_ni_for(int l, int e) { return (256 / (l / e)) > 1 ? 256 / (l / e) : 1; }

template <class T, int L>
static cudaError_t run_evolve1d(const Evolve1DBatchArgs &a, cudaStream_t st)
{
    constexpr int E = sizeof(T) == 4 ? 16 : 8;
    constexpr int PADS = sizeof(T) == 4 ? 4 : 3;
    constexpr int NI = res_ni_for(L, E);
    const size_t smem = sizeof(cplx_t<T>) * padded<L, PADS>(L) * NI;
    auto k = k_evolve1d_resident<T, L, E, NI>;
    cudaError_t e = prepare_smem(k, smem);
    if (e != cudaSuccess) return e;
    k<<<(a.count + NI - 1) / NI, NI * (L / E), smem, st>>>(a);
    return cudaGetLastError();
}

template <class T, int L>
static cudaError_t run_kinetic1d(const void *psi, const void *tw, double dtk, double *sums,
                                 cudaStream_t st)
{
    constexpr int E = sizeof(T) == 4 ? 16 : 8;
    constexpr int PADS = sizeof(T) == 4 ? 4 : 3;
    const size_t smem = sizeof(cplx_t<T>) * padded<L, PADS>(L);
    cudaError_t e = prepare_smem(k_kinetic1d<T, L, E>, smem);
    if (e != cudaSuccess) return e;
    k_kinetic1d<T, L, E><<<1, L / E, smem, st>>>(psi, tw, dtk, sums);
    return cudaGetLastError();
}

// The queue kernel (complex64): tiles of QT = 8192 sites, the largest
// resident length, QT / E = 512 threads per CTA.  complex128 batches keep one
// launch per size class (its instantiation over lengths 1024 .. 4096 spilled).
int queue_tile_sites(int prec) { return prec == 1 ? 8192 : 0; }

template <class T, int QT>
static cudaError_t run_queue(const Evolve1DQueueArgs &a, cudaStream_t st)
{
    constexpr int E = sizeof(T) == 4 ? 16 : 8;
    constexpr int PADS = sizeof(T) == 4 ? 4 : 3;
    const size_t smem = sizeof(cplx_t<T>) * padded<QT, PADS>(QT);
    auto k = k_evolve1d_queue<T, QT, E>;
    cudaError_t e = prepare_smem(k, smem);
    if (e != cudaSuccess) return e;
    static int occ = 0;
    k<<<persistent_grid(k, QT / E, smem, a.ntiles, occ), QT / E, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_evolve1d_queue(int prec, const Evolve1DQueueArgs &a, cudaStream_t st)
{
    if (a.ntiles <= 0) return cudaSuccess;
    if (prec != 1) return cudaErrorNotSupported;
    return run_queue<float, 8192>(a, st);
}

#define QSG_1D_CASES(X, T) \
    X(T, 64) X(T, 128) X(T, 256) X(T, 512) X(T, 1024) X(T, 2048) X(T, 4096)

cudaError_t launch_evolve1d(int prec, int n, const Evolve1DBatchArgs &a, cudaStream_t st)
{
#define X(T, L) case L: return run_evolve1d<T, L>(a, st);
    if (prec == 1) {
        switch (n) { QSG_1D_CASES(X, float) X(float, 8192) default: break; }
    } else {
        switch (n) { QSG_1D_CASES(X, double) default: break; }
    }
#undef X
    return cudaErrorNotSupported;
}

cudaError_t launch_kinetic1d(int prec, int n, const void *psi, const void *tw, double dtk,
                             double *sums, cudaStream_t st)
{
#define X(T, L) case L: return run_kinetic1d<T, L>(psi, tw, dtk, sums, st);
    if (prec == 1) {
        switch (n) { QSG_1D_CASES(X, float) X(float, 8192) default: break; }
    } else {
        switch (n) { QSG_1D_CASES(X, double) default: break; }
    }
#undef X
    return cudaErrorNotSupported;
}

// ---------------------------------------------------------------------------
// infinite wall: a 2n line per CTA, 2n <= 8192 (complex64) / 4096 (complex128)
// ---------------------------------------------------------------------------

bool wall1d_supported(int prec, uint64_t n)
{
    if (n < 64 || (n & (n - 1))) return false;
    return prec == 1 ? 2 * n <= 8192 : 2 * n <= 4096;
}

template <class T, int L2>
static cudaError_t run_wall(const Evolve1DBatchArgs &a, cudaStream_t st)
{
    constexpr int E = sizeof(T) == 4 ? 16 : 8;
    constexpr int PADS = sizeof(T) == 4 ? 4 : 3;
    const size_t smem = sizeof(cplx_t<T>) * padded<L2, PADS>(L2);
    auto k = k_evolve1d_wall<T, L2, E>;
    cudaError_t e = prepare_smem(k, smem);
    if (e != cudaSuccess) return e;
    k<<<a.count, L2 / E, smem, st>>>(a);
    return cudaGetLastError();
}

template <class T, int L2>
static cudaError_t run_wallkin(const void *psi, const void *tw, double dtk, double *sums, cudaStream_t st)
{
    constexpr int E = sizeof(T) == 4 ? 16 : 8;
    constexpr int PADS = sizeof(T) == 4 ? 4 : 3;
    const size_t smem = sizeof(cplx_t<T>) * padded<L2, PADS>(L2);
    auto k = k_kinetic1d_wall<T, L2, E>;
    cudaError_t e = prepare_smem(k, smem);
    if (e != cudaSuccess) return e;
    k<<<1, L2 / E, smem, st>>>(psi, tw, dtk, sums);
    return cudaGetLastError();
}

cudaError_t launch_wall1d(int prec, int n, const Evolve1DBatchArgs &a, cudaStream_t st)
{
#define X(T, L) case L / 2: return run_wall<T, L>(a, st);
    if (prec == 1) {
        switch (n) { QSG_1D_CASES(X, float) X(float, 8192) default: break; }
    } else {
        switch (n) { QSG_1D_CASES(X, double) default: break; }
    }
#undef X
    return cudaErrorNotSupported;
}

cudaError_t launch_kinetic1d_wall(int prec, int n, const void *psi, const void *tw, double dtk, double *sums,
                                  cudaStream_t st)
{
#define X(T, L) case L / 2: return run_wallkin<T, L>(psi, tw, dtk, sums, st);
    if (prec == 1) {
        switch (n) { QSG_1D_CASES(X, float) X(float, 8192) default: break; }
    } else {
        switch (n) { QSG_1D_CASES(X, double) default: break; }
    }
#undef X
    return cudaErrorNotSupported;
}

// ---------------------------------------------------------------------------
// four-step geometry: n = n1 * n2 (8192 .. 8388608), n1 (row, contiguous) 64 ..
// 4096 and n2 (column) 64 .. 2048; by default n1 = n2 or 2*n2, or n2 = 1024
// where that would make n2 2048 (a column pass of 2048-point columns takes two
// columns per CTA: 16-byte row segments, half a memory sector)
// ---------------------------------------------------------------------------

constexpr int fs_col_w(int prec, int n2) { return prec == 1 ? 4096 / n2 : 2048 / n2; }   // W*n2/E = 256
constexpr int fs_row_b(int prec, int n1)   // B*n1/E = 256 (512 for complex128 rows of 4096)
{
    return prec == 1 ? 4096 / n1 : (n1 >= 2048 ? 1 : 2048 / n1);
}

int fs_default_n1(uint64_t n)
{
    int lg = 0;
    while ((1ull << lg) < n) ++lg;
    const uint64_t n1 = n >> (lg / 2);
    return (int)(n / n1 > 1024 && n / 1024 <= 4096 ? n / 1024 : n1);
}

bool fs_geom(int prec, uint64_t n, FsGeom *g, int n1)
{
    if ((n & (n - 1)) || n < 8192 || n > 8388608) return false;
    if (n1 == 0) n1 = fs_default_n1(n);
    if (n1 < 64 || n1 > 4096 || (n1 & (n1 - 1)) || n % (uint64_t)n1) return false;
    const uint64_t n2 = n / (uint64_t)n1;
    if (n2 < 64 || n2 > 2048) return false;
    g->n = (int)n;
    g->n2 = (int)n2;
    g->n1 = n1;
    const int E = prec == 1 ? 16 : 8;
    const int csz = prec == 1 ? 8 : 16;
    g->col_e = E;
    g->col_w = fs_col_w(prec, g->n2);
    g->col_threads = g->col_w * (g->n2 / E);
    g->col_blocks = g->n1 / g->col_w;
    g->col_smem = (size_t)csz * col_tile_elems(csz, g->n2, g->col_w);
    g->row_e = E;
    g->row_b = fs_row_b(prec, g->n1);
    g->row_threads = g->row_b * (g->n1 / E);
    g->row_blocks = g->n2 / g->row_b;
    const int pads = prec == 1 ? 4 : 3;
    g->row_smem = (size_t)csz * g->row_b * (g->n1 + (g->n1 >> pads));
    return g->col_blocks >= 1 && g->row_blocks >= 1;
}

template <class T, int N2>
static cudaError_t run_fs_col(const FsGeom &g, const FsColArgs &a, int ninst, cudaStream_t st)
{
    constexpr int P = sizeof(T) == 4 ? 1 : 0;
    constexpr int E = P ? 16 : 8;
    constexpr int W = fs_col_w(P, N2);
    auto k = k_fs_col<T, N2, E, W>;
    cudaError_t e = prepare_smem(k, g.col_smem);
    if (e != cudaSuccess) return e;
    k<<<dim3(g.col_blocks, ninst), W * (N2 / E), g.col_smem, st>>>(a);
    return cudaGetLastError();
}

template <class T, int N1>
static cudaError_t run_fs_row(const FsGeom &g, const FsRowArgs &a, int ninst, cudaStream_t st)
{
    constexpr int P = sizeof(T) == 4 ? 1 : 0;
    constexpr int E = P ? 16 : 8;
    constexpr int B = fs_row_b(P, N1);
    auto k = k_fs_row<T, N1, E, B>;
    cudaError_t e = prepare_smem(k, g.row_smem);
    if (e != cudaSuccess) return e;
    k<<<dim3(g.row_blocks, ninst), B * (N1 / E), g.row_smem, st>>>(a);
    return cudaGetLastError();
}

template <class T, int N1>
static cudaError_t run_fs_rowkin(const FsGeom &g, const FsRowArgs &a, double dtk, double *partials,
                                 cudaStream_t st)
{
    constexpr int P = sizeof(T) == 4 ? 1 : 0;
    constexpr int E = P ? 16 : 8;
    constexpr int B = fs_row_b(P, N1);
    auto k = k_fs_row_kinetic<T, N1, E, B>;
    cudaError_t e = prepare_smem(k, g.row_smem);
    if (e != cudaSuccess) return e;
    k<<<g.row_blocks, B * (N1 / E), g.row_smem, st>>>(a, g.n2, dtk, partials);
    return cudaGetLastError();
}

#define QSG_FS_N(X, T) X(T, 64) X(T, 128) X(T, 256) X(T, 512) X(T, 1024) X(T, 2048) X(T, 4096)
#define QSG_FS_N2(X, T) X(T, 64) X(T, 128) X(T, 256) X(T, 512) X(T, 1024) X(T, 2048)

cudaError_t launch_fs_col(int prec, const FsGeom &g, const FsColArgs &a, int ninst, cudaStream_t st)
{
#define X(T, N2) case N2: return run_fs_col<T, N2>(g, a, ninst, st);
    if (prec == 1) {
        switch (g.n2) { QSG_FS_N2(X, float) default: break; }
    } else {
        switch (g.n2) { QSG_FS_N2(X, double) default: break; }
    }
#undef X
    return cudaErrorNotSupported;
}

cudaError_t launch_fs_row(int prec, const FsGeom &g, const FsRowArgs &a, int ninst, cudaStream_t st)
{
#define X(T, N1) case N1: return run_fs_row<T, N1>(g, a, ninst, st);
    if (prec == 1) {
        switch (g.n1) { QSG_FS_N(X, float) default: break; }
    } else {
        switch (g.n1) { QSG_FS_N(X, double) default: break; }
    }
#undef X
    return cudaErrorNotSupported;
}

cudaError_t launch_fs_row_kinetic(int prec, const FsGeom &g, const FsRowArgs &a, double dtk,
                                  double *partials, cudaStream_t st)
{
#define X(T, N1) case N1: return run_fs_rowkin<T, N1>(g, a, dtk, partials, st);
    if (prec == 1) {
        switch (g.n1) { QSG_FS_N(X, float) default: break; }
    } else {
        switch (g.n1) { QSG_FS_N(X, double) default: break; }
    }
#undef X
    return cudaErrorNotSupported;
}

}  // namespace qsg
