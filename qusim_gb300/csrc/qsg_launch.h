// qsg_launch.h -- host-side launchers for the kernel templates.  Each picks
// the compiled instantiation for the runtime sizes; sizes with no
// instantiation return cudaErrorNotSupported (surfaced as QSG_ERR_UNSUPPORTED).
#pragma once
#include <complex>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include <stdint.h>
#include "qsg_kernels.cuh"

namespace qsg {

// elements per thread of the 1D resident transforms and of the default plans,
// per precision (0 fp64, 1 mixed)
inline int elems_per_thread(int prec) { return prec == 1 ? 16 : 8; }

// 1D resident evolver: supported n (power of two); a.count instances
bool evolve1d_supported(int prec, uint64_t n);
cudaError_t launch_evolve1d(int prec, int n, const Evolve1DBatchArgs &a, cudaStream_t st);

// 1D resident evolver, every resident size in one persistent launch fed by a
// tile queue (k_evolve1d_queue): sites per tile, and the launch
int queue_tile_sites(int prec);
cudaError_t launch_evolve1d_queue(int prec, const Evolve1DQueueArgs &a, cudaStream_t st);

// 1D periodic evolution of a length that is not a power of two (Bluestein,
// qsg_blue.cuh): the transform length M for n (0: unsupported), the chirp w
// and FFT_M(conj chirp) / M in long double, the launches
struct BlueArgs;
int blue_m_for(int prec, uint64_t n);
int blue_elems(int prec);
void blue_tables(uint64_t n, int m, std::vector<std::complex<long double>> &w,
                 std::vector<std::complex<long double>> &hs);
// the same tables for the long buffers of the four-step passes (m up to 2^22),
// computed in double-double arithmetic on host threads and rounded to double
void blue_tables_dd(uint64_t n, uint64_t m, std::vector<std::complex<double>> &w,
                    std::vector<std::complex<double>> &hs);
cudaError_t launch_evolve1d_blue(int prec, int m, const BlueArgs &a, cudaStream_t st);
cudaError_t launch_kinetic1d_blue(int prec, int m, const BlueArgs &a, double dtk, double *sums, cudaStream_t st);
// 2D grids with a side that is not a power of two: row pass (rows of ny), column pass
// (columns of nx; with kinetic, the forward transform and the kinetic-energy partials)
struct Blue2DArgs;
int blue_rows_per_cta(int prec, int m);
int blue_cols_per_cta(int prec, int m);
cudaError_t launch_row_blue(int prec, int m, const Blue2DArgs &a, cudaStream_t st);
cudaError_t launch_col_blue(int prec, int m, const Blue2DArgs &a, bool kinetic, double dtx, double dty,
                            double *partials, cudaStream_t st);

// psi0 / V from expressions in the reference calculator's language (qsg_expr.cu):
// compile both and sample them into psi (nx ny complex128) and V (real) on st
int sample_expr(int dim, const char *psi_expr, const char *v_expr, int nx, int ny, double x0, double y0, double dx,
                double dy, void *psi, double *V, cudaStream_t st, std::string &err);

// 1D infinite wall (2n line per CTA)
bool wall1d_supported(int prec, uint64_t n);
cudaError_t launch_wall1d(int prec, int n, const Evolve1DBatchArgs &a, cudaStream_t st);
cudaError_t launch_kinetic1d_wall(int prec, int n, const void *psi, const void *tw, double dtk, double *sums,
                                  cudaStream_t st);

// 1D four-step geometry (n = n1 * n2, 2^13 .. 2^23; n1 in 64 .. 4096, n2 in
// 64 .. 2048) and passes over ninst instances
struct FsGeom {
    int n, n1, n2;
    int col_e, col_w, col_threads, col_blocks;
    size_t col_smem;
    int row_e, row_b, row_threads, row_blocks;
    size_t row_smem;
};
// n1 = 0: the default split (n1 = n2 or 2 n2; 4096 x 1024 for 2^22)
bool fs_geom(int prec, uint64_t n, FsGeom *g, int n1 = 0);
int fs_default_n1(uint64_t n);
cudaError_t launch_fs_col(int prec, const FsGeom &g, const FsColArgs &a, int ninst, cudaStream_t st);
cudaError_t launch_fs_row(int prec, const FsGeom &g, const FsRowArgs &a, int ninst, cudaStream_t st);
cudaError_t launch_fs_row_kinetic(int prec, const FsGeom &g, const FsRowArgs &a, double dtk,
                                  double *partials, cudaStream_t st);

// A 2D plan: the x split and the kernel variants of the two passes.
struct Plan2D {
    int g;          // x split: Nx = g * m, column transforms of length m
    int row_e;      // elements per thread of the row transforms (radix)
    int row_nt;     // threads per row-pass CTA (256 or 512)
    int col_e;      // elements per thread of the column transforms
    int col_w;      // adjacent columns per column-pass CTA
    int row_kind = 0;  // 0: k_row_pass (unit staged in shared memory); 1: k_row_pass_tm (lines parked in TMEM)
};

// Launch geometry of a plan for a grid
struct Geom2D {
    int nx, ny, g, m;
    int row_kind;
    int row_e, row_b, row_rs, row_threads, row_blocks;
    size_t row_smem;
    int col_e, col_w, col_threads;
    size_t col_smem;
    int kin_e, kin_w, kin_threads;  // kinetic-energy column transform
    size_t kin_smem;
};
// Valid (compiled, fits the SM) geometry for the plan?
bool geom2d(int prec, int nx, int ny, const Plan2D &p, Geom2D *g);
// Plans compiled for this grid (up to cap); returns the count.
int candidate_plans(int prec, int nx, int ny, Plan2D *out, int cap);
// The plan used when no tuned plan is known.
bool default_plan(int prec, int nx, int ny, Plan2D *p);

cudaError_t launch_row_pass(int prec, const Geom2D &g, const RowPassArgs &a, cudaStream_t st);
// TMEM row pass (complex64, g = 4, ny = 2048 / 4096)
bool row_tm_supported(int ny, int g);
cudaError_t launch_row_pass_tm(const Geom2D &g, const RowPassArgs &a, cudaStream_t st);
cudaError_t launch_col_pass(int prec, const Geom2D &g, const ColPassArgs &a, cudaStream_t st);
// forward column transform with the kinetic-energy reduction (uses kin_* geometry)
cudaError_t launch_col_kinetic(int prec, const Geom2D &g, const ColPassArgs &a, double dtx,
                               double dty, double *partials, cudaStream_t st);
// 1D forward transform with the kinetic-energy reduction (one CTA)
cudaError_t launch_kinetic1d(int prec, int n, const void *psi, const void *tw, double dt_k,
                             double *sums, cudaStream_t st);

// 3D split-operator passes (qsg_evolve3d.cuh)
struct Pass3Args;
bool evolve3d_supported(int prec, uint64_t nx, uint64_t ny, uint64_t nz);
int row3_ctas(int prec, int l, size_t lines);
int col3_ctas(int prec, int l, int inner, int outer);
template <class T> cudaError_t launch3_row(int l, size_t lines, const Pass3Args &a, cudaStream_t st);
template <class T> cudaError_t launch3_col(int l, int inner, int outer, const Pass3Args &a, cudaStream_t st);

// a row-major buffer of outer x inner 8-byte elements as a 2D tensor map
// (CUtensorMap, 128 bytes at out) with boxes of box_inner x box_outer; false
// when the driver entry point is missing or a TMA rule (16-byte base, strides
// and box rows; boxes of at most 256) would be broken
bool encode_2d_map(void *base, uint64_t inner, uint64_t outer, uint32_t box_inner, uint32_t box_outer, void *out);

// 1D four-step column pass fed by tensor copies (qsg_fs_tma.cuh, complex64):
// supported column lengths, one instance buffer's tensor map (128 bytes at
// out, 64-byte aligned) and the launch (a.maps: 3 maps per instance)
bool fs_tma_supported(int prec, int n2);
bool encode_fs_map(void *base, int n1, int n2, void *out);
cudaError_t launch_fs_col_tma(const FsGeom &g, const FsColArgs &a, cudaStream_t st);

// momentum-form column pass fed by tensor copies (qsg_col_tma.cuh): compiled
// tile shapes, the two tensor maps (work buffer, state; 2 x 128 bytes, 64-byte
// aligned storage at maps) and the launch
bool col_tma_supported(int m, int e, int w);
bool encode_col_tma_maps(void *work, void *psi, int nx, int ny, int w, void *maps);
cudaError_t launch_col_pass_tma(const Geom2D &g, const ColPassArgs &a, const void *maps, cudaStream_t st);

// record `msg` as the calling thread's qsg_last_error(); returns code
int set_last_error(int code, const std::string &msg);

// runtime mirror of Plan<L, E>: stage-major twiddle layout
struct PlanRT {
    int L, E, nst, logr0, loge;
    PlanRT(int L_, int E_);
    int radix_log(int s) const { return s == 0 ? logr0 : loge; }
    int p_log(int s) const { return s == 0 ? 0 : logr0 + (s - 1) * loge; }
    int tw_size() const;
};

}  // namespace qsg
