// qsg_launch.h -- host-side launchers for the kernel templates.  Each picks
// the compiled instantiation for the runtime sizes; sizes with no
// instantiation return cudaErrorNotSupported (surfaced as QSG_ERR_UNSUPPORTED).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "qsg_kernels.cuh"

namespace qsg {

// elements per thread of every line transform, per precision (0 fp64, 1 mixed)
inline int elems_per_thread(int prec) { return prec == 1 ? 16 : 8; }

// 1D resident evolver: supported n (power of two)
bool evolve1d_supported(int prec, uint64_t n);
cudaError_t launch_evolve1d(int prec, int n, const Evolve1DArgs &a, cudaStream_t st);

// 2D geometry chosen for a grid
struct Geom2D {
    int nx, ny, g, m;   // x split: nx = g * m
    int row_b;          // row groups per CTA
    int row_threads, row_blocks;
    size_t row_smem;
    int col_w, col_threads;
    size_t col_smem;
};
bool geom2d(int prec, int nx, int ny, Geom2D *g);
cudaError_t launch_row_pass(int prec, const Geom2D &g, bool in_split, bool out_split,
                            const RowPassArgs &a, cudaStream_t st);
cudaError_t launch_col_pass(int prec, const Geom2D &g, const ColPassArgs &a, cudaStream_t st);
// forward transform of the column pass with the kinetic-energy reduction
cudaError_t launch_col_kinetic(int prec, const Geom2D &g, const ColPassArgs &a, double dtx,
                               double dty, double *partials, cudaStream_t st);
// 1D forward transform with the kinetic-energy reduction (one CTA)
cudaError_t launch_kinetic1d(int prec, int n, const void *psi, const void *tw, double dt_k,
                             double *sums, cudaStream_t st);

// runtime mirror of Plan<L, E>: stage-major twiddle layout
struct PlanRT {
    int L, E, nst, logr0, loge;
    PlanRT(int L_, int E_);
    int radix_log(int s) const { return s == 0 ? logr0 : loge; }
    int p_log(int s) const { return s == 0 ? 0 : logr0 + (s - 1) * loge; }
    int tw_size() const;
};

}  // namespace qsg
