// qsg_aux.h -- phase tables, reductions and format conversion (off the
// per-step path, except the renormalisation scale).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace qsg {

// out[i] = exp(f * V[i]) (fp64 tables) or exp(f * V[i]) - 1 (complex64 tables).
// f = -i dt c / hbar: SplittingMethod2D::InitExpV (src/SplittingMethod2D.cpp:38-54).
cudaError_t launch_vtable(int prec, void *out, const double *V, size_t n, double fre, double fim,
                          cudaStream_t st);
// out[i] = scale * exp(f * fold(i)^2) (fp64) or exp(f * fold(i)^2) - 1 (complex64),
// i < n; fold(i) = i > n/2 ? n - i : i (src/DeviceTemplate.h:544-547, 754-769).
cudaError_t launch_ktable1d(int prec, void *out, int n, double fre, double fim, double scale,
                            cudaStream_t st);
// infinite-wall kinetic table: scale * exp(f i^2) (fp64) or exp(f i^2) - 1 (complex64), i < n
cudaError_t launch_ktable_wall(int prec, void *out, int n, double fre, double fim, double scale, cudaStream_t st);
// four-step kinetic table in row layout: entry k2*n1 + k1 holds the factor of
// frequency k = k2 + n2*k1 (same forms as launch_ktable1d)
cudaError_t launch_ktable_fs(int prec, void *out, int n1, int n2, double fre, double fim, double scale,
                             cudaStream_t st);
// fp64 2D kinetic table: scale * exp(alpha (fold(i)^2 DTx + fold(j)^2 DTy)), index j + i*ny
// (MulExpK2D on ones, src/SplittingMethod2D.cpp:56-79, src/DeviceTemplate.h:794-819).
cudaError_t launch_ktable2d(void *out, int nx, int ny, double are, double aim, double dtx,
                            double dty, double scale, cudaStream_t st);

// psi0 (complex128) and V sampled on the device from a packet-plus-bumps
// formula (qsg_spec), point (i, j) at x0 + i*dx, y0 + j*dy, index j + i*ny
// (ny = 1 and the y terms unused in 1D)
struct SpecArgs {
    double x0, y0, dx, dy;
    double kx, ky, cx, cy, s, v0;
    int dim, nbumps;
    double bumps[32][4];
};
cudaError_t launch_sample_spec(const SpecArgs &a, int nx, int ny, void *psi, double *V, cudaStream_t st);

// host complex128 staging <-> device state
cudaError_t launch_c128_to_c64(void *out, const void *in, size_t n, cudaStream_t st);
cudaError_t launch_c64_to_c128(void *out, const void *in, size_t n, cudaStream_t st);

// Reductions over psi[lo, hi): mode 0 sum |psi|^2, 1 sum |psi|^2 V, 2 sum |psi|^2 i.
// Writes `blocks` partials; returns the number of partials via *nparts.
cudaError_t launch_reduce(int prec, const void *psi, const double *V, size_t lo, size_t hi, int mode,
                          double *partials, int max_parts, int *nparts, cudaStream_t st);
// out[k] = sum_i partials[i*stride + k], k < stride (fixed order, one block)
cudaError_t launch_finalize(const double *partials, int nparts, int stride, double *out,
                            cudaStream_t st);
// psi *= 1 / sqrt(sum[0] * dv)
cudaError_t launch_renorm(int prec, void *psi, size_t n, const double *sum, double dv,
                          cudaStream_t st);

}  // namespace qsg
