// qsg_dispatch.cuh -- variant tables and geometry rules shared by the
// instantiation units and the host planner.
#pragma once
#include "qsg_launch.h"

namespace qsg {

// Dynamic plus static shared memory above 48 KB needs the opt-in attribute;
// the kernels' static arrays (reduction scratch) stay below 1 KB.
template <class K>
static inline cudaError_t prepare_smem(K kernel, size_t smem)
{
    if (smem + 1024 > 48 * 1024)
        return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return cudaSuccess;
}

// Multiprocessors of the current device (cached per device).
static inline int sm_count()
{
    static int cache[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
    if (!cache[dev]) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = n > 0 ? n : 1;
    }
    return cache[dev];
}

// Grid of a persistent kernel: every resident CTA slot of the device, at most
// one CTA per work unit.  `occ` caches the occupancy of the instantiation.
template <class K>
static inline unsigned persistent_grid(K kernel, int threads, size_t smem, int units, int &occ)
{
    if (!occ) {
        int o = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kernel, threads, smem) != cudaSuccess || o < 1) o = 1;
        occ = o;
    }
    const long slots = (long)occ * sm_count();
    return (unsigned)(units < slots ? units : slots);
}

// Row pass: B groups of G rows per CTA so a CTA holds >= 256 threads of line
// work; the NT threads of a CTA (256 or 512) go over its NL = B*G lines in
// RS = NL*(NY/E)/NT rounds (NT >= NY/E: a line is never split across rounds).
constexpr int row_b_for(int ny, int e, int g)
{
    return (256 / (g * (ny / e))) > 1 ? 256 / (g * (ny / e)) : 1;
}
constexpr int row_work_for(int ny, int e, int g) { return row_b_for(ny, e, g) * g * (ny / e); }
constexpr size_t row_smem_for(int csz, int ny, int e, int g)
{
    return (size_t)csz * row_b_for(ny, e, g) * g * (ny + (ny >> (csz == 8 ? 4 : 3)));
}

// Instantiated variants.  X(T, NY, E, G, NT) for the row pass (NT threads),
// C(T, M, E, W) for the column pass (W*M/E threads, 128..512).
#define QSG_ROW_SMALL(X, T, E) \
    X(T, 128, E, 1, 256) X(T, 128, E, 2, 256) X(T, 128, E, 4, 256) \
    X(T, 256, E, 1, 256) X(T, 256, E, 2, 256) X(T, 256, E, 4, 256) \
    X(T, 512, E, 1, 256) X(T, 512, E, 2, 256) X(T, 512, E, 4, 256) \
    X(T, 1024, E, 1, 256) X(T, 1024, E, 2, 256) X(T, 1024, E, 4, 256)
#define QSG_ROW_VARIANTS_F32A(X) \
    QSG_ROW_SMALL(X, float, 16) \
    X(float, 2048, 16, 1, 256) X(float, 2048, 16, 2, 256) X(float, 2048, 16, 4, 256) X(float, 2048, 16, 4, 512) \
    X(float, 4096, 16, 1, 256) X(float, 4096, 16, 2, 256) X(float, 4096, 16, 2, 512) \
    X(float, 4096, 16, 4, 256) X(float, 4096, 16, 4, 512) X(float, 4096, 16, 4, 1024) \
    X(float, 8192, 16, 1, 512) X(float, 8192, 16, 2, 512) X(float, 8192, 16, 2, 1024)
#define QSG_ROW_VARIANTS_F32B(X) \
    X(float, 128, 8, 1, 256) X(float, 128, 8, 2, 256) X(float, 128, 8, 4, 256) \
    X(float, 256, 8, 1, 256) X(float, 256, 8, 2, 256) X(float, 256, 8, 4, 256) \
    X(float, 512, 8, 1, 256) X(float, 512, 8, 2, 256) X(float, 512, 8, 4, 256) \
    X(float, 1024, 8, 1, 256) X(float, 1024, 8, 2, 256) X(float, 1024, 8, 4, 256) X(float, 1024, 8, 4, 512) \
    X(float, 2048, 8, 1, 256) X(float, 2048, 8, 2, 256) X(float, 2048, 8, 2, 512) X(float, 2048, 8, 4, 512) \
    X(float, 4096, 8, 1, 512) X(float, 4096, 8, 2, 512) X(float, 4096, 8, 4, 512)
#define QSG_ROW_VARIANTS_F64(X) \
    QSG_ROW_SMALL(X, double, 8) \
    X(double, 2048, 8, 1, 256) X(double, 2048, 8, 2, 512) X(double, 2048, 8, 4, 512) \
    X(double, 4096, 8, 1, 512) X(double, 4096, 8, 2, 512)

#define QSG_COL_VARIANTS_F32(C) \
    C(float, 128, 16, 16) C(float, 128, 16, 32) \
    C(float, 256, 16, 8) C(float, 256, 16, 16) C(float, 256, 16, 32) \
    C(float, 512, 16, 4) C(float, 512, 16, 8) C(float, 512, 16, 16) C(float, 512, 32, 16) \
    C(float, 1024, 16, 4) C(float, 1024, 16, 8) C(float, 1024, 32, 8) \
    C(float, 2048, 16, 4) \
    C(float, 128, 8, 8) C(float, 128, 8, 16) C(float, 128, 8, 32) \
    C(float, 256, 8, 4) C(float, 256, 8, 8) C(float, 256, 8, 16) \
    C(float, 512, 8, 4) C(float, 512, 8, 8) \
    C(float, 1024, 8, 4)
#define QSG_COL_VARIANTS_F64(C) \
    C(double, 128, 8, 8) C(double, 128, 8, 16) \
    C(double, 256, 8, 4) C(double, 256, 8, 8) \
    C(double, 512, 8, 4) \
    C(double, 1024, 8, 4) \
    C(double, 2048, 8, 2)

// the kinetic-energy column transform: one variant per (precision, M)
constexpr int kin_e_for(int prec) { return prec == 1 ? 16 : 8; }
constexpr int kin_w_for(int prec, int m)
{
    return prec == 1 ? (m >= 2048 ? 4 : (m >= 512 ? 8 : 256 / (m / 16)))
                     : (m >= 2048 ? 2 : (m >= 512 ? 4 : 256 / (m / 8)));
}

}  // namespace qsg
