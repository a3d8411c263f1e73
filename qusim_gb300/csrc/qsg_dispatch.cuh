// qsg_dispatch.cuh -- helpers shared by the instantiation units.
#pragma once
#include "qsg_launch.h"

namespace qsg {

template <class K>
static inline cudaError_t prepare_smem(K kernel, size_t smem)
{
    if (smem > 48 * 1024)
        return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return cudaSuccess;
}

// Geometry rules (shared by the launchers and geom2d):
//  * x split G: complex64 keeps column blocks M = Nx/G <= 1024, complex128 <= 2048
//  * row pass: B groups of G rows per CTA so a CTA holds >= 256 threads of
//    line work; RS sequential rounds keep the CTA at <= 512 threads
//  * column pass: W adjacent columns per CTA (64 B rows for complex64),
//    <= 512 threads
constexpr int split_g_for(int prec, int nx)
{
    return prec == 1 ? (nx > 1024 ? nx / 1024 : 1) : (nx > 2048 ? nx / 2048 : 1);
}
constexpr int row_b_for(int ny, int e, int g)
{
    return (256 / (g * (ny / e))) > 1 ? 256 / (g * (ny / e)) : 1;
}
constexpr int row_rs_for(int ny, int e, int g)
{
    return (row_b_for(ny, e, g) * g * (ny / e)) > 512 ? row_b_for(ny, e, g) * g * (ny / e) / 512 : 1;
}
constexpr int col_w_for(int m, int e, int prec)
{
    return prec == 1 ? (512 / (m / e) < 8 ? 8 : (256 / (m / e) > 8 ? 256 / (m / e) : 8))
                     : (m >= 2048 ? 2 : (256 / (m / e) > 4 ? 256 / (m / e) : 4));
}

}  // namespace qsg
