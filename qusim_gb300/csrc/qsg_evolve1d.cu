// 1D resident evolver and 1D kinetic transform: instantiations + launchers.
#include "qsg_dispatch.cuh"

namespace qsg {

bool evolve1d_supported(int prec, uint64_t n)
{
    if (n < 64 || (n & (n - 1))) return false;
    return prec == 1 ? n <= 8192 : n <= 4096;
}

template <class T, int L>
static cudaError_t run_evolve1d(const Evolve1DArgs &a, cudaStream_t st)
{
    constexpr int E = sizeof(T) == 4 ? 16 : 8;
    constexpr int PADS = sizeof(T) == 4 ? 4 : 3;
    const size_t smem = sizeof(cplx_t<T>) * padded<L, PADS>(L);
    cudaError_t e = prepare_smem(k_evolve1d_resident<T, L, E>, smem);
    if (e != cudaSuccess) return e;
    k_evolve1d_resident<T, L, E><<<1, L / E, smem, st>>>(a);
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

#define QSG_1D_CASES(X, T) \
    X(T, 64) X(T, 128) X(T, 256) X(T, 512) X(T, 1024) X(T, 2048) X(T, 4096)

cudaError_t launch_evolve1d(int prec, int n, const Evolve1DArgs &a, cudaStream_t st)
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

}  // namespace qsg
