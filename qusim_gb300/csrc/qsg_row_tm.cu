// 2D row pass with the waiting rows parked in tensor memory: instantiations + launcher.
// Packed f32x2 arithmetic (qsg_fft.cuh), as the shared-memory row pass: with every
// complex add an explicit packed instruction the two row passes round alike.
#define QSG_PACKED_F32 1
#include <atomic>
#include "qsg_dispatch.cuh"
#include "qsg_row_tm.cuh"

namespace qsg {

bool row_tm_supported(int ny, int g) { return g == 4 && (ny == 2048 || ny == 4096); }

template <int NY, bool PL>
static cudaError_t run_row_tm(const RowPassArgs &a, cudaStream_t st)
{
    constexpr int NG = 512 / (NY / 16);  // independent row groups per CTA
    auto k = k_row_pass_tm<NY, PL>;
    const size_t smem = sizeof(float2) * NG * padded<NY, 4>(NY);  // one line buffer per group
    // the attribute belongs to the device's context: set once per device
    static std::atomic<uint64_t> ready{0};
    int dev = 0;
    cudaGetDevice(&dev);
    const uint64_t bit = dev < 64 ? 1ull << dev : 0;
    if (!bit || !(ready.load() & bit)) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        ready.fetch_or(bit);
    }
    // one CTA per SM: each takes all 512 TMEM columns of its SM
    const int ctas = (a.units + NG - 1) / NG;
    const int sms = sm_count();
    k<<<(unsigned)(ctas < sms ? ctas : sms), 512, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_row_pass_tm(const Geom2D &g, const RowPassArgs &a, cudaStream_t st)
{
    if (g.ny == 4096) return a.plain ? run_row_tm<4096, true>(a, st) : run_row_tm<4096, false>(a, st);
    if (g.ny == 2048) return a.plain ? run_row_tm<2048, true>(a, st) : run_row_tm<2048, false>(a, st);
    return cudaErrorNotSupported;
}

}  // namespace qsg
