// 3D passes, complex64 instantiations (plus the geometry helpers).
#include "qsg_evolve3d_inst.cuh"

namespace qsg {

bool evolve3d_supported(int prec, uint64_t nx, uint64_t ny, uint64_t nz)
{
    auto ok = [](uint64_t v) { return v >= 16 && v <= 1024 && (v & (v - 1)) == 0; };
    if (!ok(nx) || !ok(ny) || !ok(nz)) return false;
    // W adjacent z positions per strided CTA
    const uint64_t w = (uint64_t)std::max(w3(prec, (int)nx), w3(prec, (int)ny));
    return nz % w == 0 && nx * ny * nz <= (1ull << 30);
}
int row3_ctas(int prec, int l, size_t lines) { return (int)(lines / b3(prec, l)); }
int col3_ctas(int prec, int l, int inner, int outer) { return (inner / w3(prec, l)) * outer; }

QSG_3D_INSTANTIATE(float)

}  // namespace qsg
