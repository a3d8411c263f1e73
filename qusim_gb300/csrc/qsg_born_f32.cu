// Born-series kernels, complex64 instantiations (plus the geometry helpers).
#include "qsg_born_inst.cuh"

namespace qsg {

bool born2d_supported(int nx, int ny)
{
    auto ok = [](int v) { return v >= 64 && v <= 4096 && (v & (v - 1)) == 0; };
    return ok(nx) && ok(ny);
}

bool born1d_resident(int prec, uint64_t n)
{
    if (n < 128 || (n & (n - 1))) return false;
    return n <= (prec == 1 ? 8192u : 4096u);
}

void born_fs_split(uint64_t n, int *n1, int *n2)
{
    int lg = 0;
    while ((1ull << lg) < n) ++lg;
    *n2 = 1 << (lg / 2);
    *n1 = (int)(n >> (lg / 2));
}

bool born1d_supported(int prec, uint64_t n)
{
    if (born1d_resident(prec, n)) return true;
    return n >= 8192 && n <= (1u << 22) && (n & (n - 1)) == 0;
}

int born_split(int prec, int nx, int ny) { return born_split_c(prec, nx, ny); }
int born_row_blocks(int prec, int nx, int ny)
{
    const int g = born_split(prec, nx, ny);
    return nx / (g * born_row_b(prec, ny, g));
}
int born_fs_col_blocks(int prec, int n1, int n2) { return n1 / born_fs_w(prec, n2); }
int born_xsec_blocks(int nx) { return (nx + kXsecRows - 1) / kXsecRows; }

QSG_BORN_INSTANTIATE(float)

}  // namespace qsg
