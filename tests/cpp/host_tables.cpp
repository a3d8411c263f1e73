// Host-side Bluestein tables of libqsg.so, checked on the CPU: the chirp and
// FFT_M(conj chirp) / M of the long buffers (double-double arithmetic on host
// threads, blue_tables_dd) against the long double tables of the one-CTA
// kernels (blue_tables) and, at small sizes, against a direct O(m^2) DFT in
// long double.  Prints one JSON line of maximum differences.
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <vector>

namespace qsg {
void blue_tables(uint64_t n, int m, std::vector<std::complex<long double>> &w,
                 std::vector<std::complex<long double>> &hs);
void blue_tables_dd(uint64_t n, uint64_t m, std::vector<std::complex<double>> &w,
                    std::vector<std::complex<double>> &hs);
}  // namespace qsg

using cld = std::complex<long double>;

int main()
{
    const uint64_t cases[][2] = {{3, 8}, {100, 256}, {1000, 2048}, {4099, 16384}, {5000, 16384}, {100000, 262144}};
    std::printf("{");
    bool first = true;
    for (auto &c : cases) {
        const uint64_t n = c[0], m = c[1];
        std::vector<cld> w, hs;
        std::vector<std::complex<double>> wd, hd;
        qsg::blue_tables(n, (int)m, w, hs);
        qsg::blue_tables_dd(n, m, wd, hd);
        long double dw = 0, dh = 0, hmax = 0, ddft = 0;
        for (uint64_t j = 0; j < m; ++j) {
            dw = std::max(dw, std::abs(w[j] - cld(wd[j].real(), wd[j].imag())));
            dh = std::max(dh, std::abs(hs[j] - cld(hd[j].real(), hd[j].imag())));
            hmax = std::max(hmax, std::abs(hs[j]));
        }
        if (m <= 2048) {
            // direct DFT of the circular chirp conj(w), divided by m
            const long double pi = 3.141592653589793238462643383279502884197L;
            for (uint64_t k = 0; k < m; ++k) {
                cld s = 0;
                for (uint64_t j = 0; j < m; ++j) {
                    const uint64_t q = j < n ? j : (m - j < n ? m - j : 0);
                    if (j >= n && m - j >= n) continue;
                    const cld h = std::conj(std::polar(1.0L, -pi * (long double)((q * q) % (2 * n)) / (long double)n));
                    s += h * std::polar(1.0L, -2 * pi * (long double)((j * k) % m) / (long double)m);
                }
                ddft = std::max(ddft, std::abs(s / (long double)m - cld(hd[k].real(), hd[k].imag())));
            }
        }
        std::printf("%s\"%lu_%lu\": [%.3Le, %.3Le, %.3Le]", first ? "" : ", ", (unsigned long)n, (unsigned long)m,
                    dw, hmax > 0 ? dh / hmax : dh, hmax > 0 ? ddft / hmax : ddft);
        first = false;
    }
    std::printf("}\n");
    return 0;
}
