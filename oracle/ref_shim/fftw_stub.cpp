// FFTW is not installed on these machines and the reference's vendored
// Windows FFTW binary must not be linked.  These definitions satisfy the
// linker for src/FourierTransform.cpp; the oracle build always selects the
// KISS path (fft_lib unset), so none of them is ever reached.
#include <cstdio>
#include <cstdlib>
extern "C" {
typedef double fftw_complex[2];
typedef struct fftw_plan_s *fftw_plan;
static void fftw_unavailable(const char *what)
{
    std::fprintf(stderr, "oracle/_ref: %s called but FFTW is not available\n", what);
    std::abort();
}
fftw_complex *fftw_alloc_complex(size_t) { fftw_unavailable("fftw_alloc_complex"); return nullptr; }
void *fftw_malloc(size_t) { fftw_unavailable("fftw_malloc"); return nullptr; }
void fftw_free(void *) { fftw_unavailable("fftw_free"); }
void fftw_execute(const fftw_plan) { fftw_unavailable("fftw_execute"); }
void fftw_destroy_plan(fftw_plan) { fftw_unavailable("fftw_destroy_plan"); }
fftw_plan fftw_plan_dft_1d(int, fftw_complex *, fftw_complex *, int, unsigned)
{ fftw_unavailable("fftw_plan_dft_1d"); return nullptr; }
fftw_plan fftw_plan_dft_2d(int, int, fftw_complex *, fftw_complex *, int, unsigned)
{ fftw_unavailable("fftw_plan_dft_2d"); return nullptr; }
fftw_plan fftw_plan_dft_3d(int, int, int, fftw_complex *, fftw_complex *, int, unsigned)
{ fftw_unavailable("fftw_plan_dft_3d"); return nullptr; }
}
