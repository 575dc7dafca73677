/* Oracle compat shim (test infrastructure): the FFTW3 subset genetIC calls
 * (genetIC/src/tools/numerics/fourier.hpp:45-61,486-563,605-624): 3-D r2c/c2r
 * (double and float, in place with FFTW's padded rows) and 3-D complex DFTs,
 * unnormalised, FFTW sign convention (forward e^{-i...}, backward e^{+i...}).
 * Implemented in compat_fftw.cpp with a textbook mixed-radix Cooley-Tukey FFT. */
#ifndef COMPAT_FFTW3_H
#define COMPAT_FFTW3_H
#ifdef __cplusplus
extern "C" {
#endif
typedef double fftw_complex[2];
typedef float fftwf_complex[2];
typedef struct compat_fft_plan *fftw_plan;
typedef struct compat_fft_plan *fftwf_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)
int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);
fftw_plan fftw_plan_dft_r2c_3d(int n0, int n1, int n2, double *in, fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_3d(int n0, int n1, int n2, fftw_complex *in, double *out, unsigned flags);
fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
fftwf_plan fftwf_plan_dft_r2c_3d(int n0, int n1, int n2, float *in, fftwf_complex *out, unsigned flags);
fftwf_plan fftwf_plan_dft_c2r_3d(int n0, int n1, int n2, fftwf_complex *in, float *out, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftwf_execute(const fftwf_plan p);
void fftw_destroy_plan(fftw_plan p);
void fftwf_destroy_plan(fftwf_plan p);
#ifdef __cplusplus
}
#endif
#endif
