/*
 * fftw3.h -- TEST INFRASTRUCTURE ONLY: the part of the FFTW3 C interface
 * that the reference's src/fftw.cpp uses (plans for real <-> half-complex
 * and complex transforms of rank 1-3, their execution on new arrays, plan
 * destruction), declared so that the reference's CPU sources compile into
 * the oracle's reference build.  The functions are implemented by
 * oracle/ref/fftw_shim.cpp on a double-precision FFT of this project (FFTW
 * itself is not installed here).  Conventions as FFTW's: unnormalised
 * transforms, sign -1 forward, row-major arrays, the last dimension halved
 * (n/2 + 1) on the complex side of real transforms.
 */
#ifndef GBR_ORACLE_FFTW3_SHIM_H
#define GBR_ORACLE_FFTW3_SHIM_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef float fftwf_complex[2];
typedef struct gbr_shim_plan_s *fftw_plan;
typedef struct gbr_shim_plan_s *fftwf_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_DESTROY_INPUT (1U << 0)
#define FFTW_PRESERVE_INPUT (1U << 4)

fftw_plan fftw_plan_dft_r2c(int rank, const int *n, double *in, fftw_complex *out, unsigned flags);
fftw_plan fftw_plan_dft_c2r(int rank, const int *n, fftw_complex *in, double *out, unsigned flags);
fftw_plan fftw_plan_dft(int rank, const int *n, fftw_complex *in, fftw_complex *out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_execute_dft_r2c(const fftw_plan p, double *in, fftw_complex *out);
void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex *in, double *out);
void fftw_execute_dft(const fftw_plan p, fftw_complex *in, fftw_complex *out);
void fftw_destroy_plan(fftw_plan p);
void fftw_cleanup(void);
void *fftw_malloc(size_t n);
void fftw_free(void *p);
void fftw_plan_with_nthreads(int n);
int fftw_init_threads(void);
void fftw_cleanup_threads(void);

fftwf_plan fftwf_plan_dft_r2c(int rank, const int *n, float *in, fftwf_complex *out, unsigned flags);
fftwf_plan fftwf_plan_dft_c2r(int rank, const int *n, fftwf_complex *in, float *out, unsigned flags);
fftwf_plan fftwf_plan_dft(int rank, const int *n, fftwf_complex *in, fftwf_complex *out, int sign, unsigned flags);
void fftwf_execute(const fftwf_plan p);
void fftwf_execute_dft_r2c(const fftwf_plan p, float *in, fftwf_complex *out);
void fftwf_execute_dft_c2r(const fftwf_plan p, fftwf_complex *in, float *out);
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex *in, fftwf_complex *out);
void fftwf_destroy_plan(fftwf_plan p);
void fftwf_cleanup(void);
void *fftwf_malloc(size_t n);
void fftwf_free(void *p);
void fftwf_plan_with_nthreads(int n);
int fftwf_init_threads(void);
void fftwf_cleanup_threads(void);

#ifdef __cplusplus
}
#endif
#endif
