/*
 * Project-written stand-in for the subset of the FFTW3 API that the mflib
 * matched filter calls (src/matchedFilter.cpp:613-649, :763-796, :1032,
 * :1069, :1089, :1204, :1241, :1261).  TEST INFRASTRUCTURE ONLY: it lets the
 * reference sources compile unchanged into oracle/_ref/ so the oracle's
 * restatement can be checked against them.  Conventions follow FFTW:
 * unnormalised transforms, r2c output of n/2+1 complex values, many-plans
 * with stride 1 and distance idist/odist between transforms.
 */
#ifndef ORC_SHIM_FFTW3_H
#define ORC_SHIM_FFTW3_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef double fftw_complex[2];
typedef float fftwf_complex[2];
typedef struct orc_fftw_plan_s *fftw_plan;
typedef struct orc_fftwf_plan_s *fftwf_plan;
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_PATIENT (1U << 5)

fftw_plan fftw_plan_many_dft_r2c(int rank, const int *n, int howmany,
                                 double *in, const int *inembed, int istride, int idist,
                                 fftw_complex *out, const int *onembed, int ostride, int odist,
                                 unsigned flags);
fftw_plan fftw_plan_many_dft_c2r(int rank, const int *n, int howmany,
                                 fftw_complex *in, const int *inembed, int istride, int idist,
                                 double *out, const int *onembed, int ostride, int odist,
                                 unsigned flags);
fftw_plan fftw_plan_dft_r2c_1d(int n, double *in, fftw_complex *out, unsigned flags);
void fftw_execute_dft_r2c(const fftw_plan p, double *in, fftw_complex *out);
void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex *in, double *out);
void fftw_destroy_plan(fftw_plan p);
void fftw_free(void *p);

fftwf_plan fftwf_plan_many_dft_r2c(int rank, const int *n, int howmany,
                                   float *in, const int *inembed, int istride, int idist,
                                   fftwf_complex *out, const int *onembed, int ostride, int odist,
                                   unsigned flags);
fftwf_plan fftwf_plan_many_dft_c2r(int rank, const int *n, int howmany,
                                   fftwf_complex *in, const int *inembed, int istride, int idist,
                                   float *out, const int *onembed, int ostride, int odist,
                                   unsigned flags);
fftwf_plan fftwf_plan_dft_r2c_1d(int n, float *in, fftwf_complex *out, unsigned flags);
void fftwf_execute_dft_r2c(const fftwf_plan p, float *in, fftwf_complex *out);
void fftwf_execute_dft_c2r(const fftwf_plan p, fftwf_complex *in, float *out);
void fftwf_destroy_plan(fftwf_plan p);
void fftwf_free(void *p);
#ifdef __cplusplus
}
#endif
#endif
