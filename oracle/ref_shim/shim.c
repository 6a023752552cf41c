/*
 * shim.c -- implementation of the FFTW3/MKL stand-ins in fftw/fftw3.h and
 * mkl.h, built on the oracle's own real FFT (oracle/orc_fft.h).
 * TEST INFRASTRUCTURE ONLY: linked into oracle/_ref/ together with the
 * unchanged reference sources, never into the product.
 */
#define _POSIX_C_SOURCE 200112L
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "fftw/fftw3.h"
#include "mkl.h"

#define ORC_R double
#define ORC_FN(name) name##_d
#include "../orc_fft.h"
#undef ORC_R
#undef ORC_FN
#define ORC_R float
#define ORC_FN(name) name##_f
#include "../orc_fft.h"
#undef ORC_R
#undef ORC_FN

void *MKL_calloc(size_t num, size_t size, int alignment)
{
    size_t bytes = num*size;
    if (alignment < (int) sizeof(void *)) { alignment = (int) sizeof(void *); }
    void *p = NULL;
    if (posix_memalign(&p, (size_t) alignment, bytes > 0 ? bytes : 1) != 0) { return NULL; }
    memset(p, 0, bytes);
    return p;
}
void MKL_free(void *p) { free(p); }
void *mkl_calloc(size_t num, size_t size, int alignment) { return MKL_calloc(num, size, alignment); }
void mkl_free(void *p) { free(p); }
void mkl_finalize(void) { }

struct orc_fftw_plan_s
{
    rfft_plan_d plan;
    int howmany, idist, odist, r2c;
    cpx_d *work;
    cpx_d *spec;
};

struct orc_fftwf_plan_s
{
    rfft_plan_f plan;
    int howmany, idist, odist, r2c;
    cpx_f *work;
    cpx_f *spec;
};

static fftw_plan mkplan_d(int n, int howmany, int idist, int odist, int r2c)
{
    fftw_plan p = (fftw_plan) calloc(1, sizeof(*p));
    rfft_plan_init_d(&p->plan, n);
    p->howmany = howmany; p->idist = idist; p->odist = odist; p->r2c = r2c;
    p->work = (cpx_d *) malloc(sizeof(cpx_d)*(size_t) (n/2 + 1));
    p->spec = (cpx_d *) malloc(sizeof(cpx_d)*(size_t) (n/2 + 1));
    return p;
}

static fftwf_plan mkplan_f(int n, int howmany, int idist, int odist, int r2c)
{
    fftwf_plan p = (fftwf_plan) calloc(1, sizeof(*p));
    rfft_plan_init_f(&p->plan, n);
    p->howmany = howmany; p->idist = idist; p->odist = odist; p->r2c = r2c;
    p->work = (cpx_f *) malloc(sizeof(cpx_f)*(size_t) (n/2 + 1));
    p->spec = (cpx_f *) malloc(sizeof(cpx_f)*(size_t) (n/2 + 1));
    return p;
}

fftw_plan fftw_plan_many_dft_r2c(int rank, const int *n, int howmany, double *in,
                                 const int *inembed, int istride, int idist,
                                 fftw_complex *out, const int *onembed, int ostride, int odist,
                                 unsigned flags)
{
    (void) rank; (void) in; (void) inembed; (void) istride; (void) out; (void) onembed;
    (void) ostride; (void) flags;
    return mkplan_d(n[0], howmany, idist, odist, 1);
}

fftw_plan fftw_plan_many_dft_c2r(int rank, const int *n, int howmany, fftw_complex *in,
                                 const int *inembed, int istride, int idist,
                                 double *out, const int *onembed, int ostride, int odist,
                                 unsigned flags)
{
    (void) rank; (void) in; (void) inembed; (void) istride; (void) out; (void) onembed;
    (void) ostride; (void) flags;
    return mkplan_d(n[0], howmany, idist, odist, 0);
}

fftw_plan fftw_plan_dft_r2c_1d(int n, double *in, fftw_complex *out, unsigned flags)
{
    (void) in; (void) out; (void) flags;
    return mkplan_d(n, 1, n, n/2 + 1, 1);
}

void fftw_execute_dft_r2c(const fftw_plan p, double *in, fftw_complex *out)
{
    int ns = p->plan.n/2 + 1;
    for (int h = 0; h < p->howmany; ++h)
    {
        rfft_r2c_d(&p->plan, in + (size_t) h*p->idist, p->spec, p->work);
        double *o = (double *) (out + (size_t) h*p->odist);
        for (int k = 0; k < ns; ++k) { o[2*k] = p->spec[k].re; o[2*k + 1] = p->spec[k].im; }
    }
}

void fftw_execute_dft_c2r(const fftw_plan p, fftw_complex *in, double *out)
{
    int ns = p->plan.n/2 + 1;
    for (int h = 0; h < p->howmany; ++h)
    {
        const double *i = (const double *) (in + (size_t) h*p->idist);
        for (int k = 0; k < ns; ++k) { p->spec[k].re = i[2*k]; p->spec[k].im = i[2*k + 1]; }
        rfft_c2r_d(&p->plan, p->spec, out + (size_t) h*p->odist, p->work);
    }
}

void fftw_destroy_plan(fftw_plan p)
{
    if (!p) { return; }
    rfft_plan_free_d(&p->plan);
    free(p->work); free(p->spec); free(p);
}

void fftw_free(void *p) { free(p); }

fftwf_plan fftwf_plan_many_dft_r2c(int rank, const int *n, int howmany, float *in,
                                   const int *inembed, int istride, int idist,
                                   fftwf_complex *out, const int *onembed, int ostride, int odist,
                                   unsigned flags)
{
    (void) rank; (void) in; (void) inembed; (void) istride; (void) out; (void) onembed;
    (void) ostride; (void) flags;
    return mkplan_f(n[0], howmany, idist, odist, 1);
}

fftwf_plan fftwf_plan_many_dft_c2r(int rank, const int *n, int howmany, fftwf_complex *in,
                                   const int *inembed, int istride, int idist,
                                   float *out, const int *onembed, int ostride, int odist,
                                   unsigned flags)
{
    (void) rank; (void) in; (void) inembed; (void) istride; (void) out; (void) onembed;
    (void) ostride; (void) flags;
    return mkplan_f(n[0], howmany, idist, odist, 0);
}

fftwf_plan fftwf_plan_dft_r2c_1d(int n, float *in, fftwf_complex *out, unsigned flags)
{
    (void) in; (void) out; (void) flags;
    return mkplan_f(n, 1, n, n/2 + 1, 1);
}

void fftwf_execute_dft_r2c(const fftwf_plan p, float *in, fftwf_complex *out)
{
    int ns = p->plan.n/2 + 1;
    for (int h = 0; h < p->howmany; ++h)
    {
        rfft_r2c_f(&p->plan, in + (size_t) h*p->idist, p->spec, p->work);
        float *o = (float *) (out + (size_t) h*p->odist);
        for (int k = 0; k < ns; ++k) { o[2*k] = p->spec[k].re; o[2*k + 1] = p->spec[k].im; }
    }
}

void fftwf_execute_dft_c2r(const fftwf_plan p, fftwf_complex *in, float *out)
{
    int ns = p->plan.n/2 + 1;
    for (int h = 0; h < p->howmany; ++h)
    {
        const float *i = (const float *) (in + (size_t) h*p->idist);
        for (int k = 0; k < ns; ++k) { p->spec[k].re = i[2*k]; p->spec[k].im = i[2*k + 1]; }
        rfft_c2r_f(&p->plan, p->spec, out + (size_t) h*p->odist, p->work);
    }
}

void fftwf_destroy_plan(fftwf_plan p)
{
    if (!p) { return; }
    rfft_plan_free_f(&p->plan);
    free(p->work); free(p->spec); free(p);
}

void fftwf_free(void *p) { free(p); }
