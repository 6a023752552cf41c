/*
 * mf_oracle.c -- CPU oracle for the matched-filtering hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (mflib_gb300/, include/)
 * links, loads or calls this file.  It is used by tests/ (as the checker),
 * by __graft_entry__.smoke() (as the checker) and by bench.py's CPU
 * baseline leg (timed as the reference's algorithm on the host cores).
 *
 * Each function restates one reference routine, cited by file:line within
 * the mflib project:
 *   orc_fft_sizes        src/matchedFilterParameters.cpp:18-104, :371-385
 *   orc_mf_d / orc_mf_f  src/matchedFilter.cpp:94-190, :507-821, :863-921,
 *                        :972-1316 (see orc_mf.h)
 *   orc_shift_and_stack  src/matchedFilter.cpp:577-592, :1319-1364
 *   orc_pearson_naive    testing/utilities.hpp:33-69 (two-pass FP64 Pearson)
 *   orc_peaks            src/peakFinder.cpp:329-446
 *   orc_dbscan           src/dbscan.cpp:187-214 -> Intel DAAL dbscan::Batch
 *                        (third-party, not vendored; restated from DAAL's
 *                        published algorithm, see the function comment)
 *
 * Parity of the restatement is pinned against the reference's own golden
 * vectors (FFT sizes, peak indices, DBSCAN labels, analytic matched-filter
 * tests) and against the reference sources compiled unchanged against a
 * project-written FFTW/MKL shim (oracle/build.py, outputs in oracle/_ref/).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>

#define ORC_API __attribute__((visibility("default")))

/* ------------------------------------------------------------------------ */
/* FFT sizing: src/matchedFilterParameters.cpp:18-104.  The flop table and
 * candidate lengths must match the reference for the block length to match. */
static const double orc_fft_flops[21] = {
    18, 59, 138, 303, 660, 1441, 3150, 6875, 14952, 32373, 69762,
    149647, 319644, 680105, 1441974, 3047619, 6422736, 13500637, 28311786,
    59244791, 59244791*2.09
};

static int orc_next_pow2(int n)
{
    if (n <= 1) { return 1; }
    int itemp = (int) ceil(log2((double) n));
    uint64_t n2t = (uint64_t) pow(2.0, itemp);
    return (int) n2t;
}

/* Returns 0 on success, -1 for invalid arguments (reference throws). */
ORC_API int orc_fft_sizes(int nb, int nx, int *nfft, int *L)
{
    if (nb < 1 || nx <= nb) { return -1; }
    int start = -1;
    for (int i = 0; i < 21; ++i)
    {
        uint64_t len = (uint64_t) 1 << (i + 1);
        if (len > (uint64_t) (nb - 1)) { start = i; break; }
    }
    if (start < 0)
    {
        *nfft = orc_next_pow2(nx);
        *L = *nfft - (nb - 1);
        return 0;
    }
    double best = DBL_MAX;
    int bn = 0, bl = 0;
    for (int i = start; i < 21; ++i)
    {
        int len = 1 << (i + 1);
        int lt = len - (nb - 1);
        double obj = ceil((double) nx/(double) lt)*orc_fft_flops[i];
        if (obj < best) { best = obj; bn = len; bl = lt; }
    }
    *nfft = bn;
    *L = bl;
    return 0;
}

/* ------------------------------------------------------------------------ */
#define ORC_R double
#define ORC_FN(name) name##_d
#include "orc_fft.h"
#include "orc_mf.h"
#undef ORC_R
#undef ORC_FN
#define ORC_R float
#define ORC_FN(name) name##_f
#include "orc_fft.h"
#include "orc_mf.h"
#undef ORC_R
#undef ORC_FN

/* Reference MatchedFilter<double>: tol 1e-12 (src/matchedFilter.cpp:1115). */
ORC_API int orc_mf_d(int multi, int nt, const int *lens, const double *const *templates,
                     int n, const double *const *signals, double *out, long ldo, int nthreads)
{
    return mf_apply_d(multi, nt, lens, templates, n, signals, out, ldo, 0, 1.e-12, nthreads);
}

/* Reference MatchedFilter<float>: tol 1e-6 (src/matchedFilter.cpp:1287).
 * float_quirk = 1 reproduces the max-length template preparation (:725). */
ORC_API int orc_mf_f(int multi, int nt, const int *lens, const double *const *templates,
                     int n, const float *const *signals, float *out, long ldo,
                     int float_quirk, int nthreads)
{
    return mf_apply_f(multi, nt, lens, templates, n, signals, out, ldo, float_quirk,
                      1.e-6f, nthreads);
}

/* Same algorithm in FP64 on FP32 inputs: the FP64 restatement used as the
 * parity reference for the FP32 GPU path. */
ORC_API int orc_mf_d_from_f(int multi, int nt, const int *lens,
                            const double *const *templates, int n,
                            const float *const *signals, double *out, long ldo, int nthreads)
{
    int nsig = multi ? nt : 1;
    double **sd = (double **) malloc(sizeof(double *)*(size_t) nsig);
    for (int s = 0; s < nsig; ++s)
    {
        sd[s] = (double *) malloc(sizeof(double)*(size_t) n);
        for (int i = 0; i < n; ++i) { sd[s][i] = (double) signals[s][i]; }
    }
    int rc = mf_apply_d(multi, nt, lens, templates, n, (const double *const *) sd, out, ldo,
                        0, 1.e-12, nthreads);
    for (int s = 0; s < nsig; ++s) { free(sd[s]); }
    free(sd);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Shift and stack, src/matchedFilter.cpp:1319-1364 with the shifts captured at
 * :577-592.  rho rows have stride ldr and at least nfilt valid lags. */
ORC_API int orc_shift_and_stack(int nt, const double *rho, long ldr, int nfilt,
                                const int *shifts, const double *weights, int stack_abs,
                                double *out, int *nout)
{
    if (nt < 1) { return -1; }
    int smax = shifts[0];
    double xnorm = 0;
    for (int t = 0; t < nt; ++t) { if (shifts[t] > smax) { smax = shifts[t]; } xnorm += weights[t]; }
    if (xnorm > 0) { xnorm = 1/xnorm; }
    int len = nfilt - smax;
    if (len < 0) { return -1; }
    for (int k = 0; k < len; ++k) { out[k] = 0; }
    for (int t = 0; t < nt; ++t)
    {
        double w = xnorm*weights[t];
        const double *p = &rho[(size_t) t*ldr];
        for (int k = 0; k < len; ++k)
        {
            double v = p[k + shifts[t]];
            out[k] += w*(stack_abs ? fabs(v) : v);
        }
    }
    *nout = len;
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Two-pass FP64 Pearson coefficient, testing/utilities.hpp:33-69:
 * template and each window demeaned, rho = <b~, x~>/(|b~| max(eps, |x~|)).
 * lags == NULL evaluates every lag 0..nx-nb; otherwise nlags given lags. */
ORC_API void orc_pearson_naive(int nb, const double *b, int nx, const double *x,
                               const int *lags, int nlags, double *xc)
{
    double bmean = 0;
    for (int i = 0; i < nb; ++i) { bmean += b[i]; }
    bmean /= (double) nb;
    double *bt = (double *) malloc(sizeof(double)*(size_t) nb);
    double eb = 0;
    for (int i = 0; i < nb; ++i) { bt[i] = b[i] - bmean; eb += bt[i]*bt[i]; }
    eb = sqrt(eb);
    int count = lags ? nlags : nx - nb + 1;
    for (int q = 0; q < count; ++q)
    {
        int i = lags ? lags[q] : q;
        const double *xp = &x[i];
        double xm = 0;
        for (int j = 0; j < nb; ++j) { xm += xp[j]; }
        xm /= (double) nb;
        double ex = 0, dot = 0;
        for (int j = 0; j < nb; ++j)
        {
            double v = xp[j] - xm;
            ex += v*v;
            dot += bt[j]*v;
        }
        ex = sqrt(ex);
        if (ex < DBL_EPSILON) { ex = DBL_EPSILON; }
        xc[q] = dot/(eb*ex);
    }
    free(bt);
}

/* ------------------------------------------------------------------------ */
/* Peak finder, src/peakFinder.cpp:329-446.
 *   candidates: i = 0 if x[1] < x[0] and x[0] > thr; 1 <= i <= n-2 if
 *   x[i] >= x[i-1], x[i+1] < x[i] and x[i] > thr (right edge of a plateau);
 *   i = n-1 if x[n-1] > x[n-2] and x[n-1] > thr.  With minDist > 0 the
 *   candidates are visited by value (descending) and kept when farther than
 *   minDist (strict) from every kept peak; the result is sorted by index.
 * Ties in value: the reference sorts with an unstable std::sort, so its
 * order among equal values is implementation-defined; this restatement
 * breaks ties by lower index first.
 * n == 1: the reference reads x[1] out of bounds (:354); here the missing
 * neighbour is treated as 0, so x[0] is a peak iff x[0] > thr and x[0] > 0. */
typedef struct { double v; int i; } orc_pk;

static int orc_pk_cmp(const void *a, const void *b)
{
    const orc_pk *p = (const orc_pk *) a, *q = (const orc_pk *) b;
    if (p->v > q->v) { return -1; }
    if (p->v < q->v) { return 1; }
    return (p->i < q->i) ? -1 : (p->i > q->i);
}

static int orc_int_cmp(const void *a, const void *b)
{
    int x = *(const int *) a, y = *(const int *) b;
    return (x > y) - (x < y);
}

ORC_API int orc_peaks(int n, const double *x, double thr, int minDist, int *peaks)
{
    if (n < 1) { return 0; }
    double xmax = x[0];
    for (int i = 1; i < n; ++i) { if (x[i] > xmax) { xmax = x[i]; } }
    if (xmax < thr) { return 0; }
    orc_pk *c = (orc_pk *) malloc(sizeof(orc_pk)*(size_t) n);
    int nc = 0;
    if (n == 1)
    {
        if (x[0] > thr && x[0] > 0) { c[nc].v = x[0]; c[nc].i = 0; ++nc; }
    }
    else
    {
        if (x[1] - x[0] < 0 && x[0] > thr) { c[nc].v = x[0]; c[nc].i = 0; ++nc; }
        for (int i = 1; i < n - 1; ++i)
        {
            double d0 = x[i] - x[i - 1];
            double d1 = x[i + 1] - x[i];
            if (d0 >= 0 && d1 < 0 && x[i] > thr) { c[nc].v = x[i]; c[nc].i = i; ++nc; }
        }
        if (x[n - 1] - x[n - 2] > 0 && x[n - 1] > thr) { c[nc].v = x[n - 1]; c[nc].i = n - 1; ++nc; }
    }
    int np = 0;
    if (nc == 0) { free(c); return 0; }
    if (minDist > 0)
    {
        qsort(c, (size_t) nc, sizeof(orc_pk), orc_pk_cmp);
        peaks[0] = c[0].i;
        np = 1;
        for (int q = 0; q < nc; ++q)
        {
            int idx = c[q].i;
            int dmin = abs(peaks[0] - idx);
            for (int k = 1; k < np; ++k) { int d = abs(peaks[k] - idx); if (d < dmin) { dmin = d; } }
            if (dmin > minDist) { peaks[np++] = idx; }
        }
        qsort(peaks, (size_t) np, sizeof(int), orc_int_cmp);
    }
    else
    {
        for (int q = 0; q < nc; ++q) { peaks[q] = c[q].i; }
        np = nc;
    }
    free(c);
    return np;
}

/* ------------------------------------------------------------------------ */
/* DBSCAN with Intel DAAL's published semantics (src/dbscan.cpp:187-214 calls
 * daal::algorithms::dbscan::Batch<double>(epsilon, minObservations); DAAL is
 * not vendored and no version is pinned by the reference build):
 *   neighbourhood N(i) = { j : ||x_i - x_j||_2 <= eps }, including i;
 *   i is a core point iff sum_{j in N(i)} w_j >= minObservations (w = 1
 *   when unweighted);
 *   observations are visited in index order; an unassigned core point opens
 *   cluster nClusters++ which is expanded breadth-first; a point reached by
 *   an expansion joins that cluster if it has none yet (border points join
 *   the first cluster that reaches them); everything else is noise (-1).
 * Returns the number of clusters. */
static double orc_dist(const double *a, const double *b, int nf)
{
    double s = 0;
    for (int f = 0; f < nf; ++f) { double d = a[f] - b[f]; s += d*d; }
    return sqrt(s);
}

ORC_API int orc_dbscan(int nobs, int nf, const double *X, const double *w,
                       double eps, int minObs, int *labels)
{
    const int UNDEF = -2, NOISE = -1;
    char *core = (char *) calloc((size_t) nobs, 1);
    for (int i = 0; i < nobs; ++i)
    {
        double s = 0;
        for (int j = 0; j < nobs; ++j)
        {
            if (orc_dist(&X[(size_t) i*nf], &X[(size_t) j*nf], nf) <= eps) { s += w ? w[j] : 1.0; }
        }
        core[i] = s >= (double) minObs;
        labels[i] = UNDEF;
    }
    int *queue = (int *) malloc(sizeof(int)*(size_t) (nobs > 0 ? nobs : 1));
    int ncl = 0;
    for (int i = 0; i < nobs; ++i)
    {
        if (labels[i] != UNDEF) { continue; }
        if (!core[i]) { labels[i] = NOISE; continue; }
        int cid = ncl++;
        labels[i] = cid;
        int qh = 0, qt = 0;
        queue[qt++] = i;
        while (qh < qt)
        {
            int p = queue[qh++];
            if (!core[p]) { continue; }
            for (int j = 0; j < nobs; ++j)
            {
                if (orc_dist(&X[(size_t) p*nf], &X[(size_t) j*nf], nf) > eps) { continue; }
                if (labels[j] == UNDEF || labels[j] == NOISE)
                {
                    int was_undef = labels[j] == UNDEF;
                    labels[j] = cid;
                    if (was_undef || core[j]) { queue[qt++] = j; }
                }
            }
        }
    }
    free(queue);
    free(core);
    return ncl;
}
