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
 *   orc_detect_f / _d    src/singleChannel/detector.cpp:38-284, :419-691
 *                        and src/singleChannel/relativeMagnitude.cpp:35-130
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
                /* the same predicate as the core count: a NaN distance is no neighbour */
                if (!(orc_dist(&X[(size_t) p*nf], &X[(size_t) j*nf], nf) <= eps)) { continue; }
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

/* ------------------------------------------------------------------------ */
/* Single-channel detector: Detector<T>::detect (src/singleChannel/
 * detector.cpp:419-691) for one matched-filter object, T = float or double:
 *   reduceAllCorrelations / setCorrelations + cleanReducedTemplate
 *   (:191-284), PeakFinder (orc_peaks), then per detection the clamped
 *   coefficient of the chosen template, the sign of its coefficient, the
 *   refinement quadraticRefinement (:38-91, double, returned as T) or
 *   lanczosRefinement (:93-152, in T), and the relative amplitudes of
 *   RelativeMagnitude (src/singleChannel/relativeMagnitude.cpp:35-130) in
 *   double with the window mean (the double overload's semantics).
 * SINGLE-policy detections are ordered by time, ties in template order. */
static double orc_quadratic(long n, const double *ys, long p, double dt, int use_abs)
{
    if (!(p > 0 && p < n - 1)) { return 0.0; }
    double y1 = ys[0], y2 = ys[1], y3 = ys[2];
    if (use_abs) { y1 = fabs(y1); y2 = fabs(y2); y3 = fabs(y3); }
    if (y2 < y1 || y2 < y3)
    {
        if (y2 < y1 && y2 < y3) { y1 = -y1; y2 = -y2; y3 = -y3; }
        else { return 0.0; }
    }
    y1 = fmin(y2 - 100 * DBL_EPSILON, y1);
    y3 = fmin(y2 - 100 * DBL_EPSILON, y3);
    return (dt * (y1 - y3)) / (2 * (y1 - 2 * y2 + y3));
}

typedef struct { int t; int p; } orc_det_pair;

static int orc_det_cmp(const void *a, const void *b)
{
    const orc_det_pair *x = (const orc_det_pair *) a, *y = (const orc_det_pair *) b;
    if (x->p != y->p) { return x->p < y->p ? -1 : 1; }
    return x->t < y->t ? -1 : (x->t > y->t);
}

#define ORC_DETECT(NAME, T, SINF, TEPS, TMAX)                                                            \
static T NAME##_sinc(T x)                                                                                   \
{                                                                                                           \
    const T tol = TEPS * (T) 100;                                                                           \
    if (fabs((double) x) > tol) { T pix = (T) (3.14159265358979323846 * (double) x); return SINF(pix) / pix; } \
    return (T) 1;                                                                                           \
}                                                                                                           \
static T NAME##_lanczos(T x, int a)                                                                         \
{                                                                                                           \
    if ((int) fabs((double) x) <= a) { return NAME##_sinc(x) * NAME##_sinc(x / (T) a); }                   \
    return (T) 0;                                                                                           \
}                                                                                                           \
ORC_API int NAME(int nt, long len, const T *rho, long ldr, int use_abs, int single, double thr,            \
                 int min_dist, int interp, int alpha, int nrefine, double fs, int amplitudes,              \
                 const int *tlen, const double *const *templates, const T *const *signals, long n,         \
                 int maxdet, int *o_tmpl, int *o_sample, double *o_xc, double *o_shift, int *o_sign,       \
                 int *o_have, double *o_gr, double *o_sr)                                                   \
{                                                                                                           \
    double *det = (double *) malloc(sizeof(double) * (size_t) (len > 0 ? len : 1));                        \
    int *pk = (int *) malloc(sizeof(int) * (size_t) (len > 0 ? len : 1));                                  \
    int *id = (int *) calloc((size_t) (len > 0 ? len : 1), sizeof(int));                                   \
    orc_det_pair *pairs = NULL;                                                                             \
    int np = 0, cap = 0;                                                                                    \
    for (int pass = 0; pass < (single ? nt : 1); ++pass)                                                    \
    {                                                                                                       \
        for (long k = 0; k < len; ++k)                                                                      \
        {                                                                                                   \
            T best = rho[(long) (single ? pass : 0) * ldr + k];                                             \
            if (use_abs) { best = (T) fabs((double) best); }                                                \
            int bi = single ? pass : 0;                                                                     \
            if (!single)                                                                                    \
                for (int t = 1; t < nt; ++t)                                                                \
                {                                                                                           \
                    T v = rho[(long) t * ldr + k];                                                          \
                    if (use_abs) { v = (T) fabs((double) v); }                                              \
                    if (v > best) { best = v; bi = t; }                                                     \
                }                                                                                           \
            if (best > (T) 1) { best = (T) 1; }                                                             \
            if (best < (T) -1) { best = (T) -1; }                                                           \
            det[k] = (double) best;                                                                         \
            id[k] = bi;                                                                                     \
        }                                                                                                   \
        int m = orc_peaks((int) len, det, thr, min_dist, pk);                                              \
        if (np + m > cap)                                                                                   \
        {                                                                                                   \
            cap = 2 * (np + m) + 16;                                                                        \
            pairs = (orc_det_pair *) realloc(pairs, sizeof(orc_det_pair) * (size_t) cap);                   \
        }                                                                                                   \
        for (int i = 0; i < m; ++i) { pairs[np].t = id[pk[i]]; pairs[np].p = pk[i]; ++np; }                 \
    }                                                                                                       \
    if (single && np > 1) { qsort(pairs, (size_t) np, sizeof(orc_det_pair), orc_det_cmp); }               \
    const double dt = 1.0 / fs;                                                                             \
    for (int d = 0; d < np && d < maxdet; ++d)                                                              \
    {                                                                                                       \
        const int it = pairs[d].t;                                                                          \
        const long p = pairs[d].p;                                                                          \
        const T *xc = rho + (long) it * ldr;                                                                \
        const T v = xc[p];                                                                                  \
        T c = v > (T) 1 ? (T) 1 : (v < (T) -1 ? (T) -1 : v);                                                \
        o_tmpl[d] = it; o_sample[d] = (int) p; o_xc[d] = (double) c;                                        \
        o_sign[d] = v < (T) 0 ? -1 : (v == (T) 0 ? 0 : 1);                                                  \
        double shift = 0.0;                                                                                 \
        if (interp == 1)                                                                                    \
        {                                                                                                   \
            double ys[3] = {0.0, 0.0, 0.0};                                                                 \
            if (p > 0 && p < len - 1) { ys[0] = xc[p - 1]; ys[1] = xc[p]; ys[2] = xc[p + 1]; }              \
            shift = (double) (T) orc_quadratic(len, ys, p, dt, use_abs);                                    \
        }                                                                                                   \
        else if (interp == 0)                                                                               \
        {                                                                                                   \
            const T dtw = (T) (1.0 / (double) nrefine);                                                     \
            T opt = 0, ymax = -TMAX;                                                                        \
            for (int idx = 1; idx < nrefine; ++idx)                                                         \
            {                                                                                               \
                const T sh = (T) (-0.5 + (double) (dtw * (T) idx));                                         \
                const T x = (T) p + sh;                                                                     \
                T y = 0;                                                                                    \
                const int fl = (int) floor((double) x);                                                     \
                for (int a = -alpha; a <= alpha; ++a)                                                       \
                {                                                                                           \
                    const int i = fl - a + 1;                                                               \
                    const T xi = x - (T) i;                                                                 \
                    const T xv = (i >= 0 && i < len) ? xc[i] : (T) 0;                                       \
                    y = y + xv * NAME##_lanczos(xi, alpha);                                                 \
                }                                                                                           \
                if (use_abs) { y = (T) fabs((double) y); }                                                  \
                if (y > ymax) { opt = (T) (dt * (double) sh); ymax = y; }                                   \
            }                                                                                               \
            shift = (double) opt;                                                                           \
        }                                                                                                   \
        o_shift[d] = shift;                                                                                 \
        o_have[d] = 0; o_gr[d] = 0; o_sr[d] = 0;                                                            \
        const int L = tlen[it];                                                                             \
        if (amplitudes && p + L <= n)                                                                       \
        {                                                                                                   \
            const double *b = templates[it];                                                                \
            const T *y = signals[it] + p;                                                                   \
            double sb = 0, sy = 0;                                                                          \
            for (int j = 0; j < L; ++j) { sb += b[j]; sy += (double) y[j]; }                                \
            const double mb = sb / L, my = sy / L;                                                          \
            double bb = 0, yy = 0, by = 0;                                                                  \
            for (int j = 0; j < L; ++j)                                                                     \
            {                                                                                               \
                const double db = b[j] - mb, dy = (double) y[j] - my;                                       \
                bb += db * db; yy += dy * dy; by += db * dy;                                                \
            }                                                                                               \
            if (bb > 0 && yy > 0) { o_have[d] = 1; o_gr[d] = fabs(by) / bb; o_sr[d] = sqrt(yy / bb); }      \
        }                                                                                                   \
    }                                                                                                       \
    free(det); free(pk); free(id); free(pairs);                                                             \
    return np;                                                                                              \
}

ORC_DETECT(orc_detect_f, float, sinf, FLT_EPSILON, FLT_MAX)
ORC_DETECT(orc_detect_d, double, sin, DBL_EPSILON, DBL_MAX)
