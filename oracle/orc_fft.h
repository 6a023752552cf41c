/*
 * orc_fft.h -- real FFT used by the CPU oracle (TEST INFRASTRUCTURE ONLY).
 *
 * This header is included twice by mf_oracle.c, once with ORC_R = double and
 * once with ORC_R = float, so that the oracle can restate both precisions of
 * the reference matched filter (src/matchedFilter.cpp double path :972-1141,
 * float path :1144-1316).  The reference calls FFTW's r2c/c2r (unnormalised,
 * r2c output length N/2+1, src/matchedFilter.cpp:613-649); this file
 * provides the same conventions with an iterative radix-2 transform of
 * N/2 complex points plus the standard even/odd real-signal packing.
 * Twiddles are computed in double precision with cos/sin and rounded once.
 */
#ifndef ORC_R
#error "define ORC_R (double|float) and ORC_FN(name) before including"
#endif

typedef struct { ORC_R re, im; } ORC_FN(cpx);

typedef struct
{
    int n;              /* real transform length N (power of two >= 2) */
    int p;              /* complex length P = N/2 */
    ORC_FN(cpx) *tw;    /* P/2 twiddles exp(-2 pi i k / P) */
    ORC_FN(cpx) *post;  /* P+1 twiddles exp(-2 pi i k / N) */
    int *rev;           /* bit reversal permutation of length P */
    ORC_FN(cpx) *work;  /* scratch of length P (not thread safe) */
} ORC_FN(rfft_plan);

static void ORC_FN(rfft_plan_init)(ORC_FN(rfft_plan) *pl, int n)
{
    pl->n = n;
    pl->p = n/2;
    int p = pl->p;
    int half = p/2 > 0 ? p/2 : 1;
    pl->tw = (ORC_FN(cpx) *) malloc(sizeof(ORC_FN(cpx))*(size_t) half);
    pl->post = (ORC_FN(cpx) *) malloc(sizeof(ORC_FN(cpx))*(size_t) (p + 1));
    pl->rev = (int *) malloc(sizeof(int)*(size_t) p);
    pl->work = (ORC_FN(cpx) *) malloc(sizeof(ORC_FN(cpx))*(size_t) p);
    const double twopi = 6.283185307179586476925286766559;
    for (int k = 0; k < half; ++k)
    {
        double a = -twopi*(double) k/(double) p;
        pl->tw[k].re = (ORC_R) cos(a);
        pl->tw[k].im = (ORC_R) sin(a);
    }
    for (int k = 0; k <= p; ++k)
    {
        double a = -twopi*(double) k/(double) n;
        pl->post[k].re = (ORC_R) cos(a);
        pl->post[k].im = (ORC_R) sin(a);
    }
    int bits = 0;
    while ((1 << bits) < p) { ++bits; }
    for (int i = 0; i < p; ++i)
    {
        int r = 0;
        for (int b = 0; b < bits; ++b) { if (i & (1 << b)) { r |= 1 << (bits - 1 - b); } }
        pl->rev[i] = r;
    }
}

static void ORC_FN(rfft_plan_free)(ORC_FN(rfft_plan) *pl)
{
    free(pl->tw); free(pl->post); free(pl->rev); free(pl->work);
    pl->tw = NULL; pl->post = NULL; pl->rev = NULL; pl->work = NULL;
}

/* In-place complex FFT of length P; sign = -1 forward, +1 backward, no scaling. */
static void ORC_FN(cfft)(const ORC_FN(rfft_plan) *pl, ORC_FN(cpx) *a, int sign)
{
    int p = pl->p;
    for (int i = 0; i < p; ++i)
    {
        int j = pl->rev[i];
        if (j > i) { ORC_FN(cpx) t = a[i]; a[i] = a[j]; a[j] = t; }
    }
    for (int len = 2; len <= p; len <<= 1)
    {
        int hl = len/2;
        int step = p/len;
        for (int i = 0; i < p; i += len)
        {
            for (int k = 0; k < hl; ++k)
            {
                ORC_FN(cpx) w = pl->tw[k*step];
                if (sign > 0) { w.im = -w.im; }
                ORC_FN(cpx) u = a[i + k];
                ORC_FN(cpx) v = a[i + k + hl];
                ORC_FN(cpx) t;
                t.re = v.re*w.re - v.im*w.im;
                t.im = v.re*w.im + v.im*w.re;
                a[i + k].re = u.re + t.re;      a[i + k].im = u.im + t.im;
                a[i + k + hl].re = u.re - t.re; a[i + k + hl].im = u.im - t.im;
            }
        }
    }
}

/* r2c: x[N] real -> X[N/2+1] complex, unnormalised (FFTW convention).
 * `work` must hold P complex values. */
static void ORC_FN(rfft_r2c)(const ORC_FN(rfft_plan) *pl, const ORC_R *x,
                             ORC_FN(cpx) *X, ORC_FN(cpx) *work)
{
    int p = pl->p;
    if (pl->n == 1) { X[0].re = x[0]; X[0].im = 0; return; }
    for (int i = 0; i < p; ++i) { work[i].re = x[2*i]; work[i].im = x[2*i + 1]; }
    ORC_FN(cfft)(pl, work, -1);
    for (int k = 0; k <= p; ++k)
    {
        ORC_FN(cpx) zk = work[k % p];
        ORC_FN(cpx) zc = work[(p - k) % p];
        zc.im = -zc.im;
        /* even part E = (zk + zc)/2, odd part O = (zk - zc)/(2i) */
        ORC_R er = (ORC_R) 0.5*(zk.re + zc.re), ei = (ORC_R) 0.5*(zk.im + zc.im);
        ORC_R dr = (ORC_R) 0.5*(zk.re - zc.re), di = (ORC_R) 0.5*(zk.im - zc.im);
        ORC_R orr = di, oi = -dr;
        ORC_FN(cpx) w = pl->post[k];
        X[k].re = er + (w.re*orr - w.im*oi);
        X[k].im = ei + (w.re*oi + w.im*orr);
    }
}

/* c2r: X[N/2+1] Hermitian half spectrum -> x[N], unnormalised (FFTW convention). */
static void ORC_FN(rfft_c2r)(const ORC_FN(rfft_plan) *pl, const ORC_FN(cpx) *X,
                             ORC_R *x, ORC_FN(cpx) *work)
{
    int p = pl->p;
    if (pl->n == 1) { x[0] = X[0].re; return; }
    for (int k = 0; k < p; ++k)
    {
        ORC_FN(cpx) a = X[k];
        ORC_FN(cpx) b = X[p - k];
        b.im = -b.im;
        ORC_R er = a.re + b.re, ei = a.im + b.im;
        ORC_R dr = a.re - b.re, di = a.im - b.im;
        ORC_FN(cpx) w = pl->post[k];      /* exp(-2 pi i k/N); need the conjugate */
        ORC_R orr = dr*w.re + di*w.im;
        ORC_R oi = di*w.re - dr*w.im;
        work[k].re = er - oi;               /* Ze + i*Zo */
        work[k].im = ei + orr;
    }
    ORC_FN(cfft)(pl, work, +1);
    for (int i = 0; i < p; ++i) { x[2*i] = work[i].re; x[2*i + 1] = work[i].im; }
}
