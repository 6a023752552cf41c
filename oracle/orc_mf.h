/*
 * orc_mf.h -- CPU restatement of the reference matched filter
 * (TEST INFRASTRUCTURE ONLY; included twice by mf_oracle.c with
 * ORC_R = double and ORC_R = float).
 *
 * Follows, step for step:
 *   template preparation   src/matchedFilter.cpp:168-190 (called at :575 for
 *                          double with the template's own length and at :725
 *                          for float with the maximum template length)
 *   spectra + plans        src/matchedFilter.cpp:595-649 / :745-796
 *   dead-trace flag        src/matchedFilter.cpp:886-894
 *   overlap-add loop       src/matchedFilter.cpp:1004-1113 / :1176-1285
 *   normalisation          src/matchedFilter.cpp:94-166, driven at :1115-1139
 *                          (tol 1e-12 double) / :1287-1314 (tol 1e-6 float)
 * FFT and block length come from orc_fft_sizes (src/matchedFilterParameters.cpp:47-104).
 */

/* restates normalizeSignal, src/matchedFilter.cpp:94-166 */
static void ORC_FN(normalize_signal)(int n, int lent, const ORC_R *y, ORC_R *yNum,
                                     ORC_R tol, ORC_R tooBig)
{
    const ORC_R zero = 0;
    ORC_R *s = (ORC_R *) calloc((size_t) lent + 16, sizeof(ORC_R));
    ORC_R *s2 = (ORC_R *) calloc((size_t) lent + 16, sizeof(ORC_R));
    ORC_R scalNum = (ORC_R) sqrt((double) lent);
    int scalDen = lent;
    for (int i = 0; i < n - lent + 1; i += lent)
    {
        const ORC_R *yp = &y[i];
        ORC_R *yn = &yNum[i];
        ORC_R sum = 0, sum2 = 0;
        for (int j = 0; j < lent; ++j) { sum += yp[j]; sum2 += yp[j]*yp[j]; }
        s[0] = sum;
        s2[0] = sum2;
        for (int j = 1; j < lent; ++j)
        {
            ORC_R dm = yp[lent - 1 + j] - yp[j - 1];
            ORC_R dp = yp[lent - 1 + j] + yp[j - 1];
            s[j] = s[j - 1] + dm;
            s2[j] = s2[j - 1] + dp*dm;
        }
        for (int j = 0; j < lent; ++j)
        {
            ORC_R arg = (ORC_R) scalDen*s2[j] - s[j]*s[j];
            if (arg < zero) { arg = zero; }
            ORC_R den = (ORC_R) sqrt(arg);
            ORC_R num = scalNum*yn[j];
            ORC_R d = den > tol ? den : tol;
            yn[j] = num/d;
            if (fabs((double) yn[j]) > (double) tooBig) { yn[j] = zero; }
        }
    }
    free(s);
    free(s2);
}

/* restates demeanNormalizeAndReverseTemplate, src/matchedFilter.cpp:168-190 */
static void ORC_FN(prep_template)(int nb, const ORC_R *b, ORC_R *bOut)
{
    double mean = 0;
    for (int i = 0; i < nb; ++i) { mean += b[i]; }
    mean = (ORC_R) (mean/(double) nb);
    ORC_R norm = 0;
    for (int i = 0; i < nb; ++i)
    {
        bOut[i] = b[nb - 1 - i] - (ORC_R) mean;
        norm += bOut[i]*bOut[i];
    }
    norm = (ORC_R) sqrt(norm);
    if (norm > 0) { norm = (ORC_R) (1.0/(double) norm); }
    for (int i = 0; i < nb; ++i) { bOut[i] = bOut[i]*norm; }
}

/*
 * Full reference MatchedFilter<T>: initialize + setSignal + apply.
 *   multi      1 = MULTI_CHANNEL (signal it feeds template it), 0 = SINGLE_CHANNEL
 *   templates  nt pointers to FP64 template samples (WaveformTemplate stores FP64)
 *   signals    nt (multi) or 1 (single) pointers to n samples of type ORC_R
 *   out        nt rows of ldo samples: row t receives the filtered row starting
 *              at lag 0 (reference offset L_t-1), i.e. out[t*ldo + k] is the
 *              coefficient at lag k for k in [0, n - L_t]; ldo >= n.
 *   float_quirk 1 = prepare templates over the maximum length (float path :725)
 * Returns 0 on success.
 */
static int ORC_FN(mf_apply)(int multi, int nt, const int *lens,
                            const double *const *templates, int n,
                            const ORC_R *const *signals, ORC_R *out, long ldo,
                            int float_quirk, ORC_R tol, int nthreads)
{
    int maxLen = 0;
    for (int t = 0; t < nt; ++t) { if (lens[t] > maxLen) { maxLen = lens[t]; } }
    int nx = n + maxLen - 1;
    int nfft = 0, L = 0;
    if (orc_fft_sizes(maxLen, nx, &nfft, &L) != 0) { return -1; }
    int nspec = nfft/2 + 1;
    long ldm = nx + 64;
    ORC_FN(rfft_plan) plan;
    ORC_FN(rfft_plan_init)(&plan, nfft);
    ORC_FN(cpx) *B = (ORC_FN(cpx) *) calloc((size_t) nt*nspec, sizeof(ORC_FN(cpx)));
    {
        ORC_R *tdata = (ORC_R *) calloc((size_t) maxLen, sizeof(ORC_R));
        ORC_R *seg = (ORC_R *) calloc((size_t) nfft, sizeof(ORC_R));
        ORC_FN(cpx) *work = (ORC_FN(cpx) *) calloc((size_t) nfft/2 + 1, sizeof(ORC_FN(cpx)));
        for (int t = 0; t < nt; ++t)
        {
            memset(tdata, 0, sizeof(ORC_R)*(size_t) maxLen);
            for (int i = 0; i < lens[t]; ++i) { tdata[i] = (ORC_R) templates[t][i]; }
            memset(seg, 0, sizeof(ORC_R)*(size_t) nfft);
            ORC_FN(prep_template)(float_quirk ? maxLen : lens[t], tdata, seg);
            ORC_FN(rfft_r2c)(&plan, seg, &B[(size_t) t*nspec], work);
        }
        free(tdata); free(seg); free(work);
    }
    int nsig = multi ? nt : 1;
    ORC_R *Y = (ORC_R *) calloc((size_t) nsig*ldm, sizeof(ORC_R));
    unsigned char *dead = (unsigned char *) calloc((size_t) nt, 1);
    for (int s = 0; s < nsig; ++s)
    {
        ORC_R mn = signals[s][0], mx = signals[s][0];
        for (int i = 0; i < n; ++i)
        {
            ORC_R v = signals[s][i];
            Y[(size_t) s*ldm + i] = v;
            if (v < mn) { mn = v; }
            if (v > mx) { mx = v; }
        }
        if (fabs((double) mn) == fabs((double) mx))
        {
            /* SingleChannel::MatchedFilter::setSignal always writes signal
               slot 0 (src/singleChannel/matchedFilter.cpp:62-67), so only
               template 0 carries the dead flag in single-channel mode. */
            dead[s] = 1;
        }
    }
    ORC_R *F = (ORC_R *) calloc((size_t) nt*ldm, sizeof(ORC_R));
    ORC_R xnorm = (ORC_R) (1.0/(double) nfft);
    ORC_FN(cpx) *Xs = (ORC_FN(cpx) *) calloc((size_t) nsig*nspec, sizeof(ORC_FN(cpx)));
    for (int istart = 0; istart < nx; istart += L)
    {
        int iend = istart + L < nx ? istart + L : nx;
        int ncopy = iend - istart;
        int yend = istart + nfft < nx ? istart + nfft : nx;
        int nupdate = yend - istart;
        #pragma omp parallel for num_threads(nthreads) schedule(static)
        for (int s = 0; s < nsig; ++s)
        {
            ORC_R *seg = (ORC_R *) calloc((size_t) nfft, sizeof(ORC_R));
            ORC_FN(cpx) *work = (ORC_FN(cpx) *) malloc(sizeof(ORC_FN(cpx))*(size_t) nspec);
            memcpy(seg, &Y[(size_t) s*ldm + istart], sizeof(ORC_R)*(size_t) ncopy);
            ORC_FN(rfft_r2c)(&plan, seg, &Xs[(size_t) s*nspec], work);
            free(seg); free(work);
        }
        #pragma omp parallel for num_threads(nthreads) schedule(static)
        for (int t = 0; t < nt; ++t)
        {
            ORC_FN(cpx) *Xt = (ORC_FN(cpx) *) malloc(sizeof(ORC_FN(cpx))*(size_t) nspec);
            ORC_FN(cpx) *work = (ORC_FN(cpx) *) malloc(sizeof(ORC_FN(cpx))*(size_t) nspec);
            ORC_R *yseg = (ORC_R *) malloc(sizeof(ORC_R)*(size_t) nfft);
            const ORC_FN(cpx) *X = &Xs[(size_t) (multi ? t : 0)*nspec];
            const ORC_FN(cpx) *Bt = &B[(size_t) t*nspec];
            /* plain product B*X (templates were reversed), :1038-1051 */
            for (int w = 0; w < nspec; ++w)
            {
                Xt[w].re = Bt[w].re*X[w].re - Bt[w].im*X[w].im;
                Xt[w].im = Bt[w].re*X[w].im + Bt[w].im*X[w].re;
            }
            ORC_FN(rfft_c2r)(&plan, Xt, yseg, work);
            ORC_R *ydst = &F[(size_t) t*ldm + istart];
            for (int i = 0; i < nupdate; ++i) { ydst[i] = ydst[i] + yseg[i]*xnorm; }
            free(Xt); free(work); free(yseg);
        }
    }
    #pragma omp parallel for num_threads(nthreads) schedule(dynamic)
    for (int t = 0; t < nt; ++t)
    {
        if (dead[t]) { continue; }
        const ORC_R *y = &Y[(size_t) (multi ? t : 0)*ldm];
        ORC_FN(normalize_signal)(n, lens[t], y, &F[(size_t) t*ldm + lens[t] - 1], tol, (ORC_R) 1.1);
    }
    for (int t = 0; t < nt; ++t)
    {
        const ORC_R *src = &F[(size_t) t*ldm + lens[t] - 1];
        int nv = n - lens[t] + 1;
        for (int k = 0; k < nv; ++k) { out[(size_t) t*ldo + k] = src[k]; }
        for (long k = nv; k < ldo; ++k) { out[(size_t) t*ldo + k] = 0; }
    }
    free(Xs); free(F); free(Y); free(dead); free(B);
    ORC_FN(rfft_plan_free)(&plan);
    return 0;
}
