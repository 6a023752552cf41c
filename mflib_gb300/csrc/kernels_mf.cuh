// kernels_mf.cuh -- matched-filter kernels (templated on the sample type).
//
// Design (GB300, one CTA per (signal block, channel, template group)):
//   * Overlap-save instead of the reference's overlap-add: block b of a
//     channel reads samples [b*S, b*S + N) and yields the S lags
//     [b*S, b*S + S) of every template on that channel, S <= N - Lmax + 1.
//     No block writes another block's outputs, so nothing is accumulated in
//     HBM (the reference accumulates y[istart+i] += ... across blocks,
//     src/matchedFilter.cpp:1093-1112).
//   * The N-sample segment and the plan's twiddle table are staged into
//     shared memory by TMA bulk copies (cp.async.bulk + mbarrier, bounded
//     wait); the next template's spectrum is prefetched the same way while
//     the current one is transformed.
//   * The segment mean m is subtracted before both the FFT and the sliding
//     sums.  The numerator is invariant to it (templates are zero-mean,
//     src/matchedFilter.cpp:172-189) and so is the window variance, but the
//     FP32 rounding error of both no longer scales with the DC level.
//   * Sliding-window sums of y and y^2 over each template length
//     (normalizeSignal, src/matchedFilter.cpp:94-166) are accumulated in
//     double-float for FP32 data (about 48 significant bits; GB300's FP64
//     rate is a small fraction of its FP32 rate) and in double for FP64 data.
//   * Forward real FFT of the segment once.  Per template the conj(B_t)/N
//     multiply and the inverse real-FFT pre-processing are fused into the
//     first inverse pass, and the Pearson epilogue
//     rho = sqrt(L) num / max(tol, sqrt(max(0, L s2 - s1^2))), rho := 0 when
//     |rho| > 1.1, is fused into the last pass (coalesced 2-lag stores).
#pragma once
#include "fft_stockham.cuh"
#include "kernels_util.cuh"

namespace mfgpu {

constexpr int kThreads = 256;

// power-of-two scale that maps |v| <= range onto |v * s| < 2^e
__device__ __forceinline__ float tc_pow2_scale(float range, int e)
{
    if (!(range > 0.f) || !isfinite(range)) return 1.f;
    int ex;
    frexpf(range, &ex);  // range < 2^ex
    return ldexpf(1.f, e - ex);
}

template <class T> struct XcorrParams
{
    const T *x;               // channel signals, row stride ldx (zero padded tail)
    long ldx;
    const cx<T> *Bc;          // conj(spectrum)/N of each template, row stride ldb = P + 2
    long ldb;
    T *rho;                   // output rows, stride ldr
    long ldr;
    const int *grp_chan;      // work group g: channel grp_chan[g] and templates
    const int *grp_tb;        //   tids[grp_tb[g] .. grp_te[g])
    const int *grp_te;
    const int *tids;
    const int *tlen;          // template lengths
    const int *nvalid;        // valid lags per template (n - L_t + 1)
    const unsigned char *dead;// dead-trace flag per channel
    const cx<T> *twt;         // twiddle table of the plan (FftPlan layout)
    const cx<T> *twt_split;   // mode 4: pass twiddles in the split layout (FftPlan::tws_off)
    const T *den;             // SHARED_DEN: sqrt(L)/max(tol, den) per channel and lag, row stride ldd
    long ldd;
    int S;                    // lags per block (multiple of 32)
    T tol;
    int *err;
    // fused peak candidates (pk_on != 0): lags [k0+1, k0+S-2] of block b of
    // template t that pass the candidate rule on a trace of pk_len lags with
    // threshold pk_thr go to slot (t * pk_stride + b): count pk_cnt (zeroed
    // before the launch; may exceed kPkCap), up to kPkCap (index, value)
    // pairs in pk_idx / pk_val, in no particular order.
    int pk_on;
    int pk_stride;
    int pk_len;
    T pk_thr;
    int *pk_cnt;
    int *pk_idx;
    T *pk_val;
    // test of the bounded-wait error path: expect the segment copy's bytes
    // without issuing the copy (nothing in flight) and give up after a short
    // wait, reporting KERR_TMA_TIMEOUT
    int test_skip_copy;
    // persistent launch: a device ticket (0 before the launch) handing out
    // ntiles tiles, block t % nblk of work group t / nblk; null: grid launch
    int *ticket;
    int ntiles;
    int nblk;
};

template <class T> struct SpecParams
{
    const double *tmpl;       // concatenated FP64 template samples
    const long *toff;         // offset of each template
    const int *tlen;
    cx<T> *Bc;
    long ldb;
    const cx<T> *twt;
};

// Shared-memory carve-up of the correlator (used by host and device).
//   head | xs (staged segment; with SD also the first FFT work buffer W0) |
//   [W0] | [W1 (MODE 2, 3, 4)] | UV (per-bin U, V pairs of the block spectrum) |
//   pass twiddles | [2 spectrum buffers (MODE 1)] | invd (two rows in MODE 4)
// MODE 0: whole CTA per transform, spectra read from L2;  MODE 1: whole CTA,
// spectra TMA-prefetched;  MODE 2: two 128-thread teams transform different
// templates with their own named barriers, spectra read from L2;  MODE 4:
// 512 threads, two 256-thread teams, each normalising its own templates
// (several lengths), pass twiddles in the split layout.
template <class T, int LOG2P> struct XcorrLayout
{
    using acc = typename acc_t<T>::type;
    static constexpr int P = 1 << LOG2P, N = 2 * P, NCH = N / 32;
    static constexpr size_t up(size_t v) { return (v + 127) & ~size_t(127); }
    static constexpr size_t seg = sizeof(T) * N;
    static constexpr size_t fft = sizeof(cx<T>) * spad_size(P);
    // after the chunk prefixes: two rows of NCH values (per-chunk partial
    // sums, or in mode 4 the chunk totals of y and y^2)
    static constexpr size_t head(bool sd, int mode = 0)
    {
        return up(64 + 32 * sizeof(T) + (sd ? 0 : 2 * sizeof(acc) * (NCH + 1) + 2 * sizeof(T) * NCH));
    }
    // pass twiddles only; mode 4 holds them in the split layout (FftPlan::tws_off)
    static constexpr size_t tw_bytes_of(int mode)
    {
        return sizeof(cx<T>) * (mode == 4 ? FftPlan<LOG2P>::tws_total() : FftPlan<LOG2P>::post_off());
    }
    static constexpr size_t tw_bytes = tw_bytes_of(0);
    static constexpr size_t uv = sizeof(cx<T>) * 2 * P;
    static constexpr size_t brow = sizeof(cx<T>) * (P + 2);
    // With SHARED_DEN, and in mode 3, the first work buffer overlays the
    // segment; mode 3 builds a padded demeaned copy in the second team's
    // buffer before the forward FFT.
    static constexpr size_t padded = sizeof(T) * (N + N / 32);
    // Without SHARED_DEN (modes 0, 1, 4: templates of several lengths) the
    // segment's region holds, after the forward FFT, the in-chunk prefix sums
    // of y and y^2, interleaved (2 N values, and a zero pair at position N:
    // the prefix where the last lag's window ends), and the CTA (each team in
    // mode 4) keeps 8 values per 32-lag run of its template's window
    // statistics
    static constexpr size_t q12 = sizeof(T) * 2 * (N + 2);
    static __host__ __device__ size_t rd_bytes(int S) { return up(8 * sizeof(T) * (size_t) (S / 32)); }
    static_assert(((sizeof(cx<T>) * spad_size(P) + 127) & ~size_t(127)) >= sizeof(T) * (N + N / 32),
                  "a work buffer holds the padded segment");
    static constexpr bool overlay(bool sd, int mode) { return sd || mode == 3; }
    static constexpr bool teams(int mode) { return mode >= 2; }
    static constexpr size_t xs_region(bool sd, int mode)
    {
        return up(overlay(sd, mode) ? (seg > fft ? seg : fft) : q12);
    }
    static constexpr size_t off_xs(bool sd, int mode = 0) { return head(sd, mode); }
    static constexpr size_t off_W0(bool sd, int mode)
    {
        return off_xs(sd, mode) + (overlay(sd, mode) ? 0 : xs_region(sd, mode));
    }
    static constexpr size_t off_W1(bool sd, int mode)
    {
        return off_xs(sd, mode) + xs_region(sd, mode) + (overlay(sd, mode) ? 0 : up(fft));
    }
    static constexpr size_t off_UV(bool sd, int mode) { return off_W1(sd, mode) + (teams(mode) ? up(fft) : 0); }
    static constexpr size_t off_tw(bool sd, int mode) { return off_UV(sd, mode) + up(uv); }
    static constexpr size_t off_B(bool sd, int mode) { return off_tw(sd, mode) + up(tw_bytes_of(mode)); }
    static constexpr size_t off_invd(bool sd, int mode) { return off_B(sd, mode) + (mode == 1 ? 2 * up(brow) : 0); }
    // one normalisation row (one template length), else run statistics:
    // one row, or one per team in mode 4
    static __host__ __device__ size_t invd_bytes(bool sd, int mode, int S)
    {
        return overlay(sd, mode) ? up(sizeof(T) * (size_t) S) : (mode == 4 ? 2 : 1) * rd_bytes(S);
    }
    // fused peak candidates: per team two chunk masks (one bit per 64 lags,
    // P/32 chunks)
    static constexpr int mask_words = (P / 32 + 31) / 32;
    static __host__ __device__ size_t off_M(bool sd, int mode, int S)
    {
        return off_invd(sd, mode) + invd_bytes(sd, mode, S);
    }
    static size_t bytes(bool sd, int mode, int S)
    {
        return off_M(sd, mode, S) + sizeof(unsigned) * 2 * (teams(mode) ? 2 : 1) * mask_words;
    }
};

// Compensated sum for block means: FP32 values accumulate in double-float
// (one TwoSum per value, low words summed), FP64 in double.  A block of
// identical samples gets exactly that sample as its mean, so the mean
// subtraction leaves exact zeros (and, for nearly constant blocks, no
// residual offset that would dominate the block's energy).
template <class T> struct MeanAcc;
template <> struct MeanAcc<float>
{
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add(float v)
    {
        const df s = two_sum(hi, v);
        hi = s.hi;
        lo += s.lo;
    }
    __device__ __forceinline__ void add(const MeanAcc &o)
    {
        const df s = two_sum(hi, o.hi);
        hi = s.hi;
        lo += s.lo + o.lo;
    }
    __device__ __forceinline__ MeanAcc shfl_xor(int o) const
    {
        MeanAcc r;
        r.hi = __shfl_xor_sync(0xffffffffu, hi, o);
        r.lo = __shfl_xor_sync(0xffffffffu, lo, o);
        return r;
    }
    __device__ __forceinline__ float mean(int n) const
    {
        const df q = quick_two_sum(hi, lo);
        return q.hi / (float) n + q.lo / (float) n;
    }
};
template <> struct MeanAcc<double>
{
    double s = 0.0;
    __device__ __forceinline__ void add(double v) { s += v; }
    __device__ __forceinline__ void add(const MeanAcc &o) { s += o.s; }
    __device__ __forceinline__ MeanAcc shfl_xor(int o) const
    {
        MeanAcc r;
        r.s = __shfl_xor_sync(0xffffffffu, s, o);
        return r;
    }
    __device__ __forceinline__ double mean(int n) const { return s / (double) n; }
};

// block-wide mean of n values from the per-thread accumulators; red holds
// at least 2 * kThreads / 32 values of T
// (NTH threads in the CTA; red holds at least 2 * NTH / 32 values of T)
template <class T, int NTH = kThreads> __device__ __forceinline__ T block_mean(MeanAcc<T> a, T *red, int n)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a.add(a.shfl_xor(o));
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    MeanAcc<T> *r = reinterpret_cast<MeanAcc<T> *>(red);
    __syncthreads();
    if (l == 0) r[w] = a;
    __syncthreads();
    MeanAcc<T> t = r[0];
#pragma unroll
    for (int i = 1; i < NTH / 32; ++i) t.add(r[i]);
    return t.mean(n);
}

template <class T> __device__ __forceinline__ T block_sum(T v, T *red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    T s = 0;
#pragma unroll
    for (int i = 0; i < kThreads / 32; ++i) s += red[i];
    return s;
}

// real-FFT post-processing in place: A[0..P-1] holds Z = FFT_P(x_even + i x_odd);
// on return A[k] = X[k] for k = 0..P (X[P] in the spare slot spad(P)).
template <class T, int LOG2P>
__device__ __forceinline__ void rfft_post(cx<T> *A, const cx<T> *post, int tid)
{
    constexpr int P = 1 << LOG2P;
    for (int k = tid; k <= P / 2; k += kThreads)
    {
        if (k == 0)
        {
            cx<T> z = A[0];
            A[0] = cmk(z.x + z.y, (T) 0);
            A[spad(P)] = cmk(z.x - z.y, (T) 0);
            continue;
        }
        cx<T> zk = A[spad(k)], zp = A[spad(P - k)];
        cx<T> E = cscale(zk + cconj(zp), (T) 0.5);
        cx<T> D = cscale(zk - cconj(zp), (T) 0.5);
        cx<T> O = cmk(D.y, -D.x);  // D / i
        cx<T> wO = cmul(post[k], O);
        A[spad(k)] = E + wO;
        A[spad(P - k)] = cconj(E - wO);
    }
}

// ----------------------------------------------------------------------------
// Template spectra: demean and unit-normalise the template in FP64
// (src/matchedFilter.cpp:168-190; the double path uses the template's own
// length, :575), zero pad to N, forward real FFT, store conj(B)/N for
// k = 0..P.  The template is not reversed: correlation uses conj(B).
template <class T, int LOG2P>
__global__ void __launch_bounds__(kThreads) template_spectra_kernel(SpecParams<T> p)
{
    constexpr int P = 1 << LOG2P;
    constexpr int N = 2 * P;
    extern __shared__ __align__(16) unsigned char smem_spec[];
    cx<T> *A = reinterpret_cast<cx<T> *>(smem_spec);
    double *red = reinterpret_cast<double *>(smem_spec + sizeof(cx<T>) * spad_size(P));
    const int t = blockIdx.x, tid = threadIdx.x;
    const int L = p.tlen[t];
    const double *b = p.tmpl + p.toff[t];
    double s = 0;
    for (int i = tid; i < L; i += kThreads) s += b[i];
    const double mean = block_sum<double>(s, red) / (double) L;
    double q = 0;
    for (int i = tid; i < L; i += kThreads) { double d = b[i] - mean; q += d * d; }
    const double nrm2 = block_sum<double>(q, red);
    const double inv = nrm2 > 0 ? 1.0 / sqrt(nrm2) : 0.0;
    auto ld = [&](int e) -> cx<T> {
        T re = 0, im = 0;
        if (2 * e < L) re = (T) ((b[2 * e] - mean) * inv);
        if (2 * e + 1 < L) im = (T) ((b[2 * e + 1] - mean) * inv);
        return cmk(re, im);
    };
    auto st = [&](int e, cx<T> v) { A[spad(e)] = v; };
    fft_run<T, LOG2P, kThreads, false, true>(A, p.twt, tid, ld, st);
    __syncthreads();
    rfft_post<T, LOG2P>(A, p.twt + FftPlan<LOG2P>::post_off(), tid);
    __syncthreads();
    const T scale = (T) (1.0 / (double) N);
    cx<T> *out = p.Bc + (long) t * p.ldb;
    for (int k = tid; k <= P; k += kThreads) out[k] = cscale(cconj(A[spad(k)]), scale);
}

// ----------------------------------------------------------------------------
// Sliding-window statistics of the staged segment.
// Window-sum arithmetic shared by the per-channel normalisation kernel and
// the correlator's in-CTA normalisation (several template lengths).
// Shared-memory sample layouts pad one word per 32 samples.
__host__ __device__ constexpr int den_pad(int i) { return i + (i >> 5); }
template <class T> struct DenOps;
template <> struct DenOps<float>
{
    using acc = df;
    // run sums with deferred low words
    struct Run { float h1, l1, h2, l2; };
    static __device__ __forceinline__ Run run_zero() { return Run{0.f, 0.f, 0.f, 0.f}; }
    static __device__ __forceinline__ df zero() { return df{0.f, 0.f}; }
    static __device__ __forceinline__ void run_add(Run &s, float v)
    {
        const float t = s.h1 + v, bb = t - s.h1;
        s.l1 += (s.h1 - (t - bb)) + (v - bb);
        s.h1 = t;
        const float p = v * v, pe = fmaf(v, v, -p);
        const float u = s.h2 + p, b2 = u - s.h2;
        s.l2 += ((s.h2 - (u - b2)) + (p - b2)) + pe;
        s.h2 = u;
    }
    static __device__ __forceinline__ df s1(const Run &s) { return quick_two_sum(s.h1, s.l1); }
    static __device__ __forceinline__ df s2(const Run &s) { return quick_two_sum(s.h2, s.l2); }
    // addition for the scans: one TwoSum, low words added (about 44 bits)
    static __device__ __forceinline__ df add(df a, df b)
    {
        df s = two_sum(a.hi, b.hi);
        s.lo += a.lo + b.lo;
        return quick_two_sum(s.hi, s.lo);
    }
    static __device__ __forceinline__ df neg(df a) { return df{-a.hi, -a.lo}; }
    static __device__ __forceinline__ df shfl_up(df a, int d)
    {
        return df{__shfl_up_sync(0xffffffffu, a.hi, d), __shfl_up_sync(0xffffffffu, a.lo, d)};
    }
    // V = L s2 - s1^2 as (hi, lo)
    static __device__ __forceinline__ void var0(df w1, df w2, int L, float &vh, float &vl)
    {
        df a = two_prod((float) L, w2.hi);
        a.lo = fmaf((float) L, w2.lo, a.lo);
        df b = two_prod(w1.hi, w1.hi);
        b.lo = fmaf(2.f * w1.hi, w1.lo, b.lo);
        const df v = two_sum(a.hi, -b.hi);
        vh = v.hi;
        vl = v.lo + (a.lo - b.lo);
    }
    static __device__ __forceinline__ float hi(df a) { return a.hi; }
    // a window with V <= 0 is constant (the sums are exact there) and its
    // exact numerator against a zero-mean template is 0: rho = 0 instead of
    // the numerator's rounding error times sqrt(L)/tol
    static __device__ __forceinline__ float out(float var, float sqrtL, float tol)
    {
        return var > tol * tol ? sqrtL * rsqrtf(var) : (var > 0.f ? sqrtL / tol : 0.f);
    }
};
template <> struct DenOps<double>
{
    using acc = double;
    struct Run { double a1, a2; };
    static __device__ __forceinline__ Run run_zero() { return Run{0.0, 0.0}; }
    static __device__ __forceinline__ double zero() { return 0.0; }
    static __device__ __forceinline__ void run_add(Run &s, double v)
    {
        s.a1 += v;
        s.a2 = fma(v, v, s.a2);
    }
    static __device__ __forceinline__ double s1(const Run &s) { return s.a1; }
    static __device__ __forceinline__ double s2(const Run &s) { return s.a2; }
    static __device__ __forceinline__ double add(double a, double b) { return a + b; }
    static __device__ __forceinline__ double neg(double a) { return -a; }
    static __device__ __forceinline__ double shfl_up(double a, int d) { return __shfl_up_sync(0xffffffffu, a, d); }
    static __device__ __forceinline__ void var0(double w1, double w2, int L, double &vh, double &vl)
    {
        vh = fma((double) L, w2, -w1 * w1);
        vl = 0.0;
    }
    static __device__ __forceinline__ double hi(double a) { return a; }
    // sqrt(L) / max(sqrt(V), tol) as in the reference; the common branch
    // with one reciprocal square root instead of a square root and a
    // division (FP64 arithmetic is costly on this GPU)
    static __device__ __forceinline__ double out(double var, double sqrtL, double tol)
    {
        return var > tol * tol ? sqrtL * rsqrt(var) : (var > 0.0 ? sqrtL / tol : 0.0);
    }
};

template <class T> struct SegStats
{
    using A = acc_t<T>;
    using acc = typename A::type;
    const T *xs;   // raw segment, N samples (until the forward FFT)
    T *yp;         // after the forward FFT: demeaned segment, one pad word per 32 (den_pad)
    T m;           // segment mean
    acc *c1, *c2;  // chunk prefix sums of (x - m) (N/32 + 1 entries each)
    T *p1, *p2;    // per chunk: sums of the first L mod 32 samples (N/32 entries each)
};

// Chunk sums over 32 samples with a per-lane skew (conflict-free banks),
// then an exclusive scan by warp 0.
template <class T, int N, int NTH = kThreads>
__device__ __forceinline__ void seg_chunk_prefix(SegStats<T> st, int tid)
{
    using A = acc_t<T>;
    using acc = typename A::type;
    constexpr int NCH = N / 32;
    const int lane = tid & 31;
    for (int j = tid; j < NCH; j += NTH)
    {
        acc s1 = A::zero(), s2 = A::zero();
        const T *xp = st.xs + 32 * j;
#pragma unroll 8
        for (int i = 0; i < 32; ++i)
        {
            T v = xp[(i + lane) & 31] - st.m;
            s1 = A::add_val(s1, v);
            s2 = A::add_sq(s2, v);
        }
        st.c1[j + 1] = s1;
        st.c2[j + 1] = s2;
    }
    __syncthreads();
    if (tid < 32)
    {
        constexpr int PER = (NCH + 31) / 32;
        acc v1[PER], v2[PER];
        acc r1 = A::zero(), r2 = A::zero();
#pragma unroll
        for (int i = 0; i < PER; ++i)
        {
            int j = lane * PER + i;
            v1[i] = j < NCH ? st.c1[j + 1] : A::zero();
            v2[i] = j < NCH ? st.c2[j + 1] : A::zero();
            r1 = A::add(r1, v1[i]);
            r2 = A::add(r2, v2[i]);
        }
        __syncwarp();
        // inclusive warp scan of lane totals
        acc i1 = r1, i2 = r2;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            acc u1 = A::shfl_up(i1, o), u2 = A::shfl_up(i2, o);
            if (lane >= o) { i1 = A::add(i1, u1); i2 = A::add(i2, u2); }
        }
        acc e1 = A::shfl_up(i1, 1), e2 = A::shfl_up(i2, 1);  // exclusive offsets
        if (lane == 0) { e1 = A::zero(); e2 = A::zero(); }
        // rewrite chunk sums as exclusive prefixes: c[j] = sum_{i<j} chunk_i
#pragma unroll
        for (int i = 0; i < PER; ++i)
        {
            int j = lane * PER + i;
            if (j < NCH)
            {
                st.c1[j] = e1;
                st.c2[j] = e2;
                e1 = A::add(e1, v1[i]);
                e2 = A::add(e2, v2[i]);
                if (j == NCH - 1) { st.c1[NCH] = e1; st.c2[NCH] = e2; }
            }
        }
    }
    __syncthreads();
}

// Rewrites the staged segment (free once the forward FFT has read it) as
// y = x - m with one pad word per 32 samples, for conflict-free strided
// reads by seg_inv_den.  The padded copy (st.yp) fits the segment's region
// or one FFT work buffer.
template <class T, int N, int NTH = kThreads>
__device__ __forceinline__ void seg_make_padded(SegStats<T> st, int tid)
{
    constexpr int PER = (N + NTH - 1) / NTH;
    T v[PER];
#pragma unroll
    for (int i = 0; i < PER; ++i)
    {
        const int e = tid + i * NTH;
        v[i] = e < N ? st.xs[e] - st.m : (T) 0;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < PER; ++i)
    {
        const int e = tid + i * NTH;
        if (e < N) st.yp[den_pad(e)] = v[i];
    }
    __syncthreads();
}

// invd[k] = sqrt(L)/max(tol, sqrt(V_k)), V_k = L s2 - s1^2 over [k, k+L),
// 0 where V_k <= 0 (a constant window), for k in [0, S) (S a multiple of
// 32), from the padded demeaned segment: exact (double-float / double)
// window sums at each 32-lag run start -- chunk prefixes plus the partial
// sums of the first L mod 32 samples of a chunk -- then 32 lags of
// corrections in the data type (DenOps; the same scheme as den_kernel).
// Ends with a barrier.
template <class T, int N, int NT = kThreads, int BAR = 0>
__device__ __forceinline__ void seg_inv_den(SegStats<T> st, int L, int S, T tol, T *invd, int tid, int bar_id = 0)
{
    using A = acc_t<T>;
    using O = DenOps<T>;
    using acc = typename A::type;
    constexpr int NCH = N / 32;
    const int Lq = L >> 5, re = L & 31;
    for (int j = tid; j < NCH; j += NT)
    {
        T a = 0, b = 0;
        const T *yc = st.yp + 33 * j;
        for (int i = 0; i < re; ++i)
        {
            const T v = yc[i];
            a += v;
            b = fma(v, v, b);
        }
        st.p1[j] = a;
        st.p2[j] = b;
    }
    team_sync<BAR, NT>(bar_id);
    const T sqrtL = sqrt((T) L), Lt = (T) L;
    for (int v = tid; v < S / 32; v += NT)
    {
        const acc w1 = A::add_val(A::sub(st.c1[v + Lq], st.c1[v]), st.p1[v + Lq]);
        const acc w2 = A::add_val(A::sub(st.c2[v + Lq], st.c2[v]), st.p2[v + Lq]);
        T vh, vl;
        O::var0(w1, w2, L, vh, vl);
        const T c2s = (T) 2 * O::hi(w1);
        T d1 = 0, d2 = 0;
        T o[32];
        const int base = 32 * v;
#pragma unroll
        for (int q = 0; q < 32; ++q)
        {
            const T var = vh + (vl + fma(Lt, d2, -d1 * (d1 + c2s)));
            o[q] = O::out(var, sqrtL, tol);
            if (q < 31)
            {
                const T yin = st.yp[den_pad(base + q + L)], yout = st.yp[den_pad(base + q)];
                const T dd = yin - yout;
                d2 = fma(yin + yout, dd, d2);
                d1 += dd;
            }
        }
        // the row's 16-byte chunks are stored XOR-swizzled by the run index
        // (chunk c at c ^ (v & 7)): the eight threads of a wavefront then
        // hit eight different bank groups instead of one; inv_den_pair()
        // undoes it
        T *dst = invd + base;
        const int sw = v & 7;
        if constexpr (sizeof(T) == 4)
        {
#pragma unroll
            for (int q = 0; q < 32; q += 4)
                *reinterpret_cast<float4 *>(dst + (((q >> 2) ^ sw) << 2)) =
                    make_float4(o[q], o[q + 1], o[q + 2], o[q + 3]);
        }
        else
        {
#pragma unroll
            for (int q = 0; q < 32; q += 2)
                *reinterpret_cast<double2 *>(dst + (((q >> 1) ^ sw) << 1)) = make_double2(o[q], o[q + 1]);
        }
    }
    team_sync<BAR, NT>(bar_id);
}

// Index of the pair (lags 2e, 2e + 1) in a normalisation row written by
// seg_inv_den (rows of 32 lags, 16-byte chunks swizzled by the row index)
template <class T> __device__ __forceinline__ int inv_den_pair(int e)
{
    if constexpr (sizeof(T) == 4) return e ^ ((e >> 3) & 14);  // 2 pairs per chunk, 8 chunks per row
    else return e ^ ((e >> 4) & 7);                             // 1 pair per chunk, 16 chunks per row
}

template <class T> __device__ __forceinline__ void store2(T *dst, T a, T b);
template <> __device__ __forceinline__ void store2<float>(float *dst, float a, float b)
{
    *reinterpret_cast<float2 *>(dst) = make_float2(a, b);
}
template <> __device__ __forceinline__ void store2<double>(double *dst, double a, double b)
{
    *reinterpret_cast<double2 *>(dst) = make_double2(a, b);
}

template <class T> __device__ __forceinline__ T clamp_rho(T v) { return fabs(v) > (T) 1.1 ? (T) 0 : v; }

// four consecutive values (16-byte aligned) in vector loads / stores
template <class T> struct vec4;
template <> struct vec4<float>
{
    static __device__ __forceinline__ void load(const float *p, float (&v)[4])
    {
        const float4 a = *reinterpret_cast<const float4 *>(p);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    }
    static __device__ __forceinline__ void store(float *p, const float (&v)[4])
    {
        *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
    }
};
template <> struct vec4<double>
{
    static __device__ __forceinline__ void load(const double *p, double (&v)[4])
    {
        const double2 a = reinterpret_cast<const double2 *>(p)[0], b = reinterpret_cast<const double2 *>(p)[1];
        v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
    }
    static __device__ __forceinline__ void store(double *p, const double (&v)[4])
    {
        reinterpret_cast<double2 *>(p)[0] = make_double2(v[0], v[1]);
        reinterpret_cast<double2 *>(p)[1] = make_double2(v[2], v[3]);
    }
};

// two consecutive complex values in one 16-byte shared load (FP32)
template <class T> __device__ __forceinline__ void load_pair(const cx<T> *p, cx<T> &a, cx<T> &b);
template <> __device__ __forceinline__ void load_pair<float>(const cx<float> *p, cx<float> &a, cx<float> &b)
{
    const float4 q = *reinterpret_cast<const float4 *>(p);
    a = cmk(q.x, q.y);
    b = cmk(q.z, q.w);
}
template <> __device__ __forceinline__ void load_pair<double>(const cx<double> *p, cx<double> &a, cx<double> &b)
{
    a = p[0];
    b = p[1];
}

// Mode 4 (each template normalised for its own length) keeps no
// normalisation rows.  Once per CTA, after the forward FFT has read the
// staged segment, its region is rewritten as the in-chunk exclusive prefix
// sums of y = x - m and y^2, interleaved: q12[k] = (sum, sum of squares of
// y[32 (k/32) .. k)), one warp scan per 32-sample chunk, q12[N] = q12[N + 1]
// = 0 (a window ending at the segment's end reads q12[N]), and the chunk
// totals go to tot1 / tot2.  Ends with a barrier.
template <class T, int N, int NTH>
__device__ __forceinline__ void seg_prefix_q12(SegStats<T> st, cx<T> *q12, T *tot1, T *tot2, int tid)
{
    constexpr int NCH = N / 32, NW = NTH / 32, CPW = (NCH + NW - 1) / NW;
    const int w = tid >> 5, lane = tid & 31;
    T v[CPW];
#pragma unroll
    for (int i = 0; i < CPW; ++i)
    {
        const int j = w + i * NW;
        v[i] = j < NCH ? st.xs[32 * j + lane] - st.m : (T) 0;
    }
    __syncthreads();  // q12 overlays the segment
    if (tid < 2) q12[N + tid] = cmk((T) 0, (T) 0);
#pragma unroll
    for (int i = 0; i < CPW; ++i)
    {
        const int j = w + i * NW;
        if (j >= NCH) break;
        T a = v[i], b = v[i] * v[i];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const T ua = __shfl_up_sync(0xffffffffu, a, o), ub = __shfl_up_sync(0xffffffffu, b, o);
            if (lane >= o) { a += ua; b += ub; }
        }
        const T ea = __shfl_up_sync(0xffffffffu, a, 1), eb = __shfl_up_sync(0xffffffffu, b, 1);
        q12[32 * j + lane] = lane ? cmk(ea, eb) : cmk((T) 0, (T) 0);
        if (lane == 31)
        {
            tot1[j] = a;
            tot2[j] = b;
        }
    }
    __syncthreads();
}

// Per 32-lag run v of a template of length L = 32 Lq + re (mode 4): the
// exact (double-float) window statistics at the run's first lag 32 v, as in
// seg_inv_den -- chunk prefixes of chunks [v, j), j = v + Lq, plus the first
// re samples of chunk j -- stored as rd[4v..4v+3] = (V0 hi, V0 lo), (2 W1
// hi, 0), (-a1, t1 - a1), (-a2, t2 - a2): a = the partial sums of chunk j
// up to re, t = its totals.  Lag 32 v + q of the run then needs only the
// prefix sums at its head and tail (inv_den_wide).
template <class T, int NTT>
__device__ __forceinline__ void seg_run_stats(SegStats<T> st, const cx<T> *q12, const T *tot1, const T *tot2, int L,
                                              int S, cx<T> *rd, int ttid)
{
    using A = acc_t<T>;
    using O = DenOps<T>;
    const int Lq = L >> 5, re = L & 31;
    for (int v = ttid; v < S / 32; v += NTT)
    {
        const int j = v + Lq;
        const cx<T> a = q12[32 * j + re];
        const auto w1 = A::add_val(A::sub(st.c1[j], st.c1[v]), a.x);
        const auto w2 = A::add_val(A::sub(st.c2[j], st.c2[v]), a.y);
        T vh, vl;
        O::var0(w1, w2, L, vh, vl);
        rd[4 * v] = cmk(vh, vl);
        rd[4 * v + 1] = cmk((T) 2 * O::hi(w1), (T) 0);
        rd[4 * v + 2] = cmk(-a.x, tot1[j] - a.x);
        rd[4 * v + 3] = cmk(-a.y, tot2[j] - a.y);
    }
}

// sqrt(L)/max(tol, sqrt(V)) for the lags k and k + 1 (k even) of a template
// of length L = 32 Lq + re, from its run statistics (seg_run_stats) and the
// prefix sums: the window moved by q = k mod 32 lags from the run start
// gained sum y over [32 v + L, k + L) and lost it over [32 v, k), so
//   V(k) = V0 + L d2 - d1 (d1 + 2 W1),  d = (tail prefix - a (+ t when k + L
// passed into chunk j + 1)) - head prefix,
// the same correction the sliding form accumulates, here without a serial
// chain.
template <class T>
__device__ __forceinline__ cx<T> inv_den_wide(const cx<T> *q12, const cx<T> *rd, int k, int L, int re, T Lt,
                                              T sqrtL, T tol)
{
    using O = DenOps<T>;
    const int v = k >> 5, q = k & 31;
    cx<T> r0, r1, ra, rb, h0, h1, t0, t1;
    load_pair<T>(rd + 4 * v, r0, r1);
    load_pair<T>(rd + 4 * v + 2, ra, rb);
    load_pair<T>(q12 + k, h0, h1);
    if ((L & 1) == 0) load_pair<T>(q12 + k + L, t0, t1);
    else { t0 = q12[k + L]; t1 = q12[k + L + 1]; }
    const bool c0 = q + re >= 32, c1 = q + 1 + re >= 32;
    const T d10 = (t0.x + (c0 ? ra.y : ra.x)) - h0.x, d20 = (t0.y + (c0 ? rb.y : rb.x)) - h0.y;
    const T d11 = (t1.x + (c1 ? ra.y : ra.x)) - h1.x, d21 = (t1.y + (c1 ? rb.y : rb.x)) - h1.y;
    const T v0 = r0.x + (r0.y + fma(Lt, d20, -d10 * (d10 + r1.x)));
    const T v1 = r0.x + (r0.y + fma(Lt, d21, -d11 * (d11 + r1.x)));
    return cmk(O::out(v0, sqrtL, tol), O::out(v1, sqrtL, tol));
}

// Bounded wait on a TMA phase; on timeout record the error and let every
// thread return (the caller returns when this yields false).
__device__ __forceinline__ bool xcorr_wait(uint64_t *bar, uint32_t parity, int *err, uint32_t limit = (1u << 24))
{
    bool ok = mbar_wait_bounded(bar, parity, limit);
    if (!__syncthreads_and(ok))
    {
        if (threadIdx.x == 0) atomicExch(err, KERR_TMA_TIMEOUT);
        return false;
    }
    return true;
}

// ----------------------------------------------------------------------------
// Fused overlap-save correlator: one CTA per (block, template group).
// SHARED_DEN: every template has the same length, so the normalisation was
// precomputed per channel (den_kernel) and the first FFT work buffer
// overlays the staged segment.  MODE: see XcorrLayout.
template <class T, int LOG2P, bool SHARED_DEN, int MODE>
__device__ __forceinline__ int xcorr_tile(const XcorrParams<T> &p, const int bx, const int g)
{
    using Acc = acc_t<T>;
    using acc = typename Acc::type;
    using LY = XcorrLayout<T, LOG2P>;
    using PL = FftPlan<LOG2P>;
    constexpr bool PREFETCH = MODE == 1;
    constexpr bool TEAMS = MODE >= 2;
    // mode 4: 512 threads in two 256-thread teams, each normalising its own
    // templates (several lengths) into its own row; split twiddle table
    constexpr bool WIDE = MODE == 4;
    constexpr int NTH = WIDE ? 2 * kThreads : kThreads;  // threads of the CTA
    static_assert(!(WIDE && SHARED_DEN), "mode 4 normalises each template inside the CTA");
    // mode 3: two teams, one template length, normalisation computed in the
    // CTA (once, before the forward FFT) instead of read from den_kernel
    constexpr bool OWN_DEN = MODE == 3;
    static_assert(!(OWN_DEN && SHARED_DEN), "mode 3 computes its own normalisation");
    // templates of several lengths (modes 0, 1, 4): each lag's normalisation
    // computed in the last inverse pass from in-chunk prefix sums and the
    // template's run statistics (inv_den_wide)
    constexpr bool PERLAG = !SHARED_DEN && !OWN_DEN;
    constexpr int P = LY::P, N = LY::N, NCH = LY::NCH;
    const int tid = threadIdx.x;
    const int c = p.grp_chan[g];
    const long k0 = (long) bx * p.S;
    const int S = p.S;
    const int t_begin = p.grp_tb[g], t_end = p.grp_te[g];
    const int ntl = t_end - t_begin;
    if (ntl <= 0) return 0;

    if (p.dead[c])
    {
        // dead trace (|min| == |max|, src/matchedFilter.cpp:886-894): rho = 0
        for (int ti = t_begin; ti < t_end; ++ti)
        {
            const int t = p.tids[ti];
            const long nv = p.nvalid[t];
            T *dst = p.rho + (long) t * p.ldr;
            for (int k = tid; k < S; k += NTH)
                if (k0 + k < nv) dst[k0 + k] = (T) 0;
        }
        return 0;
    }

    extern __shared__ __align__(128) unsigned char smem_x[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_x);  // [0] segment+twiddles, [1],[2] spectra
    T *red = reinterpret_cast<T *>(smem_x + 64);
    acc *c1 = reinterpret_cast<acc *>(smem_x + 64 + 32 * sizeof(T));  // only without SHARED_DEN
    acc *c2 = c1 + (NCH + 1);
    T *xs = reinterpret_cast<T *>(smem_x + LY::off_xs(SHARED_DEN, MODE));
    cx<T> *W0 = reinterpret_cast<cx<T> *>(smem_x + LY::off_W0(SHARED_DEN, MODE));
    cx<T> *W1 = reinterpret_cast<cx<T> *>(smem_x + LY::off_W1(SHARED_DEN, MODE));
    cx<T> *UV = reinterpret_cast<cx<T> *>(smem_x + LY::off_UV(SHARED_DEN, MODE));
    cx<T> *tws = reinterpret_cast<cx<T> *>(smem_x + LY::off_tw(SHARED_DEN, MODE));
    cx<T> *Bs0 = reinterpret_cast<cx<T> *>(smem_x + LY::off_B(SHARED_DEN, MODE));
    cx<T> *Bs1 = reinterpret_cast<cx<T> *>(smem_x + LY::off_B(SHARED_DEN, MODE) + LY::up(LY::brow));
    T *invd_s = reinterpret_cast<T *>(smem_x + LY::off_invd(SHARED_DEN, MODE));
    unsigned *Mk = reinterpret_cast<unsigned *>(smem_x + LY::off_M(SHARED_DEN, MODE, S));
    cx<T> *W = W0;
    const cx<T> *post = p.twt + PL::post_off();  // real-FFT twiddles, read once per CTA from L2
    constexpr uint32_t kTwBytes = (uint32_t) LY::tw_bytes_of(MODE);

    // ---- stage segment, pass twiddles and the first spectrum with bulk async copies
    if (tid < 2 * (TEAMS ? 2 : 1) * LY::mask_words) Mk[tid] = 0u;  // chunk masks of the fused peak candidates
    if (tid == 0)
    {
        mbar_init(&bar[0], 1);
        if (PREFETCH) { mbar_init(&bar[1], 1); mbar_init(&bar[2], 1); }
        fence_proxy_async_smem();
        const uint32_t den_bytes = SHARED_DEN ? (uint32_t) (sizeof(T) * S) : 0u;
        mbar_arrive_expect_tx(&bar[0], (uint32_t) LY::seg + kTwBytes + den_bytes);
        if (!p.test_skip_copy)
        {
            tma_load_1d(xs, p.x + (long) c * p.ldx + k0, (uint32_t) LY::seg, &bar[0]);
            tma_load_1d(tws, WIDE ? p.twt_split : p.twt, kTwBytes, &bar[0]);
            if (SHARED_DEN) tma_load_1d(invd_s, p.den + (long) c * p.ldd + k0, den_bytes, &bar[0]);
        }
        if (PREFETCH)
        {
            mbar_arrive_expect_tx(&bar[1], (uint32_t) LY::brow);
            tma_load_1d(Bs0, p.Bc + (long) p.tids[t_begin] * p.ldb, (uint32_t) LY::brow, &bar[1]);
        }
    }
    __syncthreads();
    if (!xcorr_wait(&bar[0], 0, p.err, p.test_skip_copy ? (1u << 12) : (1u << 24)))
    {
        if (PREFETCH) mbar_wait_bounded(&bar[1], 0);  // let the spectrum copy land before exiting
        return -1;
    }

    // ---- segment mean; sliding-window normalisation (precomputed per
    //      channel by den_kernel when every template shares one length)
    MeanAcc<T> macc;
    for (int i = tid; i < N; i += NTH) macc.add(xs[i]);
    const T m = block_mean<T, NTH>(macc, red, N);
    SegStats<T> st;
    st.xs = xs; st.yp = xs; st.m = m; st.c1 = c1; st.c2 = c2;
    st.p1 = reinterpret_cast<T *>(c2 + NCH + 1);
    st.p2 = st.p1 + NCH;
    if constexpr (!SHARED_DEN) seg_chunk_prefix<T, N, NTH>(st, tid);
    if constexpr (OWN_DEN)
    {
        // the second team's buffer is free until the teams start: padded
        // demeaned copy there, then the CTA's one normalisation row
        st.yp = reinterpret_cast<T *>(W1);
        seg_make_padded<T, N>(st, tid);
        seg_inv_den<T, N>(st, p.tlen[p.tids[t_begin]], S, p.tol, invd_s, tid);
    }

    // ---- forward real FFT of (x - m), read straight from the staged segment
    //      (with SHARED_DEN the work buffer overlays the segment)
    {
        const cx<T> *xs2 = reinterpret_cast<const cx<T> *>(xs);
        auto ld = [&](int e) -> cx<T> {
            cx<T> v = xs2[e];
            return cmk(v.x - m, v.y - m);
        };
        auto stb = [&](int e, cx<T> v) { W[spad(e)] = v; };
        fft_run<T, LOG2P, NTH, false, true, decltype(ld), decltype(stb), SHARED_DEN || OWN_DEN, 0, WIDE>(W, tws, tid,
                                                                                                        ld, stb);
        __syncthreads();
        // Real-FFT post-processing to X[k], k = 0..P, then the per-bin pairs
        //   U[e] = X[e] (1 + i wc_e),  V[e] = conj(X[P-e]) (1 - i wc_e),
        // wc_e = exp(+2 pi i e/N), so that the inverse pre-processing of
        // Y = B X becomes Z'[e] = B[e] U[e] + conj(B[P-e]) V[e].
        for (int k = tid; k <= P / 2; k += NTH)
        {
            cx<T> xk, xp;  // X[k], X[P-k]
            if (k == 0)
            {
                const cx<T> z = W[0];
                xk = cmk(z.x + z.y, (T) 0);
                xp = cmk(z.x - z.y, (T) 0);
            }
            else
            {
                const cx<T> zk = W[spad(k)], zp = W[spad(P - k)];
                const cx<T> E = cscale(zk + cconj(zp), (T) 0.5);
                const cx<T> D = cscale(zk - cconj(zp), (T) 0.5);
                const cx<T> wO = cmul(post[k], cmk(D.y, -D.x));
                xk = E + wO;
                xp = cconj(E - wO);
            }
            const cx<T> wc = cconj(post[k]);                  // exp(+2 pi i k/N)
            const cx<T> iw = cmk(-wc.y, wc.x);                // i wc_k
            UV[2 * k] = cmul(xk, cmk((T) 1 + iw.x, iw.y));    // U[k]
            UV[2 * k + 1] = cmul(cconj(xp), cmk((T) 1 - iw.x, -iw.y));  // V[k]
            if (k > 0 && k < P / 2)
            {
                // wc_{P-k} = -conj(wc_k), so i wc_{P-k} = (iw.x, -iw.y)
                UV[2 * (P - k)] = cmul(xp, cmk((T) 1 + iw.x, -iw.y));
                UV[2 * (P - k) + 1] = cmul(cconj(xk), cmk((T) 1 - iw.x, iw.y));
            }
        }
        __syncthreads();
    }
    cx<T> *q12 = reinterpret_cast<cx<T> *>(xs);
    if constexpr (PERLAG)
    {
        // the segment's region is free now: in-chunk prefix sums of y and
        // y^2, from which the epilogue derives each template's normalisation
        // (inv_den_wide)
        seg_prefix_q12<T, N, NTH>(st, q12, st.p1, st.p2, tid);
    }

    // ---- per template: fused conj-multiply + inverse FFT + Pearson epilogue
    //      BAR/NTT select the barrier domain: the whole CTA, or one team.
    //
    // Fused peak candidates (p.pk_on): the last pass also sets bit c of the
    // template's chunk mask when a lag in [64c, 64c+64) exceeds the
    // threshold.  After the team's next barrier (the next template's, or a
    // final one), which makes the team's global stores visible to the team,
    // only the flagged chunks are read back (from L2) and examined: the
    // candidate rule for the lags [k0+1, k0+S-2], whose neighbours both lie
    // in this block.  The block's first and last lags are decided from the
    // stored trace after the launch.
    const bool pk = p.pk_on != 0;
    const long pk_n = p.pk_len;
    const T pk_thr = p.pk_thr;
    constexpr int MW = LY::mask_words;
    auto pk_scan = [&](auto nt_tag, const unsigned *mk, int t, int ttid) {
        constexpr int NTT = decltype(nt_tag)::value;
        const T *Rt = p.rho + (long) t * p.ldr + k0;
        const long nv = p.nvalid[t];
        const int kmax = (int) (nv - k0 < (long) S ? nv - k0 : (long) S);
#pragma unroll 1
        for (int w = 0; w < MW; ++w)
        {
            unsigned m = mk[w];
            while (m)
            {
                const int c = 32 * w + __ffs(m) - 1;
                m &= m - 1;
                for (int l = 64 * c + ttid; l < 64 * c + 64; l += NTT)
                {
                    if (l < 1 || l > S - 2 || k0 + l >= pk_n) continue;  // then also l < kmax
                    const T xi = __ldcg(Rt + l);
                    if (!(xi > pk_thr)) continue;
                    const T xr = l + 1 < kmax ? __ldcg(Rt + l + 1) : (T) 0;  // unused at the trace's last lag
                    if (cand_rule<T>(__ldcg(Rt + l - 1), xi, xr, k0 + l, pk_n, pk_thr))
                    {
                        const long slot = (long) t * p.pk_stride + bx;
                        const int pos = atomicAdd(p.pk_cnt + slot, 1);
                        if (pos < kPkCap)
                        {
                            p.pk_idx[slot * kPkCap + pos] = (int) (k0 + l);
                            p.pk_val[slot * kPkCap + pos] = xi;
                        }
                    }
                }
            }
        }
    };
    auto template_body = [&](auto bar_tag, auto nt_tag, int j, const cx<T> *B, cx<T> *Wt, unsigned *mk, int ttid,
                             int bar_id, const T *invd_row) {
        constexpr int BAR = decltype(bar_tag)::value;
        constexpr int NTT = decltype(nt_tag)::value;
        const int t = p.tids[t_begin + j];
        const long nv = p.nvalid[t];
        T *dst = p.rho + (long) t * p.ldr + k0;
        auto pre = [&](int e) -> cx<T> {
            cx<T> u, v;
            load_pair<T>(UV + 2 * e, u, v);
            const cx<T> b1 = B[e], b2 = B[P - e];
            // b1 u + conj(b2) v
            return cmk(b1.x * u.x - b1.y * u.y + b2.x * v.x + b2.y * v.y,
                       b1.x * u.y + b1.y * u.x + b2.x * v.y - b2.y * v.x);
        };
        // lags [k0, k0 + kmax) of this block are stored (kmax <= S, even S)
        const int kmax = (int) (nv - k0 < (long) S ? nv - k0 : (long) S);
        const cx<T> *invd2 = reinterpret_cast<const cx<T> *>(invd_row);
        const int L = p.tlen[t], re = L & 31;
        const T Lt = (T) L, sqrtL = sqrt(Lt);
        auto epi = [&](int e, cx<T> z) {
            const int k = 2 * e;
            if (k >= kmax) return;
            // rows from den_kernel (TMA) are plain, rows from seg_inv_den
            // swizzled; several lengths: the pair from the run statistics
            cx<T> d;
            if constexpr (PERLAG) d = inv_den_wide<T>(q12, invd2, k, L, re, Lt, sqrtL, p.tol);
            else d = invd2[SHARED_DEN ? e : inv_den_pair<T>(e)];
            const T r0 = clamp_rho(z.x * d.x);
            const T r1 = clamp_rho(z.y * d.y);
            if (k + 1 < kmax) store2<T>(dst + k, r0, r1);
            else dst[k] = r0;
            if (pk && (r0 > pk_thr || r1 > pk_thr)) atomicOr(mk + (e >> 10), 1u << ((e >> 5) & 31));
        };
        fft_run<T, LOG2P, NTT, true, false, decltype(pre), decltype(epi), false, BAR, WIDE>(Wt, tws, ttid, pre, epi,
                                                                                           bar_id);
    };

    if constexpr (WIDE)
    {
        // two teams of 256 threads; each keeps its own work buffer, chunk
        // masks, run statistics (its templates' own lengths) and barrier
        const int team = tid >> 8, ttid = tid & 255, bar_id = 1 + team;
        unsigned *mkt = Mk + team * 2 * MW;
        cx<T> *Wt = team ? W1 : W0;
        // the team's run statistics (seg_run_stats), passed as the epilogue's row
        cx<T> *rd_t = reinterpret_cast<cx<T> *>(reinterpret_cast<unsigned char *>(invd_s) + team * LY::rd_bytes(S));
        int t_prev = -1, it = 0, Lt = -1;
        for (int j = team; j < ntl; j += 2, ++it)
        {
            const int t = p.tids[t_begin + j];
            const cx<T> *B = p.Bc + (long) t * p.ldb;
            if (it > 0)
            {
                team_sync<-1, kThreads>(bar_id);
                if (pk)
                {
                    pk_scan(std::integral_constant<int, kThreads>(), mkt + ((it - 1) & 1) * MW, t_prev, ttid);
                    if (ttid < MW) mkt[(it & 1) * MW + ttid] = 0u;
                }
            }
            const int L = p.tlen[t];
            if (L != Lt)
            {
                // read in the last inverse pass, after the passes' barriers;
                // the previous template's epilogue finished at the barrier above
                seg_run_stats<T, kThreads>(st, q12, st.p1, st.p2, L, S, rd_t, ttid);
                Lt = L;
            }
            template_body(std::integral_constant<int, -1>(), std::integral_constant<int, kThreads>(), j, B, Wt,
                          mkt + (it & 1) * MW, ttid, bar_id, reinterpret_cast<const T *>(rd_t));
            t_prev = t;
        }
        if (pk && it > 0)
        {
            team_sync<-1, kThreads>(bar_id);
            pk_scan(std::integral_constant<int, kThreads>(), mkt + ((it - 1) & 1) * MW, t_prev, ttid);
        }
    }
    else if constexpr (TEAMS)
    {
        // two teams of 128 threads; each keeps its own work buffer, chunk
        // masks and barrier
        // one code path for both teams: named barrier 1 + team, chosen at
        // run time
        const int team = tid >> 7, ttid = tid & 127, bar_id = 1 + team;
        unsigned *mkt = Mk + team * 2 * MW;
        cx<T> *Wt = team ? W1 : W0;
        int t_prev = -1, it = 0;
        for (int j = team; j < ntl; j += 2, ++it)
        {
            const cx<T> *B = p.Bc + (long) p.tids[t_begin + j] * p.ldb;
            if (it > 0)
            {
                team_sync<-1, 128>(bar_id);
                if (pk)
                {
                    pk_scan(std::integral_constant<int, 128>(), mkt + ((it - 1) & 1) * MW, t_prev, ttid);
                    if (ttid < MW) mkt[(it & 1) * MW + ttid] = 0u;
                }
            }
            template_body(std::integral_constant<int, -1>(), std::integral_constant<int, 128>(), j, B, Wt,
                          mkt + (it & 1) * MW, ttid, bar_id, invd_s);
            t_prev = p.tids[t_begin + j];
        }
        if (pk && it > 0)
        {
            team_sync<-1, 128>(bar_id);
            pk_scan(std::integral_constant<int, 128>(), mkt + ((it - 1) & 1) * MW, t_prev, ttid);
        }
    }
    else
    {
        int Lrd = -1;  // length of the run statistics in invd_s
        for (int j = 0; j < ntl; ++j)
        {
            const int t = p.tids[t_begin + j];
            if (j > 0)
            {
                __syncthreads();  // previous template finished reading W and its spectrum buffer
                if (pk)
                {
                    pk_scan(std::integral_constant<int, kThreads>(), Mk + ((j - 1) & 1) * MW,
                            p.tids[t_begin + j - 1], tid);
                    if (tid < MW) Mk[(j & 1) * MW + tid] = 0u;
                }
            }
            const cx<T> *B;
            if constexpr (PREFETCH)
            {
                if (tid == 0 && j + 1 < ntl)
                {
                    fence_proxy_async_smem();
                    uint64_t *nb = &bar[1 + ((j + 1) & 1)];
                    mbar_arrive_expect_tx(nb, (uint32_t) LY::brow);
                    tma_load_1d(((j + 1) & 1) ? Bs1 : Bs0, p.Bc + (long) p.tids[t_begin + j + 1] * p.ldb,
                                (uint32_t) LY::brow, nb);
                }
                if (!xcorr_wait(&bar[1 + (j & 1)], (uint32_t) ((j >> 1) & 1), p.err))
                {
                    if (j + 1 < ntl) mbar_wait_bounded(&bar[1 + ((j + 1) & 1)], (uint32_t) (((j + 1) >> 1) & 1));
                    return -1;
                }
                B = (j & 1) ? Bs1 : Bs0;
            }
            else
            {
                B = p.Bc + (long) t * p.ldb;
            }
            if constexpr (PERLAG)
            {
                // run statistics of the template's length, read in the last
                // inverse pass after the passes' barriers; the previous
                // template's epilogue finished at the barrier above
                const int L = p.tlen[t];
                if (L != Lrd)
                {
                    seg_run_stats<T, kThreads>(st, q12, st.p1, st.p2, L, S, reinterpret_cast<cx<T> *>(invd_s), tid);
                    Lrd = L;
                }
            }
            template_body(std::integral_constant<int, 0>(), std::integral_constant<int, kThreads>(), j, B, W,
                          Mk + (j & 1) * MW, tid, 0, invd_s);
        }
        if (pk)
        {
            __syncthreads();
            pk_scan(std::integral_constant<int, kThreads>(), Mk + ((ntl - 1) & 1) * MW, p.tids[t_end - 1], tid);
        }
    }
    return 1;
}

// The correlator kernel.  Grid launch (PERSIST false): CTA (x, y) is block x
// of work group y.  Persistent launch (PERSIST true, an option): each CTA
// takes tiles from the device ticket p.ticket (tile t = block t % nblk of
// group t / nblk) until ntiles are handed out, invalidating and setting up
// its mbarriers again between tiles; a tile whose bounded wait gave up ends
// the CTA.  On GB300 the persistent form measured slower than the grid
// (10.39 against 9.68 ms for the 2,000-template bank at 1/10 of a day, 4.50
// against 4.16 ms for the 24-channel day): the hardware block scheduler
// already balances these many equal tiles, and the tile loop costs
// registers (spills in the mode-4 form).
template <class T, int LOG2P, bool SHARED_DEN, int MODE, bool PERSIST = false>
__global__ void __launch_bounds__(MODE == 4 ? 2 * kThreads : kThreads,
                                  (sizeof(T) == 4 && LOG2P <= 11 && MODE != 4) ? 2 : 1)
    xcorr_kernel(XcorrParams<T> p)
{
    if constexpr (!PERSIST)
    {
        xcorr_tile<T, LOG2P, SHARED_DEN, MODE>(p, blockIdx.x, blockIdx.y);
    }
    else
    {
        extern __shared__ __align__(128) unsigned char smem_x[];
        uint64_t *bar = reinterpret_cast<uint64_t *>(smem_x);
        int *tslot = reinterpret_cast<int *>(smem_x + 32);  // free bytes between the barriers and the scratch
        for (;;)
        {
            if (threadIdx.x == 0) *tslot = atomicAdd(p.ticket, 1);
            __syncthreads();
            const int t = *tslot;
            __syncthreads();  // every thread has the ticket before thread 0 draws the next
            if (t >= p.ntiles) return;
            const int st = xcorr_tile<T, LOG2P, SHARED_DEN, MODE>(p, t % p.nblk, t / p.nblk);
            if (st < 0) return;
            if (st > 0)
            {
                __syncthreads();  // every wait of the tile has returned, no copy in flight
                if (threadIdx.x == 0)
                    for (int i = 0; i < (MODE == 1 ? 3 : 1); ++i) mbar_inval(&bar[i]);
                __syncthreads();
            }
        }
    }
}

// ----------------------------------------------------------------------------
// Per-channel normalisation for one template length L (normalizeSignal,
// src/matchedFilter.cpp:94-166): den[c][k] = sqrt(L)/max(tol, sqrt(max(0, V_k)))
// with V_k = L s2 - s1^2, where s1, s2 are the sums of y and y^2 over
// [k, k+L) and y = x - m (m = mean of the CTA's samples; V is invariant to
// the shift).
//
// One CTA per (lag block, channel).  The CTA stages 32 * kThreads * R
// samples (R = den_runs_per_thread(L)) in shared memory with one pad word per
// 32 (conflict-free strided access) and covers den_lags_per_cta(L) =
// 32 (kThreads R - ceil(L/32)) lags, so every thread sums exactly R runs.
//   1. Sums of y and y^2 over each 32-sample run, and over its first L mod 32
//      samples, to about 48 bits for FP32 data (TwoSum / TwoProd with a
//      deferred low word) and in double for FP64 data.
//   2. Block-wide exclusive scans of the run sums.
//   3. Thread u owns the 32-lag runs v = u + kThreads i: the exact V at lag
//      32v comes from the prefixes (double-float), then 32 lags of
//      corrections in the data type,
//        V_k = V_{32v} + L D2 - D1 (D1 + 2 s1_{32v}),
//      D1 = sum of (y_in - y_out), D2 = sum of (y_in + y_out)(y_in - y_out)
//      over the lags slid so far.  The corrections involve at most 64
//      samples against the L of the window, so their rounding error stays a
//      small multiple of the unit roundoff of V (times 1 + |window mean| /
//      window deviation), unlike a plain running sum over the whole trace.
constexpr int kDenRun = 32;
__host__ __device__ constexpr int den_tail_runs(int L) { return (L + kDenRun - 1) / kDenRun; }
__host__ __device__ constexpr int den_runs_per_thread(int L) { return 1 + den_tail_runs(L) / (kThreads / 2); }
__host__ __device__ constexpr int den_lags_per_cta(int L)
{
    return kDenRun * (kThreads * den_runs_per_thread(L) - den_tail_runs(L));
}

template <class T> struct DenLayout
{
    using acc = typename acc_t<T>::type;
    static constexpr int nruns(int L) { return kThreads * den_runs_per_thread(L); }
    static constexpr size_t y_bytes(int L)
    {
        return ((sizeof(T) * (size_t) den_pad(nruns(L) * kDenRun)) + 15) & ~size_t(15);
    }
    // prefixes P1, P2 (nruns + 1 each), partial sums Q1, Q2 (nruns each),
    // warp totals (2 x 32), block-sum scratch
    static constexpr size_t bytes(int L)
    {
        return y_bytes(L) + sizeof(acc) * (4 * (size_t) nruns(L) + 2 + 64) + 32 * sizeof(T);
    }
};

// Exclusive block scan of one accumulator per thread; *total = block sum.
// wsum: 32 entries of scratch.
template <class T>
__device__ __forceinline__ typename DenOps<T>::acc den_block_scan(typename DenOps<T>::acc v,
                                                                  typename DenOps<T>::acc *wsum,
                                                                  typename DenOps<T>::acc *total)
{
    using O = DenOps<T>;
    using acc = typename O::acc;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    acc x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const acc y = O::shfl_up(x, o);
        if (lane >= o) x = O::add(x, y);
    }
    acc ex = O::shfl_up(x, 1);
    __syncthreads();  // wsum free
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0)
    {
        acc t = lane < kThreads / 32 ? wsum[lane] : O::zero();
#pragma unroll
        for (int o = 1; o < kThreads / 32; o <<= 1)
        {
            const acc y = O::shfl_up(t, o);
            if (lane >= o) t = O::add(t, y);
        }
        if (lane < kThreads / 32) wsum[lane] = t;  // inclusive warp offsets
    }
    __syncthreads();
    *total = wsum[kThreads / 32 - 1];
    if (w > 0) ex = lane > 0 ? O::add(ex, wsum[w - 1]) : wsum[w - 1];
    else if (lane == 0) ex = O::zero();
    return ex;
}

template <class T>
__global__ void __launch_bounds__(kThreads) den_kernel(const T *x, long ldx, int L, T *den, long ldd, T tol)
{
    using O = DenOps<T>;
    using acc = typename O::acc;
    extern __shared__ __align__(16) unsigned char smem_den[];
    const int tid = threadIdx.x;
    const int c = blockIdx.y;
    const int R = den_runs_per_thread(L);
    const int nruns = kThreads * R;
    const int lpc = den_lags_per_cta(L);
    const long k0 = (long) blockIdx.x * lpc;
    T *y = reinterpret_cast<T *>(smem_den);
    acc *P1 = reinterpret_cast<acc *>(smem_den + DenLayout<T>::y_bytes(L));
    acc *P2 = P1 + (nruns + 1);
    acc *Q1 = P2 + (nruns + 1);
    acc *Q2 = Q1 + nruns;
    acc *wsum = Q2 + nruns;
    T *red = reinterpret_cast<T *>(wsum + 64);

    // ---- stage 32 * nruns samples (16-byte loads; k0 and ldx are multiples
    //      of 32), eight loads in flight per thread before the first use
    const T *xr = x + (long) c * ldx + k0;
    constexpr int VW = 16 / sizeof(T), NB = 8;
    const int nvec = nruns * kDenRun / VW;
    MeanAcc<T> macc;
    for (int i0 = tid; i0 < nvec; i0 += kThreads * NB)
    {
        T v[NB][VW];
#pragma unroll
        for (int b = 0; b < NB; ++b)
        {
            const int i = i0 + b * kThreads;
            if (i >= nvec) break;
            if constexpr (sizeof(T) == 4)
            {
                const float4 a = reinterpret_cast<const float4 *>(xr)[i];
                v[b][0] = a.x; v[b][1] = a.y; v[b][2] = a.z; v[b][3] = a.w;
            }
            else
            {
                const double2 a = reinterpret_cast<const double2 *>(xr)[i];
                v[b][0] = a.x; v[b][1] = a.y;
            }
        }
#pragma unroll
        for (int b = 0; b < NB; ++b)
        {
            const int i = i0 + b * kThreads;
            if (i >= nvec) break;
#pragma unroll
            for (int q = 0; q < VW; ++q)
            {
                y[den_pad(VW * i + q)] = v[b][q];
                macc.add(v[b][q]);
            }
        }
    }
    const T m = block_mean<T>(macc, red, nruns * kDenRun);

    // ---- run sums (run j = tid + kThreads r) and partial sums of the first re samples
    const int re = L & (kDenRun - 1), Lq = L >> 5;
    acc c1 = O::zero(), c2 = O::zero();  // running carries over the rounds
    for (int r = 0; r < R; ++r)
    {
        const int j = tid + kThreads * r;
        typename O::Run a = O::run_zero(), pa = O::run_zero();
#pragma unroll
        for (int q = 0; q < kDenRun; ++q)
        {
            if (q == re) pa = a;
            O::run_add(a, y[33 * j + q] - m);
        }
        const acc a1 = O::s1(a), a2 = O::s2(a);
        Q1[j] = O::s1(pa);
        Q2[j] = O::s2(pa);
        acc t1, t2;
        const acc e1 = den_block_scan<T>(a1, wsum, &t1);
        const acc e2 = den_block_scan<T>(a2, wsum + 32, &t2);
        P1[j] = O::add(c1, e1);
        P2[j] = O::add(c2, e2);
        c1 = O::add(c1, t1);
        c2 = O::add(c2, t2);
    }
    if (tid == 0) { P1[nruns] = c1; P2[nruns] = c2; }
    __syncthreads();

    // ---- lag runs v = tid + kThreads i, 32 lags each
    const T sqrtL = sqrt((T) L);
    const T Lt = (T) L;
    const int nlr = lpc / kDenRun;
    T *drow = den + (long) c * ldd + k0;
    // Each thread's 32 results go to shared memory first (rows of 32 lags
    // over the samples' buffer, 16-byte chunks swizzled by the row index so
    // the stores are conflict-free), then the CTA's row is written to global
    // memory in coalesced 16-byte stores.  Round r's rows lie below every
    // sample that a later round reads, so one barrier per round suffices.
    constexpr int CPR = kDenRun / VW;  // 16-byte chunks per row of 32 lags
    T *ob = y;
    const int rounds = (nlr + kThreads - 1) / kThreads;
    for (int r = 0; r < rounds; ++r)
    {
        const int v = tid + kThreads * r;
        const bool act = v < nlr;
        T o[kDenRun];
        if (act)
        {
            // window [32v, 32v + L): prefixes at runs v and v + Lq, plus the
            // first re samples of run v + Lq
            const acc w1 = O::add(O::add(P1[v + Lq], Q1[v + Lq]), O::neg(P1[v]));
            const acc w2 = O::add(O::add(P2[v + Lq], Q2[v + Lq]), O::neg(P2[v]));
            T vh, vl;
            O::var0(w1, w2, L, vh, vl);
            const T c2s = (T) 2 * O::hi(w1);
            T d1 = 0, d2 = 0;
            const int base = 32 * v;
#pragma unroll
            for (int q = 0; q < kDenRun; ++q)
            {
                const T var = vh + (vl + fma(Lt, d2, -d1 * (d1 + c2s)));
                o[q] = O::out(var, sqrtL, tol);
                // the CTA mean comes off each sample first: both differences
                // are exact for samples near a large common offset
                const T yin = y[den_pad(base + q + L)] - m, yout = y[den_pad(base + q)] - m;
                const T dd = yin - yout;
                d2 = fma(yin + yout, dd, d2);
                d1 += dd;
            }
        }
        __syncthreads();  // this round's samples read
        if (act)
        {
            T *row = ob + 32 * v;
            const int sw = v & 7;
            if constexpr (sizeof(T) == 4)
            {
#pragma unroll
                for (int q = 0; q < kDenRun; q += 4)
                    *reinterpret_cast<float4 *>(row + (((q >> 2) ^ sw) << 2)) =
                        make_float4(o[q], o[q + 1], o[q + 2], o[q + 3]);
            }
            else
            {
#pragma unroll
                for (int q = 0; q < kDenRun; q += 2)
                    *reinterpret_cast<double2 *>(row + (((q >> 1) ^ sw) << 1)) = make_double2(o[q], o[q + 1]);
            }
        }
    }
    __syncthreads();
    for (int i = tid; i < nlr * CPR; i += kThreads)
    {
        const int v = i / CPR, ch = i % CPR;
        const T *src = ob + 32 * v + ((ch ^ (v & 7)) * VW);
        if constexpr (sizeof(T) == 4)
            reinterpret_cast<float4 *>(drow)[i] = *reinterpret_cast<const float4 *>(src);
        else
            reinterpret_cast<double2 *>(drow)[i] = *reinterpret_cast<const double2 *>(src);
    }
}

// ----------------------------------------------------------------------------
// Dead-trace detection (src/matchedFilter.cpp:886-894): per channel min and
// max over n samples, flag when |min| == |max|.  Two launches: partial
// min/max per (chunk, channel), then a per-channel reduction.
template <class T>
__global__ void __launch_bounds__(kThreads) minmax_partial_kernel(const T *x, long ldx, long n, int chunk,
                                                                 T *pmin, T *pmax, int nchunks)
{
    __shared__ T smin[kThreads / 32], smax[kThreads / 32];
    const int c = blockIdx.y, j = blockIdx.x;
    long beg = (long) j * chunk, end = beg + chunk < n ? beg + chunk : n;
    const T *xp = x + (long) c * ldx;
    T mn = xp[beg < n ? beg : 0], mx = mn;
    for (long i = beg + threadIdx.x; i < end; i += kThreads)
    {
        T v = xp[i];
        mn = v < mn ? v : mn;
        mx = v > mx ? v : mx;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        T a = __shfl_xor_sync(0xffffffffu, mn, o), b = __shfl_xor_sync(0xffffffffu, mx, o);
        mn = a < mn ? a : mn;
        mx = b > mx ? b : mx;
    }
    if ((threadIdx.x & 31) == 0) { smin[threadIdx.x >> 5] = mn; smax[threadIdx.x >> 5] = mx; }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        for (int i = 1; i < kThreads / 32; ++i)
        {
            mn = smin[i] < mn ? smin[i] : mn;
            mx = smax[i] > mx ? smax[i] : mx;
        }
        mn = smin[0] < mn ? smin[0] : mn;
        mx = smax[0] > mx ? smax[0] : mx;
        pmin[(long) c * nchunks + j] = mn;
        pmax[(long) c * nchunks + j] = mx;
    }
}

// one CTA per channel (blockIdx.x): partials pmin/pmax[c * nchunks + j]
template <class T>
__global__ void minmax_final_kernel(const T *pmin, const T *pmax, int nchunks, unsigned char *dead, float *range)
{
    __shared__ T smin[32], smax[32];
    pmin += (long) blockIdx.x * nchunks;
    pmax += (long) blockIdx.x * nchunks;
    dead += blockIdx.x;
    T mn = pmin[0], mx = pmax[0];
    for (int j = threadIdx.x; j < nchunks; j += blockDim.x)
    {
        mn = pmin[j] < mn ? pmin[j] : mn;
        mx = pmax[j] > mx ? pmax[j] : mx;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        T a = __shfl_xor_sync(0xffffffffu, mn, o), b = __shfl_xor_sync(0xffffffffu, mx, o);
        mn = a < mn ? a : mn;
        mx = b > mx ? b : mx;
    }
    if ((threadIdx.x & 31) == 0) { smin[threadIdx.x >> 5] = mn; smax[threadIdx.x >> 5] = mx; }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        for (int i = 1; i < (int) (blockDim.x >> 5); ++i)
        {
            mn = smin[i] < mn ? smin[i] : mn;
            mx = smax[i] > mx ? smax[i] : mx;
        }
        *dead = fabs(mn) == fabs(mx) ? 1 : 0;
        if (range) range[blockIdx.x] = (float) (mx - mn);  // max - min (tensor-core strip scale)
    }
}

}  // namespace mfgpu
