// kernels_mf.cuh -- matched-filter kernels (templated on the sample type).
//
// Design (GB300, one CTA per (signal block, channel)):
//   * Overlap-save instead of the reference's overlap-add: block b of a
//     channel reads samples [b*S, b*S + N) and yields the S lags
//     [b*S, b*S + S) of every template on that channel, S <= N - Lmax + 1.
//     No block writes another block's outputs, so nothing is accumulated in
//     HBM (the reference accumulates y[istart+i] += ... across blocks,
//     src/matchedFilter.cpp:1093-1112).
//   * The N-sample segment is staged into shared memory by one TMA bulk
//     copy (cp.async.bulk + mbarrier, bounded wait).
//   * The segment mean m is subtracted before both the FFT and the sliding
//     sums.  The numerator is invariant to it (templates are zero-mean,
//     src/matchedFilter.cpp:172-189) and so is the window variance, but the
//     FP32 rounding error of both no longer scales with the DC level.
//   * Sliding-window sums of y and y^2 over each template length
//     (normalizeSignal, src/matchedFilter.cpp:94-166) are accumulated in
//     double-float for FP32 data (about 48 significant bits; GB300's FP64
//     rate is a small fraction of its FP32 rate) and in double for FP64 data.
//   * Forward real FFT of the segment once; per template: conj(B_t)/N
//     multiply fused into the pre-processing of the inverse real FFT, the
//     inverse complex FFT, and the Pearson epilogue
//     rho = sqrt(L) num / max(tol, sqrt(max(0, L s2 - s1^2))), rho := 0 when
//     |rho| > 1.1, written with 16-byte stores.
#pragma once
#include "device_common.cuh"

namespace mfgpu {

constexpr int kThreads = 256;

template <class T> struct XcorrParams
{
    const T *x;               // channel signals, row stride ldx (zero padded tail)
    long ldx;
    const cx<T> *Bc;          // conj(spectrum)/N of each template, row stride ldb
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
    const cx<T> *tw;          // exp(-2 pi i m / NMAX) table
    int S;                    // lags per block (multiple of 32)
    T tol;
    int *err;
};

template <class T> struct SpecParams
{
    const double *tmpl;       // concatenated FP64 template samples
    const long *toff;         // offset of each template
    const int *tlen;
    cx<T> *Bc;
    long ldb;
    const cx<T> *tw;
};

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

// ----------------------------------------------------------------------------
// Template spectra: demean and unit-normalise the template in FP64
// (src/matchedFilter.cpp:168-190; the double path uses the template's own
// length, :575), zero pad to N, forward real FFT, store conj(B)/N for
// k = 0..P.  The template is not reversed: correlation uses conj(B).
template <class T, int LOG2P, int NMAX>
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
    double mean = block_sum<double>(s, red) / (double) L;
    double q = 0;
    for (int i = tid; i < L; i += kThreads) { double d = b[i] - mean; q += d * d; }
    double nrm2 = block_sum<double>(q, red);
    double inv = nrm2 > 0 ? 1.0 / sqrt(nrm2) : 0.0;
    for (int n = tid; n < P; n += kThreads)
    {
        T re = 0, im = 0;
        if (2 * n < L) re = (T) ((b[2 * n] - mean) * inv);
        if (2 * n + 1 < L) im = (T) ((b[2 * n + 1] - mean) * inv);
        A[spad(n)] = cmk(re, im);
    }
    __syncthreads();
    fft_passes<T, LOG2P, kThreads, false, NMAX>(A, p.tw, tid);
    const T scale = (T) (1.0 / (double) N);
    cx<T> *out = p.Bc + (long) t * p.ldb;
    for (int k = tid; k <= P / 2; k += kThreads)
    {
        if (k == 0)
        {
            cx<T> z = A[0];
            out[0] = cmk((z.x + z.y) * scale, (T) 0);
            out[P] = cmk((z.x - z.y) * scale, (T) 0);
            continue;
        }
        cx<T> zk = A[spad(k)], zp = A[spad(P - k)];
        cx<T> E = cscale(zk + cconj(zp), (T) 0.5);
        cx<T> D = cscale(zk - cconj(zp), (T) 0.5);
        cx<T> O = cmk(D.y, -D.x);  // D / i
        cx<T> w = p.tw[k * (NMAX / N)];
        cx<T> wO = cmul(w, O);
        cx<T> Xk = E + wO;
        cx<T> Xp = cconj(E - wO);
        out[k] = cscale(cconj(Xk), scale);
        out[P - k] = cscale(cconj(Xp), scale);
    }
}

// ----------------------------------------------------------------------------
// Sliding-window statistics of the staged segment.
template <class T> struct SegStats
{
    using A = acc_t<T>;
    using acc = typename A::type;
    const T *xs;   // raw segment, N samples
    T m;           // segment mean
    acc *c1, *c2;  // chunk prefix sums (N/32 + 1 entries each)
};

// Chunk sums over 32 samples with a per-lane skew (conflict-free banks),
// then an exclusive scan by warp 0.
template <class T, int N>
__device__ __forceinline__ void seg_chunk_prefix(SegStats<T> st, int tid)
{
    using A = acc_t<T>;
    using acc = typename A::type;
    constexpr int NCH = N / 32;
    const int lane = tid & 31;
    for (int j = tid; j < NCH; j += kThreads)
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

// inv_den[k] = sqrt(L)/max(tol, sqrt(max(0, L*s2 - s1^2))) for k in [0, S).
// Thread u slides over an odd-length run of lags (odd stride = no bank
// conflicts); the run's first window comes from the chunk prefixes plus a
// skewed partial sum.
template <class T, int N>
__device__ __forceinline__ void seg_inv_den(SegStats<T> st, int L, int S, T tol, T *invd, int tid)
{
    using A = acc_t<T>;
    using acc = typename A::type;
    const int RL = ((S + kThreads - 1) / kThreads) | 1;
    const int k = tid * RL;
    const int lane = tid & 31;
    const int kend = min(S, k + RL);
    // prefix sums at positions k and k + L
    acc a1 = A::zero(), a2 = A::zero(), b1 = A::zero(), b2 = A::zero();
    const int pk = k < S ? k : 0, pe = (k < S ? k : 0) + L;
    const int ck = pk >> 5, ce = pe >> 5, rk = pk & 31, re = pe & 31;
#pragma unroll 4
    for (int s = 0; s < 32; ++s)
    {
        int j = (s + lane) & 31;
        if (j < rk) { T v = st.xs[32 * ck + j] - st.m; a1 = A::add_val(a1, v); a2 = A::add_sq(a2, v); }
        if (j < re) { T v = st.xs[32 * ce + j] - st.m; b1 = A::add_val(b1, v); b2 = A::add_sq(b2, v); }
    }
    if (k >= S) return;
    acc w1 = A::sub(A::add(st.c1[ce], b1), A::add(st.c1[ck], a1));
    acc w2 = A::sub(A::add(st.c2[ce], b2), A::add(st.c2[ck], a2));
    for (int q = k; q < kend; ++q)
    {
        invd[q] = A::inv_den(w1, w2, L, tol);
        if (q + 1 < kend)
        {
            T vin = st.xs[q + L] - st.m, vout = st.xs[q] - st.m;
            w1 = A::add_val(A::add_val(w1, vin), -vout);
            w2 = A::sub(A::add_sq(w2, vin), A::add_sq(A::zero(), vout));
        }
    }
}

template <class T> __device__ __forceinline__ void store4(T *dst, T a, T b, T c, T d);
template <> __device__ __forceinline__ void store4<float>(float *dst, float a, float b, float c, float d)
{
    *reinterpret_cast<float4 *>(dst) = make_float4(a, b, c, d);
}
template <> __device__ __forceinline__ void store4<double>(double *dst, double a, double b, double c, double d)
{
    reinterpret_cast<double2 *>(dst)[0] = make_double2(a, b);
    reinterpret_cast<double2 *>(dst)[1] = make_double2(c, d);
}

template <class T> __device__ __forceinline__ T clamp_rho(T v) { return fabs(v) > (T) 1.1 ? (T) 0 : v; }

// ----------------------------------------------------------------------------
// Fused overlap-save correlator: one CTA per (block, channel).
// SHARED_DEN: every template of every channel has the same length, so the
// normalisation is computed once per CTA and the inverse-FFT buffer reuses
// the staged segment's shared memory (2 CTAs per SM at N = 8192 FP32).
template <class T, int LOG2P, int NMAX, bool SHARED_DEN>
__global__ void __launch_bounds__(kThreads, (SHARED_DEN && sizeof(T) == 4) ? 2 : 1) xcorr_kernel(XcorrParams<T> p)
{
    using Acc = acc_t<T>;
    using acc = typename Acc::type;
    constexpr int P = 1 << LOG2P;
    constexpr int N = 2 * P;
    constexpr int NCH = N / 32;
    const int tid = threadIdx.x;
    const int g = blockIdx.y;
    const int c = p.grp_chan[g];
    const long k0 = (long) blockIdx.x * p.S;
    const int S = p.S;
    const int t_begin = p.grp_tb[g], t_end = p.grp_te[g];
    if (t_begin == t_end) return;

    if (p.dead[c])
    {
        // dead trace (|min| == |max|, src/matchedFilter.cpp:886-894): rho = 0
        for (int ti = t_begin; ti < t_end; ++ti)
        {
            int t = p.tids[ti];
            long nv = p.nvalid[t];
            T *dst = p.rho + (long) t * p.ldr;
            for (int k = tid; k < S; k += kThreads)
                if (k0 + k < nv) dst[k0 + k] = (T) 0;
        }
        return;
    }

    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char *sp = smem_raw;
    uint64_t *bar = reinterpret_cast<uint64_t *>(sp); sp += 16;
    T *red = reinterpret_cast<T *>(sp); sp += 32 * sizeof(T);
    acc *c1 = reinterpret_cast<acc *>(sp); sp += sizeof(acc) * (NCH + 1);
    acc *c2 = reinterpret_cast<acc *>(sp); sp += sizeof(acc) * (NCH + 1);
    sp = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(sp) + 127) & ~uintptr_t(127));
    constexpr size_t seg_bytes = sizeof(T) * N;
    constexpr size_t fft_bytes = sizeof(cx<T>) * spad_size(P);
    constexpr size_t xs_region = SHARED_DEN ? (seg_bytes > fft_bytes ? seg_bytes : fft_bytes) : seg_bytes;
    T *xs = reinterpret_cast<T *>(sp); sp += (xs_region + 127) & ~size_t(127);
    cx<T> *A = reinterpret_cast<cx<T> *>(sp); sp += (fft_bytes + 127) & ~size_t(127);
    cx<T> *W;
    if (SHARED_DEN) W = reinterpret_cast<cx<T> *>(xs);
    else { W = reinterpret_cast<cx<T> *>(sp); sp += (fft_bytes + 127) & ~size_t(127); }
    T *invd = reinterpret_cast<T *>(sp);

    // ---- stage the segment with one bulk async copy
    if (tid == 0)
    {
        mbar_init(bar, 1);
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(bar, (uint32_t) seg_bytes);
        tma_load_1d(xs, p.x + (long) c * p.ldx + k0, (uint32_t) seg_bytes, bar);
    }
    __syncthreads();
    bool ok = mbar_wait_bounded(bar, 0);
    if (!__syncthreads_and(ok))
    {
        if (tid == 0) atomicExch(p.err, KERR_TMA_TIMEOUT);
        return;
    }

    // ---- segment mean
    T s = 0;
    for (int i = tid; i < N; i += kThreads) s += xs[i];
    const T m = block_sum<T>(s, red) / (T) N;

    SegStats<T> st;
    st.xs = xs; st.m = m; st.c1 = c1; st.c2 = c2;
    seg_chunk_prefix<T, N>(st, tid);
    int Lcur = p.tlen[p.tids[t_begin]];
    seg_inv_den<T, N>(st, Lcur, S, p.tol, invd, tid);

    // ---- forward real FFT of (x - m)
    const cx<T> *xs2 = reinterpret_cast<const cx<T> *>(xs);
    for (int n = tid; n < P; n += kThreads)
    {
        cx<T> v = xs2[n];
        A[spad(n)] = cmk(v.x - m, v.y - m);
    }
    __syncthreads();
    fft_passes<T, LOG2P, kThreads, false, NMAX>(A, p.tw, tid);
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
        cx<T> O = cmk(D.y, -D.x);
        cx<T> wO = cmul(p.tw[k * (NMAX / N)], O);
        A[spad(k)] = E + wO;
        A[spad(P - k)] = cconj(E - wO);
    }
    __syncthreads();

    // ---- per template: multiply, inverse FFT, normalise, store
    for (int ti = t_begin; ti < t_end; ++ti)
    {
        const int t = p.tids[ti];
        if (!SHARED_DEN)
        {
            int L = p.tlen[t];
            if (L != Lcur)
            {
                seg_inv_den<T, N>(st, L, S, p.tol, invd, tid);
                Lcur = L;
            }
        }
        const cx<T> *B = p.Bc + (long) t * p.ldb;
        for (int k = tid; k <= P / 2; k += kThreads)
        {
            cx<T> Xk = A[spad(k)];
            if (k == 0)
            {
                cx<T> XP = A[spad(P)];
                cx<T> y0 = cmul(B[0], Xk), yP = cmul(B[P], XP);
                cx<T> e = y0 + cconj(yP), d = y0 - cconj(yP);
                W[0] = cmk(e.x - d.y, e.y + d.x);
                continue;
            }
            cx<T> Xp = A[spad(P - k)];
            cx<T> yk = cmul(B[k], Xk), yp = cmul(B[P - k], Xp);
            cx<T> wk = cconj(p.tw[k * (NMAX / N)]);          // exp(+2 pi i k/N)
            cx<T> e = yk + cconj(yp), d = cmul(yk - cconj(yp), wk);
            W[spad(k)] = cmk(e.x - d.y, e.y + d.x);             // e + i d
            cx<T> e2 = yp + cconj(yk), d2 = cmul(yp - cconj(yk), cmk(-wk.x, wk.y));
            W[spad(P - k)] = cmk(e2.x - d2.y, e2.y + d2.x);
        }
        __syncthreads();
        fft_passes<T, LOG2P, kThreads, true, NMAX>(W, p.tw, tid);
        const long nv = p.nvalid[t];
        T *dst = p.rho + (long) t * p.ldr + k0;
        for (int i = tid; i < S / 4; i += kThreads)
        {
            const int k = 4 * i;
            if (k0 + k >= nv) continue;
            cx<T> w0 = W[spad(2 * i)], w1 = W[spad(2 * i + 1)];
            T r0 = clamp_rho(w0.x * invd[k]);
            T r1 = clamp_rho(w0.y * invd[k + 1]);
            T r2 = clamp_rho(w1.x * invd[k + 2]);
            T r3 = clamp_rho(w1.y * invd[k + 3]);
            if (k0 + k + 3 < nv) store4<T>(dst + k, r0, r1, r2, r3);
            else
            {
                dst[k] = r0;
                if (k0 + k + 1 < nv) dst[k + 1] = r1;
                if (k0 + k + 2 < nv) dst[k + 2] = r2;
            }
        }
        __syncthreads();
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

template <class T>
__global__ void minmax_final_kernel(const T *pmin, const T *pmax, int nchunks, unsigned char *dead)
{
    __shared__ T smin[32], smax[32];
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
    }
}

}  // namespace mfgpu
