// kernels_fix.cuh -- accuracy safeguards of the FP32 path.
//
// The FP32 engine must stay within the FP64 Pearson coefficient's tolerance
// on every lag, also where a signal's amplitude changes by several decades
// within one FFT block or one window (the precision-stress recipe: DC
// offsets of 1e3..1e5 under a piecewise-constant envelope over six
// decades).  Three parts:
//
//  1. den_robust_kernel: the window variances M2 = sum (y - mean)^2 of one
//     template length without cancellation.  The running sums of the
//     reference (normalizeSignal, src/matchedFilter.cpp:94-166) subtract the
//     sums of samples that leave the window, so a quiet window next to a
//     loud one inherits the loud samples' rounding error.  Here each
//     32-sample chunk keeps its statistics about its own mean (cm, cs, cq);
//     the window's core (the samples shared by a run of 32 lags) combines
//     whole chunks about a reference R taken from the core (every term is
//     the sum of squares of one chunk about R, so nothing cancels); only the
//     31 samples at each edge of the run slide in and out, in FP32.  A run
//     whose sliding samples carry more than 100x the variance of its
//     quietest window is marked for the fix-up below.  Per run it also
//     records the quietest window's M2, R and the spread of the window means
//     about R (RunStat), which bound the correlators' numerator errors.
//  2. fix_flag_fft_kernel / fix_flag_tc_kernel: per 32-lag run, an upper
//     bound of the correlator's numerator rounding error against the run's
//     quietest window.  FFT form: the transform's error is spread over the
//     whole block, about 2^-24 sqrt(E_b) for a unit-norm template where E_b
//     is the block's energy about its mean.  Tensor-core form: the FP16
//     hi+lo split and FP32 accumulation err relative to |x - off|, off the
//     strip's operand offset (chosen here as the level of the strip's
//     quietest run).  Runs over the bound are flagged.
//  3. fixup_kernel: every flagged run is recomputed for all templates on its
//     channel by a direct two-pass FP32 Pearson correlation about a local
//     reference, whose error is relative to each window's own variance.  The
//     fused peak candidates of the touched blocks are recounted
//     (fix_rescan_kernel) and the tensor-core candidate flags updated.  The
//     same kernel, in direct mode and in either sample type, correlates the
//     templates too long for any FFT plan over every lag.
#pragma once
#include "kernels_mf.cuh"
#include "fix_params.h"

namespace mfgpu {

// RunStat.x when every window of the run is constant
constexpr float kRunConst = 3.0e38f;
// warps per fix-up CTA
constexpr int kFixWarps = 4;
// coefficients per fix-up chunk staged in shared memory (per template)
constexpr int kFixChunk = 64;

// Marks run r of channel c for the fix-up: one bit per run (row stride
// ldrs / 32 words) makes every run enter the list once, however many bounds
// flag it; the list holds c * ldrs + r (capacity: every run of every channel).
__device__ __forceinline__ void fix_mark(unsigned *fbits, int *flist, int *fcount, int c, int r, long ldrs)
{
    const unsigned bit = 1u << (r & 31);
    const unsigned old = atomicOr(fbits + (long) c * (ldrs >> 5) + (r >> 5), bit);
    if (!(old & bit)) flist[atomicAdd(fcount, 1)] = (int) ((long) c * ldrs + r);
}

// Shared memory of den_robust_kernel: staged samples (padded as den_kernel),
// chunk statistics, reduction scratch.
struct DenRobustLayout
{
    static constexpr int nruns(int L) { return kThreads * den_runs_per_thread(L); }
    static constexpr size_t y_bytes(int L) { return DenLayout<float>::y_bytes(L); }
    static constexpr size_t bytes(int L) { return y_bytes(L) + sizeof(float) * (3 * (size_t) nruns(L) + 64); }
};

// Window variances of length L over channel c's lags [k0, k0 + lpc), one CTA
// per (lag block, channel) as den_kernel.  den (optional) receives
// sqrt(L) / max(tol, sqrt(L M2)) per lag (0 for a constant window), rstat one
// float4 per 32-lag run: (M2 of the quietest non-constant window, or
// kRunConst, or -1 when the run is unreliable; R; max |window mean - R|; 0),
// cst one float2 per 32-sample chunk: (mean, sum of squares about it), for
// the chunks of the CTA's lags (the last CTA: every staged chunk).
__global__ void __launch_bounds__(kThreads) den_robust_kernel(const float *x, long ldx, int L, float *den, long ldd,
                                                             float tol, float4 *rstat, long ldrs, float2 *cst,
                                                             long ldc)
{
    extern __shared__ __align__(16) unsigned char smem_dr[];
    const int tid = threadIdx.x, c = blockIdx.y;
    const int R = den_runs_per_thread(L);
    const int nruns = kThreads * R;
    const int lpc = den_lags_per_cta(L);
    const long k0 = (long) blockIdx.x * lpc;
    float *y = reinterpret_cast<float *>(smem_dr);
    float *cm = reinterpret_cast<float *>(smem_dr + DenRobustLayout::y_bytes(L));
    float *cs = cm + nruns, *cq = cs + nruns;
    float *red = cq + nruns;

    // ---- stage 32 * nruns samples (16-byte loads), CTA mean
    const float *xr = x + (long) c * ldx + k0;
    constexpr int NB = 8;
    const int nvec = nruns * kDenRun / 4;
    MeanAcc<float> macc;
    for (int i0 = tid; i0 < nvec; i0 += kThreads * NB)
    {
        float4 v[NB];
#pragma unroll
        for (int b = 0; b < NB; ++b)
        {
            const int i = i0 + b * kThreads;
            if (i < nvec) v[b] = reinterpret_cast<const float4 *>(xr)[i];
        }
#pragma unroll
        for (int b = 0; b < NB; ++b)
        {
            const int i = i0 + b * kThreads;
            if (i >= nvec) break;
            const float e[4] = {v[b].x, v[b].y, v[b].z, v[b].w};
#pragma unroll
            for (int q = 0; q < 4; ++q)
            {
                y[den_pad(4 * i + q)] = e[q];
                macc.add(e[q]);
            }
        }
    }
    const float m = block_mean<float>(macc, red, nruns * kDenRun);

    // ---- chunk statistics about each chunk's own mean
    for (int r = 0; r < R; ++r)
    {
        const int j = tid + kThreads * r;
        const float *yc = y + 33 * j;
        float v[32];
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < 32; ++q)
        {
            v[q] = yc[q] - m;
            s += v[q];
        }
        const float mu = s * (1.f / 32.f);
        float a = 0.f, b = 0.f;
#pragma unroll
        for (int q = 0; q < 32; ++q)
        {
            const float d = v[q] - mu;
            a += d;
            b = fmaf(d, d, b);
        }
        cm[j] = mu;
        cs[j] = a;
        cq[j] = b;
        if (j < den_lags_per_cta(L) / kDenRun || blockIdx.x == gridDim.x - 1)
            cst[(long) c * ldc + k0 / kDenRun + j] = make_float2(mu + m, fmaf(-a, a * (1.f / 32.f), b));
    }
    __syncthreads();

    const float sqrtL = sqrtf((float) L), invL = 1.f / (float) L, Lf = (float) L;
    const int nlr = lpc / kDenRun;
    const int Lq = L >> 5, re = L & 31;
    float *drow = den ? den + (long) c * ldd + k0 : nullptr;
    float4 *rs = rstat + (long) c * ldrs + k0 / kDenRun;
    auto yv = [&](int i) { return y[den_pad(i)] - m; };
    constexpr int CPR = kDenRun / 4;
    float *ob = y;
    const int rounds = (nlr + kThreads - 1) / kThreads;
    for (int r = 0; r < rounds; ++r)
    {
        const int v = tid + kThreads * r;
        const bool act = v < nlr;
        float o[kDenRun];
        if (act)
        {
            float M2min = kRunConst, Smax = 0.f, Rabs;
            bool bad = false;
            const int b0 = 32 * v;
            if (L >= 64)
            {
                // core [32v + 31, 32v + L): sample 32v + 31, chunks v+1 .. v+Lq-1,
                // the first re samples of chunk v + Lq
                const float Rr = cm[v + 1 + (Lq - 1) / 2];
                float SC = 0.f, QC = 0.f;
                for (int j = v + 1; j < v + Lq; ++j)
                {
                    const float d = cm[j] - Rr, sj = cs[j];
                    SC += fmaf(32.f, d, sj);
                    QC += fmaf(d, fmaf(32.f, d, 2.f * sj), cq[j]);
                }
                {
                    const float z = yv(b0 + 31) - Rr;
                    SC += z;
                    QC = fmaf(z, z, QC);
                }
                for (int i = 0; i < re; ++i)
                {
                    const float z = yv(32 * (v + Lq) + i) - Rr;
                    SC += z;
                    QC = fmaf(z, z, QC);
                }
                // the run's first window adds samples 32v .. 32v + 30
                float SA = 0.f, QA = 0.f;
#pragma unroll 8
                for (int i = 0; i < 31; ++i)
                {
                    const float z = yv(b0 + i) - Rr;
                    SA += z;
                    QA = fmaf(z, z, QA);
                }
                float S = SC + SA, Q = QC + QA, QB = 0.f;
#pragma unroll
                for (int q = 0; q < kDenRun; ++q)
                {
                    const float M2 = fmaf(-S, S * invL, Q);
                    if (drow) o[q] = M2 > 0.f ? DenOps<float>::out(Lf * M2, sqrtL, tol) : 0.f;
                    if (M2 > 0.f) M2min = fminf(M2min, M2);
                    bad |= M2 < 0.f;
                    Smax = fmaxf(Smax, fabsf(S));
                    if (q < kDenRun - 1)
                    {
                        const float zo = yv(b0 + q) - Rr, zi = yv(b0 + q + L) - Rr;
                        S += zi - zo;
                        Q = fmaf(zi, zi, fmaf(-zo, zo, Q));
                        QB = fmaf(zi, zi, QB);
                    }
                }
                const float slide = QA + QB;
                if (M2min < kRunConst) bad |= slide > 100.f * M2min;
                else bad |= slide > 0.f;
                Rabs = Rr + m;
                Smax *= invL;
            }
            else
            {
                // short templates: each window about its own mean
                float R0 = 0.f;
#pragma unroll
                for (int q = 0; q < kDenRun; ++q)
                {
                    float s = 0.f;
                    for (int i = 0; i < L; ++i) s += yv(b0 + q + i);
                    const float mu = s * invL;
                    float a = 0.f, b = 0.f;
                    for (int i = 0; i < L; ++i)
                    {
                        const float d = yv(b0 + q + i) - mu;
                        a += d;
                        b = fmaf(d, d, b);
                    }
                    const float M2 = fmaf(-a, a * invL, b);
                    if (drow) o[q] = M2 > 0.f ? DenOps<float>::out(Lf * M2, sqrtL, tol) : 0.f;
                    if (M2 > 0.f) M2min = fminf(M2min, M2);
                    if (q == 0) R0 = mu;
                    Smax = fmaxf(Smax, fabsf(mu - R0));
                }
                Rabs = R0 + m;
            }
            rs[v] = make_float4(bad ? -1.f : M2min, Rabs, Smax, 0.f);
        }
        if (!drow) continue;  // uniform across the CTA
        __syncthreads();      // this round's samples read
        if (act)
        {
            float *row = ob + 32 * v;
            const int sw = v & 7;
#pragma unroll
            for (int q = 0; q < kDenRun; q += 4)
                *reinterpret_cast<float4 *>(row + (((q >> 2) ^ sw) << 2)) = make_float4(o[q], o[q + 1], o[q + 2], o[q + 3]);
        }
    }
    if (!drow) return;
    __syncthreads();
    for (int i = tid; i < nlr * CPR; i += kThreads)
    {
        const int v = i / CPR, ch = i % CPR;
        reinterpret_cast<float4 *>(drow)[i] = *reinterpret_cast<const float4 *>(ob + 32 * v + ((ch ^ (v & 7)) * 4));
    }
}

// FFT form: block b of channel c covers lags [bS, bS + S) from samples
// [bS, bS + N) (S and N multiples of 32).  Its energy about the block mean,
// E_b, combines the chunk statistics (Chan et al.'s pairwise update); run r
// of the block is flagged when coef2 * E_b > M2min_r (coef2 = (K 2^-24 /
// tol_rho)^2) or the run is unreliable.  One warp per block, 8 per CTA.
__global__ void __launch_bounds__(256) fix_flag_fft_kernel(const float2 *cst, long ldc, long nchunks, int S, int N,
                                                          int nblocks, const float4 *rstat, long ldrs, int nruns,
                                                          const int *dlags, const unsigned char *dead, unsigned *fbits,
                                                          int *flist, int *fcount, float coef2)
{
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * 8 + (threadIdx.x >> 5), c = blockIdx.y;
    if (b >= nblocks || dead[c]) return;
    const long j0 = (long) b * S / kDenRun;
    const int nj = N / kDenRun;
    float n = 0.f, mean = 0.f, M2 = 0.f;
    auto merge = [&](float nb, float mb, float qb) {
        const float nn = n + nb;
        if (nn > 0.f)
        {
            const float d = mb - mean, w = nb / nn;
            mean = fmaf(d, w, mean);
            M2 += qb + d * d * n * w;
            n = nn;
        }
    };
    for (int i = lane; i < nj; i += 32)
    {
        const long j = j0 + i;
        const float2 st = j < nchunks ? cst[(long) c * ldc + j] : make_float2(0.f, 0.f);
        merge(32.f, st.x, st.y);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        const float nb = __shfl_xor_sync(0xffffffffu, n, o), mb = __shfl_xor_sync(0xffffffffu, mean, o),
                    qb = __shfl_xor_sync(0xffffffffu, M2, o);
        merge(nb, mb, qb);
    }
    const float lim = M2 * coef2;
    // runs past the lags backed by data (a request window shorter than the
    // object's signal) are never used: none is listed
    const int r1 = min(min((int) (((long) b * S + S) / kDenRun), nruns), (*dlags + kDenRun - 1) / kDenRun);
    for (int r = (int) j0 + lane; r < r1; r += 32)
    {
        const float mm = rstat[(long) c * ldrs + r].x;
        if (mm < 0.f || (mm < kRunConst && lim > mm)) fix_mark(fbits, flist, fcount, c, r, ldrs);
    }
}

// Tensor-core form: one warp per strip j of 1024 lags (32 runs) of channel
// c.  The strip's operand offset is the reference level R of its quietest
// run (the strip's first sample when no run has a positive variance); run r
// is flagged when c1 ||x - off|| + c2 / s > tau sqrt(M2min_r), with
// ||x - off||^2 <= M2min + L (|R_r - off| + spread_r)^2 and s the strip's
// power-of-two operand scale.  256 threads (8 strips).
__global__ void __launch_bounds__(256) fix_flag_tc_kernel(const float *x, long ldx, int L, const float4 *rstat,
                                                         long ldrs, int nruns, const int *dlags, int tiles,
                                                         const unsigned char *dead,
                                                         const float *xrange, float *off_out, unsigned *fbits,
                                                         int *flist, int *fcount, float c1, float c2, float tau)
{
    const int lane = threadIdx.x & 31;
    const int j = blockIdx.x * 8 + (threadIdx.x >> 5), c = blockIdx.y;
    if (j >= tiles) return;
    const int r = 32 * j + lane;
    const float4 st = r < nruns ? rstat[(long) c * ldrs + r] : make_float4(kRunConst, 0.f, 0.f, 0.f);
    float key = (st.x >= 0.f && st.x < kRunConst) ? st.x : INFINITY;
    int src = lane;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        const float k2 = __shfl_xor_sync(0xffffffffu, key, o);
        const int s2 = __shfl_xor_sync(0xffffffffu, src, o);
        if (k2 < key || (k2 == key && s2 < src)) { key = k2; src = s2; }
    }
    float off = __shfl_sync(0xffffffffu, st.y, src);
    if (!(key < INFINITY)) off = x[(long) c * ldx + (long) j * 1024];
    if (lane == 0) off_out[(long) c * tiles + j] = off;
    if (dead[c] || r >= nruns || 32L * r >= *dlags) return;
    bool f = st.x < 0.f;
    if (!f && st.x < kRunConst)
    {
        const float s = tc_pow2_scale(xrange[c], 13);
        const float d = fabsf(st.y - off) + st.z;
        const float bound = c1 * sqrtf(fmaf((float) L * d, d, st.x)) + c2 / s;
        f = bound > tau * sqrtf(st.x);
    }
    if (f) fix_mark(fbits, flist, fcount, c, r, ldrs);
}


// Coefficient table of the fix-up batches: one CTA per (batch, slot).  The
// template is demeaned and unit-normed in FP64 (as for the spectra), rounded
// to T; bsum receives the sum of the rounded coefficients.
template <class T>
__global__ void __launch_bounds__(256) fix_prep_kernel(const double *tmpl, const long *toff, const int *tlen,
                                                      const int *btid, const long *boff, const int *bL, T *bco,
                                                      T *bsum)
{
    __shared__ double red[8];
    const int B = blockIdx.x / kFixBatch, k = blockIdx.x % kFixBatch;
    const int t = btid[B * kFixBatch + k];
    const int Lb = bL[B];
    T *dst = bco + boff[B] + k;
    auto bsum_d = [&](double v) {
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        __syncthreads();
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
        __syncthreads();
        double s = 0;
        for (int i = 0; i < 8; ++i) s += red[i];
        return s;
    };
    if (t < 0)
    {
        for (int i = threadIdx.x; i < Lb; i += 256) dst[(long) i * kFixBatch] = (T) 0;
        return;
    }
    const int L = tlen[t];
    const double *b = tmpl + toff[t];
    double s = 0;
    for (int i = threadIdx.x; i < L; i += 256) s += b[i];
    const double mean = bsum_d(s) / L;
    double q = 0;
    for (int i = threadIdx.x; i < L; i += 256) q += (b[i] - mean) * (b[i] - mean);
    const double nrm2 = bsum_d(q);
    const double inv = nrm2 > 0 ? 1.0 / sqrt(nrm2) : 0.0;
    double cs = 0;
    for (int i = threadIdx.x; i < Lb; i += 256)
    {
        const T v = i < L ? (T) ((b[i] - mean) * inv) : (T) 0;
        dst[(long) i * kFixBatch] = v;
        cs += (double) v;
    }
    cs = bsum_d(cs);
    if (threadIdx.x == 0) bsum[t] = (T) cs;
}

template <class T> __device__ __forceinline__ T fix_rho(T num, T M2, int L, T tol)
{
    if (!(M2 > (T) 0)) return (T) 0;
    const T r = num * DenOps<T>::out((T) L * M2, sqrt((T) L), tol);
    return clamp_rho(r);
}

// Sets *p = v in stream order (a CUDA-graph replay reads the current value).
__global__ void fix_set_int_kernel(int *p, int v) { *p = v; }

// Shared-memory row of samples per warp (a multiple of 16 bytes) and the
// warp's share: the row plus one staged chunk of coefficients.
template <class T> __host__ __device__ constexpr int fix_yrow(int Lmax) { return (Lmax + 64 + 3) & ~3; }
template <class T> __host__ __device__ constexpr size_t fix_warp_bytes(int Lmax)
{
    return sizeof(T) * ((size_t) fix_yrow<T>(Lmax) + kFixBatch * kFixChunk);
}

// One warp per work item, grid-strided (blockDim.x / 32 warps per CTA).
// List mode: item j is listed run i = j / nbmax with the k-th batch of its
// channel (k = j % nbmax; items past the channel's batches are skipped), so
// the runs of one amplitude step (which cluster) spread over every warp.
// Direct mode: item j is run j / ndir of direct batch j % ndir.  Per item,
// the 32 lags of each template of the batch: dot products against the
// window's samples about a local reference (coefficients staged kFixChunk at
// a time in shared memory), window mean and M2 two-pass per distinct
// template length.
template <class T> __global__ void __launch_bounds__(32 * kFixWarps) fixup_kernel(FixParams<T> p)
{
    extern __shared__ __align__(16) unsigned char smem_fx_raw[];
    T *smem_fx = reinterpret_cast<T *>(smem_fx_raw);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int yrow = fix_yrow<T>(p.Lmax);
    T *ys = smem_fx + (size_t) wid * (yrow + kFixBatch * kFixChunk);
    T *csh = ys + yrow;
    const long W = (long) gridDim.x * nw;
    const bool direct = p.flist == nullptr;
    const long U = direct ? (long) p.nruns * p.ndir : (long) *p.fcount * p.nbmax;
    for (long j = (long) blockIdx.x * nw + wid; j < U; j += W)
    {
        int B, c, r;
        if (direct)
        {
            B = p.dir_b0 + (int) (j % p.ndir);
            r = (int) (j / p.ndir);
            c = p.bch[B];
        }
        else
        {
            const int e = p.flist[j / p.nbmax], k = (int) (j % p.nbmax);
            c = (int) (e / p.ldf);
            r = (int) (e % p.ldf);
            if (k >= p.chan_nb[c] || r >= p.nruns) continue;
            B = p.chan_b0[c] + k;
        }
        const int Lb = p.bL[B];
        const int mytid = lane < kFixBatch ? p.btid[B * kFixBatch + lane] : -1;
        const int L0 = __shfl_sync(0xffffffffu, mytid >= 0 ? p.tlen[mytid] : 0, 0);
        const T *xc = p.x + (long) c * p.ldx;
        const long lag0 = 32L * r;
        const bool dead = direct && p.dead[c];
        T acc[kFixBatch];
#pragma unroll
        for (int q = 0; q < kFixBatch; ++q) acc[q] = (T) 0;
        if (!dead)
        {
            const uint4 *co = reinterpret_cast<const uint4 *>(p.bco + p.boff[B]);
            uint4 *cs4 = reinterpret_cast<uint4 *>(csh);
            constexpr int V4 = kFixBatch * (int) sizeof(T) / 16;  // 16-byte pieces per coefficient index
            const T Rref = xc[lag0 + 16 + L0 / 2];
            for (int i = lane; i < Lb + 31; i += 32) ys[i] = xc[lag0 + i] - Rref;
            for (int i0 = 0; i0 < Lb; i0 += kFixChunk)
            {
                const int ni = min(kFixChunk, Lb - i0);
                __syncwarp();  // the previous chunk (and, first, the samples) fully read / written
                for (int v = lane; v < ni * V4; v += 32) cs4[v] = co[(long) i0 * V4 + v];
                __syncwarp();
#pragma unroll 4
                for (int i = 0; i < ni; ++i)
                {
                    const T yv = ys[lane + i0 + i];
                    const T *cf = csh + i * kFixBatch;
#pragma unroll
                    for (int q = 0; q < kFixBatch; ++q) acc[q] = fma(cf[q], yv, acc[q]);
                }
            }
        }
        const long lag = lag0 + lane;
        int prevL = -1;
        T mu = 0, M2 = 0;
#pragma unroll
        for (int q = 0; q < kFixBatch; ++q)
        {
            const int t = __shfl_sync(0xffffffffu, mytid, q);
            if (t < 0) continue;  // empty slots (the batch's last ones)
            const int Lt = p.tlen[t];
            if (!dead && Lt != prevL)
            {
                T s = 0;
                for (int i = 0; i < Lt; ++i) s += ys[lane + i];
                mu = s / (T) Lt;
                T a = 0, b = 0;
                for (int i = 0; i < Lt; ++i)
                {
                    const T d = ys[lane + i] - mu;
                    a += d;
                    b = fma(d, d, b);
                }
                M2 = fma(-a, a / (T) Lt, b);
                prevL = Lt;
            }
            const T rho = dead ? (T) 0 : fix_rho<T>(fma(-mu, p.bsum[t], acc[q]), M2, Lt, p.tol);
            if (lag < p.nvalid[t])
            {
                p.rho[(long) t * p.ldr + lag] = rho;
                if (p.pk_flags && lag < p.pk_len && rho > p.pk_thr)
                {
                    const long cc = lag >> 6;
                    atomicOr(p.pk_flags + (long) t * p.pk_words + (cc >> 5), 1u << (cc & 31));
                }
            }
            if (p.pk_dirty && lane == 0)
            {
                // candidates at lags lag0 - 1 .. lag0 + 32 depend on these values
                const long S = p.row_S ? p.row_S[t] : p.S0;
                const long bl = (lag0 > 0 ? lag0 - 1 : 0) / S, bh = (lag0 + 32) / S;
                for (long bb = bl; bb <= bh && bb < p.pk_stride; ++bb) p.pk_dirty[(long) t * p.pk_stride + bb] = 1;
            }
        }
        __syncwarp();  // ys reused by the next item
    }
}

// Recounts the fused candidates of every (template, block) slot marked by the
// fix-up: body lags [bS + 1, bS + S - 2] of the trace under the correlator's
// rule.  One warp per 32 slots.
template <class T>
__global__ void __launch_bounds__(256) fix_rescan_kernel(const T *rho, long ldr, int nt, int pk_stride,
                                                        const unsigned char *dirty, const int *row_S,
                                                        const int *row_nblk, int S0, int nblk0, const int *nvalid,
                                                        int pk_len, T thr, int *cnt, int *idx, T *val)
{
    const int lane = threadIdx.x & 31;
    const long s0 = ((long) blockIdx.x * 8 + (threadIdx.x >> 5)) * 32;
    const long ns = (long) nt * pk_stride;
    if (s0 >= ns) return;
    const bool d = s0 + lane < ns && dirty[s0 + lane] != 0;
    unsigned m = __ballot_sync(0xffffffffu, d);
    while (m)
    {
        const long s = s0 + __ffs(m) - 1;
        m &= m - 1;
        const int t = (int) (s / pk_stride), b = (int) (s % pk_stride);
        const long S = row_S ? row_S[t] : S0;
        const int nb = row_nblk ? row_nblk[t] : nblk0;
        if (b >= nb) continue;
        const T *R = rho + (long) t * ldr;
        const long k0 = (long) b * S, nv = nvalid[t];
        int total = 0;
        for (long l0 = 1; l0 <= S - 2; l0 += 32)
        {
            const long l = l0 + lane;
            bool cnd = false;
            T xi = 0;
            if (l <= S - 2 && k0 + l < pk_len)
            {
                xi = R[k0 + l];
                if (xi > thr)
                {
                    const T xr = k0 + l + 1 < nv ? R[k0 + l + 1] : (T) 0;
                    cnd = cand_rule<T>(R[k0 + l - 1], xi, xr, k0 + l, pk_len, thr);
                }
            }
            const unsigned bm = __ballot_sync(0xffffffffu, cnd);
            if (cnd)
            {
                const int pos = total + __popc(bm & ((1u << lane) - 1));
                if (pos < kPkCap)
                {
                    idx[s * kPkCap + pos] = (int) (k0 + l);
                    val[s * kPkCap + pos] = xi;
                }
            }
            total += __popc(bm);
        }
        if (lane == 0) cnt[s] = total;
    }
}

}  // namespace mfgpu
