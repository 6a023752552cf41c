// kernels_peaks.cuh -- peak finder (PeakFinder<T>::apply, src/peakFinder.cpp:329-446)
// over many traces at once.
//
// Candidates follow the reference's sign-of-difference rules
// (:345-381): i = 0 if sign(x[1]-x[0]) < 0; 0 < i < n-1 if
// sign(x[i]-x[i-1]) >= 0 and sign(x[i+1]-x[i]) < 0 (right end of a
// plateau); i = n-1 if sign(x[n-1]-x[n-2]) > 0; always x[i] > threshold.
//
// Minimum-separation pruning (:396-433) is a greedy pass in value order.
// Here it runs as rounds over all traces in parallel: an undecided
// candidate is accepted when no undecided candidate within min_distance
// has a higher priority (value descending, then index ascending), and the
// undecided candidates within min_distance of an accepted one are
// rejected.  By induction on priority this accepts exactly the candidates
// the sequential greedy pass accepts under the same total order.
//
// The packed candidate arrays have a host-chosen capacity `cap`; kernels
// read the true count from device memory and never index past `cap`.  A
// count above `cap` raises the overflow flag and the host reruns with a
// larger capacity, so the common path needs a single synchronisation.
#pragma once
#include <cstdint>
#include "kernels_util.cuh"

namespace mfgpu {

constexpr int kPkThreads = 256;
constexpr int kPkPer = 16;                          // lags per thread
constexpr int kPkChunk = kPkThreads * kPkPer;       // lags per CTA

template <class T> struct PeakTraces
{
    const T *x;       // trace i starts at x + row[i] * ldx
    long ldx;
    const int *row;   // row of each trace
    int len;          // lags per trace
    T thr;
    // optional: bit c of row r (word r * fwords + c / 32) set when a lag in
    // [64c, 64c + 64) of that row exceeds thr; a warp whose 512 lags have no
    // bit set finds no candidate and skips its reads
    const unsigned *flags = nullptr;
    int fwords = 0;
};

template <class T> __device__ __forceinline__ bool is_candidate(const T *x, int i, int n, T thr)
{
    if (i >= n) return false;
    T xi = x[i];
    if (!(xi > thr)) return false;
    if (n == 1) return xi > (T) 0;  // reference reads x[1] out of bounds; 0 assumed
    if (i == 0) return sgn<T>(x[1] - x[0]) < 0;
    if (i == n - 1) return sgn<T>(x[n - 1] - x[n - 2]) > 0;
    return sgn<T>(xi - x[i - 1]) >= 0 && sgn<T>(x[i + 1] - xi) < 0;
}

template <class T> struct vec16;
template <> struct vec16<float>
{
    static __device__ __forceinline__ void load(const float *p, float *v)
    {
#pragma unroll
        for (int i = 0; i < 4; ++i)
        {
            float4 a = reinterpret_cast<const float4 *>(p)[i];
            v[4 * i] = a.x; v[4 * i + 1] = a.y; v[4 * i + 2] = a.z; v[4 * i + 3] = a.w;
        }
    }
};
template <> struct vec16<double>
{
    static __device__ __forceinline__ void load(const double *p, double *v)
    {
#pragma unroll
        for (int i = 0; i < 8; ++i)
        {
            double2 a = reinterpret_cast<const double2 *>(p)[i];
            v[2 * i] = a.x; v[2 * i + 1] = a.y;
        }
    }
};

// Candidate mask of the 16 lags [i0, i0+16) of a trace of n lags (bit q set
// when lag i0+q is a candidate).  The 16 samples are read with 16-byte
// loads: the trace storage must be readable up to round_up(n, 16) and
// 16-byte aligned at every multiple of 16.
// Called by all 32 lanes of a warp with consecutive i0 (step 16): the
// neighbours x[i0-1] and x[i0+16] come from the adjacent lanes' vectors; only
// the first and last lane of the warp read them from memory.
template <class T> __device__ __forceinline__ unsigned cand_mask16(const T *x, int i0, int n, T thr)
{
    T v[16];
    const bool any = i0 < n;
    if (any) vec16<T>::load(x + i0, v);
    else
    {
#pragma unroll
        for (int q = 0; q < 16; ++q) v[q] = (T) 0;
    }
    const int lane = threadIdx.x & 31;
    T left = __shfl_up_sync(0xffffffffu, v[15], 1);
    T right = __shfl_down_sync(0xffffffffu, v[0], 1);
    if (lane == 0) left = (any && i0 > 0) ? x[i0 - 1] : (T) 0;
    if (lane == 31) right = (i0 + 16 < n) ? x[i0 + 16] : (T) 0;
    if (!any) return 0u;
    unsigned mask = 0;
#pragma unroll
    for (int q = 0; q < 16; ++q)
    {
        const int i = i0 + q;
        if (i >= n) break;
        const T xi = v[q];
        if (!(xi > thr)) continue;
        const T xl = q > 0 ? v[q - 1] : left;
        const T xr = q < 15 ? v[q + 1] : right;
        bool cand;
        if (n == 1) cand = xi > (T) 0;  // reference reads x[1] out of bounds; 0 assumed
        else if (i == 0) cand = sgn<T>(xr - xi) < 0;
        else if (i == n - 1) cand = sgn<T>(xi - xl) > 0;
        else cand = sgn<T>(xi - xl) >= 0 && sgn<T>(xr - xi) < 0;
        if (cand) mask |= 1u << q;
    }
    return mask;
}

// Phase 1: find candidates of one chunk; write up to kPkCap of them into the
// chunk's slot, and the exact count.
template <class T>
static __global__ void __launch_bounds__(kPkThreads) peak_cand_kernel(PeakTraces<T> tr, int nchunks, int *counts,
                                                                      int *slot_idx, T *slot_val)
{
    __shared__ long long sh[32];
    const int trace = blockIdx.y, chunk = blockIdx.x;
    const T *x = tr.x + (long) tr.row[trace] * tr.ldx;
    const int n = tr.len;
    const int i0 = chunk * kPkChunk + threadIdx.x * kPkPer;
    bool scan = true;
    if (tr.flags)
    {
        // the warp's 512 lags are chunks c64 .. c64 + 7 (c64 a multiple of 8)
        const int c64 = (chunk * kPkChunk + (threadIdx.x >> 5) * 32 * kPkPer) / 64;
        scan = c64 / 32 < tr.fwords &&
               ((tr.flags[(long) tr.row[trace] * tr.fwords + c64 / 32] >> (c64 % 32)) & 0xFFu) != 0u;
    }
    unsigned mask = scan ? cand_mask16<T>(x, i0, n, tr.thr) : 0u;  // warp-uniform choice
    long long tot;
    long long r = block_excl_scan((long long) __popc(mask), sh, &tot);
    const long slot = (long) trace * nchunks + chunk;
    while (mask)
    {
        int q = __ffs(mask) - 1;
        mask &= mask - 1;
        if (r < kPkCap)
        {
            slot_idx[slot * kPkCap + r] = i0 + q;
            slot_val[slot * kPkCap + r] = x[i0 + q];
        }
        ++r;
    }
    if (threadIdx.x == 0) counts[slot] = (int) tot;
}

// Phase 3: gather the slots (or re-scan overflowed chunks) into the packed,
// index-ordered candidate arrays (entries at or beyond cap are dropped and
// flagged).
template <class T>
static __global__ void __launch_bounds__(kPkThreads) peak_gather_kernel(PeakTraces<T> tr, int nchunks, const int *counts,
                                                                        const long long *offs, const int *slot_idx,
                                                                        const T *slot_val, int *cidx, T *cval, int *ctr,
                                                                        long long cap, int *overflow)
{
    __shared__ long long sh[32];
    const int trace = blockIdx.y, chunk = blockIdx.x;
    const long slot = (long) trace * nchunks + chunk;
    const int cnt = counts[slot];
    const long long off = offs[slot];
    if (cnt == 0) return;
    if (threadIdx.x == 0 && off + cnt > cap) *overflow = 1;
    if (cnt <= kPkCap)
    {
        for (int r = threadIdx.x; r < cnt; r += kPkThreads)
        {
            if (off + r >= cap) break;
            cidx[off + r] = slot_idx[slot * kPkCap + r];
            cval[off + r] = slot_val[slot * kPkCap + r];
            ctr[off + r] = trace;
        }
        return;
    }
    const T *x = tr.x + (long) tr.row[trace] * tr.ldx;
    const int n = tr.len;
    const int i0 = chunk * kPkChunk + threadIdx.x * kPkPer;
    bool scan = true;
    if (tr.flags)
    {
        // the warp's 512 lags are chunks c64 .. c64 + 7 (c64 a multiple of 8)
        const int c64 = (chunk * kPkChunk + (threadIdx.x >> 5) * 32 * kPkPer) / 64;
        scan = c64 / 32 < tr.fwords &&
               ((tr.flags[(long) tr.row[trace] * tr.fwords + c64 / 32] >> (c64 % 32)) & 0xFFu) != 0u;
    }
    unsigned mask = scan ? cand_mask16<T>(x, i0, n, tr.thr) : 0u;  // warp-uniform choice
    long long tot;
    long long r = block_excl_scan((long long) __popc(mask), sh, &tot);
    while (mask)
    {
        int q = __ffs(mask) - 1;
        mask &= mask - 1;
        if (off + r < cap)
        {
            cidx[off + r] = i0 + q;
            cval[off + r] = x[i0 + q];
            ctr[off + r] = trace;
        }
        ++r;
    }
}

// candidate states
enum : unsigned char { PK_UNDECIDED = 0, PK_ACCEPTED = 1, PK_NEW = 2, PK_REJECTED = 3 };

template <class T> __device__ __forceinline__ bool higher(T vj, int ij, T vg, int ig)
{
    return vj > vg || (vj == vg && ij < ig);
}

__device__ __forceinline__ long long pk_count(const long long *ncand, long long cap)
{
    long long n = *ncand;
    return n < cap ? n : cap;
}

// Round step 1: accept undecided candidates that have no undecided
// higher-priority neighbour within dist.  PK_NEW counts as undecided for
// the neighbours' tests, so the outcome does not depend on timing.
template <class T>
static __global__ void __launch_bounds__(kPkThreads) peak_decide_kernel(const long long *ncand_p, long long cap,
                                                                        const int *cidx, const T *cval, const int *ctr,
                                                                        const long long *trace_beg,
                                                                        unsigned char *state, int dist,
                                                                        int *n_undecided)
{
    const long long ncand = pk_count(ncand_p, cap);
    long long g = (long long) blockIdx.x * kPkThreads + threadIdx.x;
    if (g >= ncand) return;
    if (state[g] != PK_UNDECIDED) return;
    const int t = ctr[g];
    const long long tb = trace_beg[t], te = trace_beg[t + 1];
    const int ig = cidx[g];
    const T vg = cval[g];
    bool best = true;
    for (long long j = g - 1; j >= tb && ig - cidx[j] <= dist; --j)
    {
        unsigned char s = state[j];
        if ((s == PK_UNDECIDED || s == PK_NEW) && higher<T>(cval[j], cidx[j], vg, ig)) { best = false; break; }
    }
    if (best)
        for (long long j = g + 1; j < te && cidx[j] - ig <= dist; ++j)
        {
            unsigned char s = state[j];
            if ((s == PK_UNDECIDED || s == PK_NEW) && higher<T>(cval[j], cidx[j], vg, ig)) { best = false; break; }
        }
    if (best) state[g] = PK_NEW;
    else atomicAdd(n_undecided, 1);
}

// Round step 2: newly accepted candidates reject their undecided neighbours.
static __global__ void __launch_bounds__(kPkThreads) peak_suppress_kernel(const long long *ncand_p, long long cap,
                                                                          const int *cidx, const int *ctr,
                                                                          const long long *trace_beg,
                                                                          unsigned char *state, int dist)
{
    const long long ncand = pk_count(ncand_p, cap);
    long long g = (long long) blockIdx.x * kPkThreads + threadIdx.x;
    if (g >= ncand) return;
    if (state[g] != PK_NEW) return;
    const int t = ctr[g];
    const long long tb = trace_beg[t], te = trace_beg[t + 1];
    const int ig = cidx[g];
    for (long long j = g - 1; j >= tb && ig - cidx[j] <= dist; --j)
        if (state[j] == PK_UNDECIDED) state[j] = PK_REJECTED;
    for (long long j = g + 1; j < te && cidx[j] - ig <= dist; ++j)
        if (state[j] == PK_UNDECIDED) state[j] = PK_REJECTED;
    state[g] = PK_ACCEPTED;
}

// accepted flag (as int) for the final compaction; zero past the count
static __global__ void peak_flags_kernel(const long long *ncand_p, long long cap, const unsigned char *state, int all,
                                         int *flags)
{
    const long long ncand = pk_count(ncand_p, cap);
    long long g = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= cap) return;
    flags[g] = (g < ncand && (all || state[g] == PK_ACCEPTED)) ? 1 : 0;
}

static __global__ void peak_compact_kernel(const long long *ncand_p, long long cap, const int *flags,
                                           const long long *pos, const int *cidx, int *peaks)
{
    const long long ncand = pk_count(ncand_p, cap);
    long long g = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ncand) return;
    if (flags[g]) peaks[pos[g]] = cidx[g];
}

// per-trace peak offsets: peak_off[t] = pos[trace_beg[t]]
static __global__ void peak_trace_offsets_kernel(int ntr, const long long *trace_beg, const long long *pos,
                                                 long long *peak_off)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t > ntr) return;
    peak_off[t] = pos[trace_beg[t]];
}

// trace_beg[t] = min(offs[t * nchunks], cap): candidate offsets of each trace
static __global__ void peak_trace_beg_kernel(int ntr, int nchunks, const long long *offs, long long cap,
                                             long long *trace_beg)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t > ntr) return;
    long long v = offs[(long) t * nchunks];
    trace_beg[t] = v < cap ? v : cap;
}

// ----------------------------------------------------------------------------
// Candidates gathered by the correlator.  Chunk b of a trace is correlator
// block b, lags [b*S, b*S + S): the correlator decided the body lags
// [b*S+1, b*S+S-2] from the values it stored (count body_cnt, up to kPkCap
// unordered slot entries, indexed by row * nblk + b); the seam kernel
// decides the first and last lag of each block from the stored trace and
// forms the chunk's total count.
template <class T>
static __global__ void peak_seam_kernel(PeakTraces<T> tr, int ntr, FusedSlots<T> fs, int *counts, unsigned char *ht)
{
    const long g = (long) blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (long) ntr * fs.nblk) return;
    const int trace = (int) (g / fs.nblk), b = (int) (g % fs.nblk);
    const int row = tr.row[trace];
    if (fs.row_nblk && b >= fs.row_nblk[row])
    {
        counts[g] = 0;  // past the last block of this template's plan
        ht[g] = 0;
        return;
    }
    const long S = fs.row_S ? fs.row_S[row] : fs.S;
    const T *x = tr.x + (long) row * tr.ldx;
    const long n = tr.len;
    const long i0 = (long) b * S, i1 = i0 + S - 1;
    const int h = (i0 < n && is_candidate<T>(x, (int) i0, (int) n, tr.thr)) ? 1 : 0;
    const int tl = (i1 < n && is_candidate<T>(x, (int) i1, (int) n, tr.thr)) ? 1 : 0;
    counts[g] = h + fs.cnt[(long) row * fs.nblk + b] + tl;
    ht[g] = (unsigned char) (h | (tl << 1));
}

// Packs chunk b of a trace in index order: first lag, body (slot entries
// ranked by index, or a re-scan of the stored trace when more than kPkCap
// body lags passed), last lag.  One warp per 32 consecutive chunks of a
// trace: the lanes read the 32 counts, and the warp packs the non-empty
// chunks one after another (most chunks are empty).
static_assert(kPkCap == 32, "peak_gather_fused_kernel ranks one slot entry per lane");
constexpr int kPkGatherSpan = 32;  // chunks per warp

template <class T>
static __global__ void __launch_bounds__(kPkThreads)
    peak_gather_fused_kernel(PeakTraces<T> tr, FusedSlots<T> fs, const int *counts, const unsigned char *ht,
                             const long long *offs, int *cidx, T *cval, int *ctr, long long cap, int *overflow)
{
    const int lane = threadIdx.x & 31;
    const int trace = blockIdx.y;
    const int b0 = (blockIdx.x * (kPkThreads / 32) + (threadIdx.x >> 5)) * kPkGatherSpan;
    if (b0 >= fs.nblk) return;
    const int row = tr.row[trace];
    const T *x = tr.x + (long) row * tr.ldx;
    const long n = tr.len;
    auto put = [&](long long o, long i, T v) {
        if (o < cap)
        {
            cidx[o] = (int) i;
            cval[o] = v;
            ctr[o] = trace;
        }
    };
    const int bl = b0 + lane;
    const int cnt_l = bl < fs.nblk ? counts[(long) trace * fs.nblk + bl] : 0;
    unsigned todo = __ballot_sync(0xffffffffu, cnt_l != 0);
    while (todo)
    {
        const int q = __ffs(todo) - 1;  // warp-uniform
        todo &= todo - 1;
        const int b = b0 + q;
        const int cnt = __shfl_sync(0xffffffffu, cnt_l, q);
        const long slot = (long) trace * fs.nblk + b;
        const long long off = offs[slot];
        if (lane == 0 && off + cnt > cap) *overflow = 1;
        const int hv = ht[slot];
        const long S = fs.row_S ? fs.row_S[row] : fs.S;
        const long i0 = (long) b * S;
        if (lane == 0)
        {
            if (hv & 1) put(off, i0, x[i0]);
            if (hv & 2) put(off + cnt - 1, i0 + S - 1, x[i0 + S - 1]);
        }
        const long long boff = off + (hv & 1);
        const long bs = (long) row * fs.nblk + b;
        const int bc = fs.cnt[bs];
        if (bc <= kPkCap)
        {
            // kPkCap == 32: one entry per lane, ranked by index
            const int *si = fs.idx + bs * kPkCap;
            if (lane < bc)
            {
                const int ir = si[lane];
                int rank = 0;
                for (int r = 0; r < bc; ++r) rank += si[r] < ir ? 1 : 0;
                put(boff + rank, ir, fs.val[bs * kPkCap + lane]);
            }
            continue;
        }
        const long lo = i0 + 1, hi = (i0 + S - 1 < n) ? i0 + S - 1 : n;
        long long base = boff;
        for (long c0 = lo; c0 < hi; c0 += 32 * kPkPer)
        {
            const long a = c0 + (long) lane * kPkPer;
            unsigned mask = 0;
#pragma unroll 4
            for (int r = 0; r < kPkPer; ++r)
                if (a + r < hi && cand_rule<T>(x[a + r - 1], x[a + r], a + r + 1 < n ? x[a + r + 1] : (T) 0, a + r, n,
                                               tr.thr))
                    mask |= 1u << r;
            const int c = __popc(mask);
            int incl = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
            {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            long long r = base + incl - c;
            while (mask)
            {
                const int qq = __ffs(mask) - 1;
                mask &= mask - 1;
                put(r, a + qq, x[a + qq]);
                ++r;
            }
            base += __shfl_sync(0xffffffffu, incl, 31);
        }
    }
}

}  // namespace mfgpu
