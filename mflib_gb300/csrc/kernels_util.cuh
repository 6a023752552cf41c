// kernels_util.cuh -- device-wide exclusive scan of int32 counts into int64
// offsets (three launches: tile sums, scan of tile sums, tile re-scan).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mfgpu {

constexpr int kScanThreads = 256;
constexpr int kScanPer = 8;
constexpr int kScanTile = kScanThreads * kScanPer;

// Peak candidates: slot capacity per chunk of a trace (the correlator's
// fused scan and the stand-alone scan both write chunk slots of this size).
constexpr int kPkCap = 32;

// Candidate slots written by the correlator for chunks of S lags (one chunk
// per correlator block): count, entries and blocks per trace.
template <class T> struct FusedSlots
{
    const int *cnt;
    const int *idx;
    const T *val;
    int nblk;                   // slot row stride (the largest block count)
    int S;
    // per row (template) when the plans differ (length buckets), else null
    const int *row_S = nullptr;
    const int *row_nblk = nullptr;
};

template <class T> __device__ __forceinline__ int sgn(T d) { return d > (T) 0 ? 1 : (d < (T) 0 ? -1 : 0); }

// PeakFinder<T>::apply's candidate rule (src/peakFinder.cpp:345-381) for an
// interior or last lag i (1 <= i <= n-1) with neighbours xl = x[i-1] and
// xr = x[i+1] (xr unused when i == n-1).
template <class T> __device__ __forceinline__ bool cand_rule(T xl, T xi, T xr, long i, long n, T thr)
{
    if (!(xi > thr)) return false;
    if (i == n - 1) return sgn<T>(xi - xl) > 0;
    return sgn<T>(xi - xl) >= 0 && sgn<T>(xr - xi) < 0;
}

// exclusive block scan of one int64 per thread; returns the block total
__device__ __forceinline__ long long block_excl_scan(long long v, long long *sh, long long *total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    __syncthreads();
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0)
    {
        long long s = lane < (int) (blockDim.x >> 5) ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            long long y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < (int) (blockDim.x >> 5)) sh[lane] = s;
    }
    __syncthreads();
    long long base = w > 0 ? sh[w - 1] : 0;
    *total = sh[(blockDim.x >> 5) - 1];
    return base + x - v;
}

static __global__ void __launch_bounds__(kScanThreads) scan_tile_sums_kernel(const int *in, long n, long long *tile_sums)
{
    __shared__ long long sh[32];
    long base = (long) blockIdx.x * kScanTile;
    long long s = 0;
#pragma unroll
    for (int i = 0; i < kScanPer; ++i)
    {
        long j = base + (long) i * kScanThreads + threadIdx.x;
        if (j < n) s += in[j];
    }
    long long tot;
    block_excl_scan(s, sh, &tot);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

// single CTA: exclusive scan of the tile sums in place; tile_sums[ntiles] = grand total
static __global__ void __launch_bounds__(kScanThreads) scan_tile_offsets_kernel(long long *tile_sums, long ntiles)
{
    __shared__ long long sh[32];
    long long carry = 0;
    for (long b = 0; b < ntiles; b += kScanThreads)
    {
        long j = b + threadIdx.x;
        long long v = j < ntiles ? tile_sums[j] : 0;
        long long tot;
        long long e = block_excl_scan(v, sh, &tot);
        if (j < ntiles) tile_sums[j] = carry + e;
        carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) tile_sums[ntiles] = carry;
}

static __global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(const int *in, long n, const long long *tile_off,
                                                                  long long *out)
{
    __shared__ long long sh[32];
    long base = (long) blockIdx.x * kScanTile + (long) threadIdx.x * kScanPer;
    int v[kScanPer];
    long long s = 0;
#pragma unroll
    for (int i = 0; i < kScanPer; ++i)
    {
        long j = base + i;
        v[i] = j < n ? in[j] : 0;
        s += v[i];
    }
    long long tot;
    long long e = block_excl_scan(s, sh, &tot) + tile_off[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanPer; ++i)
    {
        long j = base + i;
        if (j < n) out[j] = e;
        e += v[i];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[n] = tile_off[gridDim.x];
}

}  // namespace mfgpu
