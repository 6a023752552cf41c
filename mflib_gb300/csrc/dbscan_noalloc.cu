// dbscan_noalloc.cu -- segmented DBSCAN that performs no device allocation.
//
// Some callers cannot call cudaMalloc: a host framework that has reserved
// every byte of device memory up front for its own pools (a serving process
// that admits work against a fixed HBM budget, for example), or a real-time
// pipeline that must not allocate or free after start-up because
// cudaMalloc/cudaFree can synchronise the whole device.  For them this entry
// point runs the same DBSCAN kernels as mfgpu_dbscan_segmented, but all of its
// working memory is one file-scope __device__ array of fixed size; the
// caller supplies the inputs and outputs in device memory and a stream.
//
// The array is shared by every call in the process and on each device it
// lives until the process exits.  Calls that overlap on the GPU (on
// different streams, or from different host threads) race on it; callers
// must serialise them.  Every kernel writes each scratch word it later reads,
// so no clearing between calls is needed.
#include <cstdint>
#include <string>
#include "mfgpu.h"
#include "launch.h"
#include "kernels_dbscan.cuh"

namespace {

using namespace mfgpu;

constexpr int kMaxPoints = MFGPU_DBSCAN_NOALLOC_MAX_OBS;
constexpr int kMaxSegments = MFGPU_DBSCAN_NOALLOC_MAX_SEGMENTS;
constexpr long kTiles = (kMaxPoints + 1 + kScanTile - 1) / kScanTile + 2;

// scratch layout (bytes, each part 256-byte aligned)
constexpr size_t align256(size_t v) { return (v + 255) & ~size_t(255); }
constexpr size_t kOffSegOf = 0;
constexpr size_t kOffParent = kOffSegOf + align256(sizeof(int) * kMaxPoints);
constexpr size_t kOffIsRoot = kOffParent + align256(sizeof(int) * kMaxPoints);
constexpr size_t kOffCore = kOffIsRoot + align256(sizeof(int) * kMaxPoints);
constexpr size_t kOffPos = kOffCore + align256(kMaxPoints);
constexpr size_t kOffTiles = kOffPos + align256(sizeof(long long) * (kMaxPoints + 1));
constexpr size_t kOffSegOff = kOffTiles + align256(sizeof(long long) * kTiles);
// one feature: sorted values, permutation, positions, finite segment ends
constexpr size_t kOffXs = kOffSegOff + align256(sizeof(int) * (kMaxSegments + 1));
constexpr size_t kOffPerm = kOffXs + align256(sizeof(double) * kMaxPoints);
constexpr size_t kOffRank = kOffPerm + align256(sizeof(int) * kMaxPoints);
constexpr size_t kOffFend = kOffRank + align256(sizeof(int) * kMaxPoints);
constexpr size_t kScratchBytes = kOffFend + align256(sizeof(int) * kMaxSegments);
static_assert((kMaxPoints & (kMaxPoints - 1)) == 0, "the bitonic sort pads to a power of two within the scratch");

__device__ __align__(256) unsigned char g_dbscan_scratch[kScratchBytes];

// Device address of the scratch array in the current context.  The host-side
// symbol is not a device address; the address belongs to the context that
// loaded the module, so it is looked up on every call (a lookup, no
// allocation) rather than cached: a cached pointer would go stale after
// cudaDeviceReset or under another context on the same device.  The first
// lookup in a context loads the module, which places the array.
cudaError_t scratch_address(void **out)
{
    *out = nullptr;
    return cudaGetSymbolAddress(out, g_dbscan_scratch);
}

// Copy of the caller's offsets forced into a valid partition of [0, n):
// first 0, last n, non-decreasing and clamped to [0, n], so no later kernel
// can index outside the caller's arrays whatever the offsets hold.  The
// offsets live in device memory and the call does not wait for the GPU, so
// malformed offsets are clamped rather than rejected (the allocating entry
// point, which reads them on the host, rejects them).
__global__ void sanitize_offsets_kernel(int n, int nseg, const int *seg_off, int *safe)
{
    int prev = 0;
    safe[0] = 0;
    for (int s = 1; s < nseg; ++s)
    {
        int v = seg_off[s];
        v = v < prev ? prev : (v > n ? n : v);
        safe[s] = v;
        prev = v;
    }
    safe[nseg] = n;
}

// segment of each point by binary search over the offsets
__global__ void seg_of_kernel(int n, int nseg, const int *seg_off, int *seg_of)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int lo = 0, hi = nseg - 1;
    while (lo < hi)
    {
        int mid = (lo + hi + 1) >> 1;
        if (seg_off[mid] <= i) lo = mid;
        else hi = mid - 1;
    }
    seg_of[i] = lo;
}

mfgpu_status fail(mfgpu_status s, const std::string &m)
{
    mfgpu::set_last_error(m);
    return s;
}

}  // namespace

mfgpu_status mfgpu_dbscan_segmented_noalloc(int n_segments, const int *d_seg_offsets, int n_obs, int n_features,
                                            const double *d_X, const double *d_weights, double epsilon,
                                            int min_observations, int *d_labels, int *d_n_clusters, void *stream)
try
{
    if (n_segments < 1 || n_segments > kMaxSegments)
        return fail(MFGPU_EINVAL, "n_segments = " + std::to_string(n_segments) + " must be in [1, " +
                                      std::to_string(kMaxSegments) + "]");
    if (n_obs < 0 || n_obs > kMaxPoints)
        return fail(MFGPU_EINVAL, "n_obs = " + std::to_string(n_obs) + " exceeds the fixed scratch capacity of " +
                                      std::to_string(kMaxPoints) + " observations");
    if (n_features < 1) return fail(MFGPU_EINVAL, "No features");
    if (!(epsilon >= 0)) return fail(MFGPU_EINVAL, "epsilon must be non-negative");
    if (min_observations < 1) return fail(MFGPU_EINVAL, "minObservations must be positive");
    if (!d_seg_offsets || !d_n_clusters || (n_obs > 0 && (!d_X || !d_labels)))
        return fail(MFGPU_EINVAL, "NULL argument");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    void *base = nullptr;
    cudaError_t e = scratch_address(&base);
    if (e != cudaSuccess) return fail(MFGPU_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    unsigned char *sb = static_cast<unsigned char *>(base);
    int *seg_of = reinterpret_cast<int *>(sb + kOffSegOf);
    int *parent = reinterpret_cast<int *>(sb + kOffParent);
    int *is_root = reinterpret_cast<int *>(sb + kOffIsRoot);
    unsigned char *core = sb + kOffCore;
    long long *pos = reinterpret_cast<long long *>(sb + kOffPos);
    long long *tiles = reinterpret_cast<long long *>(sb + kOffTiles);
    int *seg_off = reinterpret_cast<int *>(sb + kOffSegOff);
    double *xs = reinterpret_cast<double *>(sb + kOffXs);
    int *perm = reinterpret_cast<int *>(sb + kOffPerm);
    int *rank = reinterpret_cast<int *>(sb + kOffRank);
    int *fend = reinterpret_cast<int *>(sb + kOffFend);

    if (n_obs == 0)
    {
        e = cudaMemsetAsync(d_n_clusters, 0, sizeof(int) * n_segments, s);
        if (e != cudaSuccess) return fail(MFGPU_ECUDA, cudaGetErrorString(e));
        return MFGPU_OK;
    }
    DbParams p;
    p.X = d_X; p.nf = n_features; p.w = d_weights; p.eps = epsilon; p.min_obs = (double) min_observations;
    p.seg_of = seg_of; p.seg_off = seg_off; p.n = n_obs;
    const unsigned blocks = (unsigned) ((n_obs + kDbThreads - 1) / kDbThreads);
    const unsigned wblocks = (unsigned) ((n_obs + kDbWarps - 1) / kDbWarps);
    sanitize_offsets_kernel<<<1, 1, 0, s>>>(n_obs, n_segments, d_seg_offsets, seg_off);
    seg_of_kernel<<<blocks, kDbThreads, 0, s>>>(n_obs, n_segments, seg_off, seg_of);
    // one feature: every segment sorted on the device (bitonic network over
    // the next power of two, at most the scratch's capacity), so each point
    // visits its neighbours only
    const bool sorted1 = n_features == 1;
    const Db1Sorted q{xs, perm, rank, fend};
    if (sorted1)
    {
        int n2 = 1;
        while (n2 < n_obs) n2 <<= 1;
        const unsigned b2 = (unsigned) ((n2 + kDbThreads - 1) / kDbThreads);
        db1_iota_kernel<<<b2, kDbThreads, 0, s>>>(perm, n2);
        for (int k = 2; k <= n2; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) db1_bitonic_kernel<<<b2, kDbThreads, 0, s>>>(p, perm, n2, j, k);
        db1_gather_kernel<<<blocks, kDbThreads, 0, s>>>(p, perm, xs, rank);
        db1_fend_kernel<<<(n_segments + 127) / 128, 128, 0, s>>>(n_segments, seg_off, xs, fend);
        db1_core_kernel<<<wblocks, kDbThreads, 0, s>>>(p, q, core, parent);
        db1_union_kernel<<<wblocks, kDbThreads, 0, s>>>(p, q, core, parent);
    }
    else
    {
        db_core_kernel<<<wblocks, kDbThreads, 0, s>>>(p, core, parent);
        db_union_kernel<<<wblocks, kDbThreads, 0, s>>>(p, core, parent);
    }
    db_roots_kernel<<<blocks, kDbThreads, 0, s>>>(n_obs, core, parent, is_root);
    const long nt = (n_obs + kScanTile - 1) / kScanTile;
    scan_tile_sums_kernel<<<(unsigned) nt, kScanThreads, 0, s>>>(is_root, n_obs, tiles);
    scan_tile_offsets_kernel<<<1, kScanThreads, 0, s>>>(tiles, nt);
    scan_apply_kernel<<<(unsigned) nt, kScanThreads, 0, s>>>(is_root, n_obs, tiles, pos);
    if (sorted1) db1_label_kernel<<<wblocks, kDbThreads, 0, s>>>(p, q, core, parent, pos, d_labels);
    else db_label_kernel<<<wblocks, kDbThreads, 0, s>>>(p, core, parent, pos, d_labels);
    db_count_kernel<<<(n_segments + 127) / 128, 128, 0, s>>>(n_segments, seg_off, pos, d_n_clusters);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(MFGPU_ECUDA, cudaGetErrorString(e));
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}
