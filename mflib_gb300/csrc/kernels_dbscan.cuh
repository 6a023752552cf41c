// kernels_dbscan.cuh -- DBSCAN (MFLib::DBSCAN::cluster, src/dbscan.cpp:187-214,
// which calls Intel DAAL dbscan::Batch<double>) on the device, for one or
// many independent segments.
//
// Semantics (DAAL's published algorithm):
//   N(i) = { j in segment(i) : ||x_i - x_j||_2 <= eps } including i;
//   core(i) iff sum_{j in N(i)} w_j >= minObservations (w = 1 unweighted);
//   clusters are the connected components of core points under the
//   eps-neighbour relation; DAAL visits observations in index order and
//   opens a new cluster at the first unassigned core point, so cluster ids
//   are ordered by each component's lowest core index;
//   a non-core point with a core neighbour takes the smallest id among its
//   neighbours' clusters (the first cluster to reach it); others are -1.
//
// Device formulation: one warp per point scans its segment; weighted
// neighbour sums; union-find with atomic CAS that always hooks the larger
// root under the smaller (so every component's root is its lowest core
// index); exclusive scan of root flags for the ids; then labels.
// One feature: |x_i - x_j| <= eps, which equals sqrt((x_i - x_j)^2) <= eps
// exactly in IEEE arithmetic and avoids the FP64 square root.
#pragma once
#include <cstdint>
#include "kernels_util.cuh"

namespace mfgpu {

constexpr int kDbThreads = 256;
constexpr int kDbWarps = kDbThreads / 32;

struct DbParams
{
    const double *X;        // [n x nf] row-major
    int nf;
    const double *w;        // weights or null
    double eps;
    double min_obs;
    const int *seg_of;      // segment of each point
    const int *seg_off;     // [nseg + 1]
    int n;
};

__device__ __forceinline__ bool db_near(const DbParams &p, int i, int j)
{
    if (p.nf == 1) return fabs(p.X[i] - p.X[j]) <= p.eps;
    const double *a = p.X + (long) i * p.nf, *b = p.X + (long) j * p.nf;
    double s = 0;
    for (int f = 0; f < p.nf; ++f)
    {
        double d = a[f] - b[f];
        s = fma(d, d, s);
    }
    return sqrt(s) <= p.eps;
}

// core flags: weighted neighbourhood size >= minObservations
static __global__ void __launch_bounds__(kDbThreads) db_core_kernel(DbParams p, unsigned char *core, int *parent)
{
    const int i = blockIdx.x * kDbWarps + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (i >= p.n) return;
    const int s = p.seg_of[i];
    const int jb = p.seg_off[s], je = p.seg_off[s + 1];
    double acc = 0;
    for (int j = jb + lane; j < je; j += 32)
        if (db_near(p, i, j)) acc += p.w ? p.w[j] : 1.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0)
    {
        core[i] = acc >= p.min_obs ? 1 : 0;
        parent[i] = i;
    }
}

// Root of x with path halving: each visited node is re-pointed at its
// grandparent.  Safe under concurrent unions: parents only ever move to an
// ancestor (unions hook a root under a smaller root), so the write never
// detaches a node from its component, and roots are never written here.
// Without it the predecessor unions of the 1-D case build chains as long as
// a component, and every find walks them.
__device__ __forceinline__ int db_find(volatile int *parent, int x)
{
    int p = parent[x];
    while (p != x)
    {
        const int g = parent[p];
        if (g != p) parent[x] = g;
        x = g;
        p = parent[x];
    }
    return x;
}

__device__ __forceinline__ void db_unite(int *parent, int a, int b)
{
    volatile int *vp = parent;
    for (int guard = 0; guard < (1 << 30); ++guard)
    {
        a = db_find(vp, a);
        b = db_find(vp, b);
        if (a == b) return;
        if (a > b) { int t = a; a = b; b = t; }
        int old = atomicCAS(parent + b, b, a);  // hook the larger root under the smaller
        if (old == b) return;
        b = old;
    }
}

// Components of the core points.  Several features: every core pair within
// eps is united.  One feature: ordered by (x, index), the components are the
// runs of consecutive core points whose gaps are at most eps (any core pair
// within eps spans only such gaps), so each core point is united with its
// predecessor in that order alone -- O(n) unions instead of O(n k) on the
// same few roots.
static __global__ void __launch_bounds__(kDbThreads) db_union_kernel(DbParams p, const unsigned char *core, int *parent)
{
    const int i = blockIdx.x * kDbWarps + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (i >= p.n || !core[i]) return;
    const int s = p.seg_of[i];
    const int jb = p.seg_off[s], je = p.seg_off[s + 1];
    if (p.nf != 1)
    {
        for (int j = i + 1 + lane; j < je; j += 32)
            if (core[j] && db_near(p, i, j)) db_unite(parent, i, j);
        return;
    }
    const double xi = p.X[i];
    double bx = 0.0;
    int bj = -1;  // predecessor: the largest (x_j, j) below (x_i, i)
    for (int j = jb + lane; j < je; j += 32)
    {
        if (j == i || !core[j]) continue;
        const double xj = p.X[j];
        const bool below = xj < xi || (xj == xi && j < i);
        if (below && (bj < 0 || xj > bx || (xj == bx && j > bj)))
        {
            bx = xj;
            bj = j;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        const double ox = __shfl_xor_sync(0xffffffffu, bx, o);
        const int oj = __shfl_xor_sync(0xffffffffu, bj, o);
        if (oj >= 0 && (bj < 0 || ox > bx || (ox == bx && oj > bj)))
        {
            bx = ox;
            bj = oj;
        }
    }
    if (lane == 0 && bj >= 0 && fabs(xi - bx) <= p.eps) db_unite(parent, i, bj);
}

// Root without writes: in the roots pass a halving write from one thread
// could land after another thread stored its node's final root and replace
// it with an intermediate ancestor.
__device__ __forceinline__ int db_find_ro(const volatile int *parent, int x)
{
    int p = parent[x];
    while (p != x)
    {
        x = p;
        p = parent[x];
    }
    return x;
}

static __global__ void db_roots_kernel(int n, const unsigned char *core, int *parent, int *is_root)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (!core[i]) { is_root[i] = 0; return; }
    int r = db_find_ro(parent, i);
    parent[i] = r;
    is_root[i] = r == i ? 1 : 0;
}

// labels: core -> id of its root; border -> smallest id among core neighbours
static __global__ void __launch_bounds__(kDbThreads) db_label_kernel(DbParams p, const unsigned char *core, const int *root,
                                                                     const long long *root_pos, int *labels)
{
    const int i = blockIdx.x * kDbWarps + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (i >= p.n) return;
    const int s = p.seg_of[i];
    const int jb = p.seg_off[s], je = p.seg_off[s + 1];
    const long long base = root_pos[jb];
    if (core[i])
    {
        if (lane == 0) labels[i] = (int) (root_pos[root[i]] - base);
        return;
    }
    long long best = 0x7fffffffffffffffLL;
    for (int j = jb + lane; j < je; j += 32)
    {
        if (!core[j] || !db_near(p, i, j)) continue;
        long long id = root_pos[root[j]] - base;
        best = id < best ? id : best;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        long long v = __shfl_xor_sync(0xffffffffu, best, o);
        best = v < best ? v : best;
    }
    if (lane == 0) labels[i] = best == 0x7fffffffffffffffLL ? -1 : (int) best;
}

// ----------------------------------------------------------------------------
// One feature with the points of every segment sorted by (x, index) on the
// host: xs[r] is the r-th smallest value of its segment (positions keep the
// segment offsets), perm[r] its point, rank[i] the position of point i.  The
// eps-neighbourhood of a point is then the contiguous range of positions
// [lo, hi) found by binary search with the same predicate |x_i - x_j| <= eps
// (a rounded difference is monotone in x_j), so every pass visits the
// neighbours only: O(n log n + sum of neighbourhood sizes) instead of a scan
// of the whole segment per point.
struct Db1Sorted
{
    const double *xs;
    const int *perm;
    const int *rank;
    // per segment, the end of its non-NaN values (NaN sorted last, no
    // neighbour of anything); null when no value is NaN
    const int *fend;
};

__device__ __forceinline__ int db1_end(const DbParams &p, const Db1Sorted &q, int s)
{
    return q.fend ? q.fend[s] : p.seg_off[s + 1];
}

// [lo, hi): positions of the segment [jb, je) within eps of the value xi
__device__ __forceinline__ void db1_range(const double *xs, int jb, int je, double xi, double eps, int &lo, int &hi)
{
    int a = jb, b = je;  // first position with xi - xs <= eps
    while (a < b)
    {
        const int m = (a + b) >> 1;
        if (xi - xs[m] <= eps) b = m;
        else a = m + 1;
    }
    lo = a;
    b = je;              // first position with xs - xi > eps
    while (a < b)
    {
        const int m = (a + b) >> 1;
        if (xs[m] - xi <= eps) a = m + 1;
        else b = m;
    }
    hi = a;
}

static __global__ void __launch_bounds__(kDbThreads) db1_core_kernel(DbParams p, Db1Sorted q, unsigned char *core,
                                                                     int *parent)
{
    const int i = blockIdx.x * kDbWarps + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (i >= p.n) return;
    const int s = p.seg_of[i];
    int lo = 0, hi = 0;
    if (lane == 0) db1_range(q.xs, p.seg_off[s], db1_end(p, q, s), p.X[i], p.eps, lo, hi);
    lo = __shfl_sync(0xffffffffu, lo, 0);
    hi = __shfl_sync(0xffffffffu, hi, 0);
    double acc = 0;
    for (int r = lo + lane; r < hi; r += 32) acc += p.w ? p.w[q.perm[r]] : 1.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0)
    {
        core[i] = acc >= p.min_obs ? 1 : 0;
        parent[i] = i;
    }
}

// each core point united with the nearest core point before it in the sorted
// order when that one lies within eps (the runs of consecutive core points
// with gaps <= eps are the components, as in db_union_kernel's 1-D case)
static __global__ void __launch_bounds__(kDbThreads) db1_union_kernel(DbParams p, Db1Sorted q, const unsigned char *core,
                                                                      int *parent)
{
    const int i = blockIdx.x * kDbWarps + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (i >= p.n || !core[i]) return;
    const int s = p.seg_of[i];
    const int jb = p.seg_off[s];
    const double xi = p.X[i];
    for (int r0 = q.rank[i] - 1; r0 >= jb; r0 -= 32)
    {
        const int r = r0 - lane;
        const bool in = r >= jb && xi - q.xs[r] <= p.eps;
        const bool hit = in && core[q.perm[r]];
        const unsigned hm = __ballot_sync(0xffffffffu, hit), im = __ballot_sync(0xffffffffu, in);
        if (hm)
        {
            const int l = __ffs(hm) - 1;  // the nearest position (lowest lane)
            if (lane == l) db_unite(parent, i, q.perm[r]);
            return;
        }
        if (im != 0xffffffffu) return;  // left the neighbourhood before finding a core point
    }
}

// border points: the smallest cluster id among their core neighbours
static __global__ void __launch_bounds__(kDbThreads) db1_label_kernel(DbParams p, Db1Sorted q, const unsigned char *core,
                                                                      const int *root, const long long *root_pos,
                                                                      int *labels)
{
    const int i = blockIdx.x * kDbWarps + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (i >= p.n) return;
    const int s = p.seg_of[i];
    const int jb = p.seg_off[s], je = db1_end(p, q, s);
    const long long base = root_pos[jb];
    if (core[i])
    {
        if (lane == 0) labels[i] = (int) (root_pos[root[i]] - base);
        return;
    }
    int lo = 0, hi = 0;
    if (lane == 0) db1_range(q.xs, jb, je, p.X[i], p.eps, lo, hi);
    lo = __shfl_sync(0xffffffffu, lo, 0);
    hi = __shfl_sync(0xffffffffu, hi, 0);
    long long best = 0x7fffffffffffffffLL;
    for (int r = lo + lane; r < hi; r += 32)
    {
        const int j = q.perm[r];
        if (!core[j]) continue;
        const long long id = root_pos[root[j]] - base;
        best = id < best ? id : best;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        const long long v = __shfl_xor_sync(0xffffffffu, best, o);
        best = v < best ? v : best;
    }
    if (lane == 0) labels[i] = best == 0x7fffffffffffffffLL ? -1 : (int) best;
}

// Device-side preparation of Db1Sorted, for callers whose data are already
// on the device: perm (n2 = a power of two >= n entries, padding indices
// n .. n2-1 sorting last) sorted by (segment, value, index) with NaN after
// every number in its segment, by a bitonic network (one launch per step),
// then the sorted values, each point's position and every segment's end of
// non-NaN values.
__device__ __forceinline__ bool db1_less(const DbParams &p, int a, int b)
{
    if (a >= p.n) return b >= p.n && a < b;
    if (b >= p.n) return true;
    const int sa = p.seg_of[a], sb = p.seg_of[b];
    if (sa != sb) return sa < sb;
    const double xa = p.X[a], xb = p.X[b];
    const bool na = isnan(xa), nb = isnan(xb);
    if (na != nb) return nb;
    if (!na && xa != xb) return xa < xb;
    return a < b;
}

static __global__ void db1_iota_kernel(int *perm, int n2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n2) perm[i] = i;
}

// one compare-exchange step (distance j, merge size k) of the bitonic network
static __global__ void db1_bitonic_kernel(DbParams p, int *perm, int n2, int j, int k)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n2) return;
    const int l = i ^ j;
    if (l <= i) return;
    const int a = perm[i], b = perm[l];
    const bool up = (i & k) == 0;
    if (up ? db1_less(p, b, a) : db1_less(p, a, b))
    {
        perm[i] = b;
        perm[l] = a;
    }
}

static __global__ void db1_gather_kernel(DbParams p, const int *perm, double *xs, int *rank)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= p.n) return;
    const int i = perm[r];
    xs[r] = p.X[i];
    rank[i] = r;
}

// fend[s]: the first position of segment s holding NaN (its end if none)
static __global__ void db1_fend_kernel(int nseg, const int *seg_off, const double *xs, int *fend)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    int a = seg_off[s], b = seg_off[s + 1];
    while (a < b)
    {
        const int m = (a + b) >> 1;
        if (isnan(xs[m])) b = m;
        else a = m + 1;
    }
    fend[s] = a;
}

static __global__ void db_count_kernel(int nseg, const int *seg_off, const long long *root_pos, int *n_clusters)
{
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    n_clusters[s] = (int) (root_pos[seg_off[s + 1]] - root_pos[seg_off[s]]);
}

}  // namespace mfgpu
