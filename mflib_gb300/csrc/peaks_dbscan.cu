// peaks_dbscan.cu -- host drivers of the peak-finder and DBSCAN pipelines
// (kernels in kernels_peaks.cuh / kernels_dbscan.cuh) and the device scan.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>
#include "launch.h"
#include "kernels_peaks.cuh"
#include "kernels_dbscan.cuh"

namespace mfgpu {

#define MF_TRY(expr)                                                                                               \
    do                                                                                                             \
    {                                                                                                              \
        cudaError_t e_ = (expr);                                                                                   \
        if (e_ != cudaSuccess)                                                                                     \
        {                                                                                                          \
            err = std::string(#expr) + ": " + cudaGetErrorString(e_);                                              \
            return -1;                                                                                             \
        }                                                                                                          \
    } while (0)

cudaError_t device_excl_scan(const int *in, long n, long long *out, long long *tiles, cudaStream_t s,
                             long long *launches)
{
    long nt = (n + kScanTile - 1) / kScanTile;
    if (nt == 0) return cudaMemsetAsync(out, 0, sizeof(long long), s);
    scan_tile_sums_kernel<<<(unsigned) nt, kScanThreads, 0, s>>>(in, n, tiles);
    scan_tile_offsets_kernel<<<1, kScanThreads, 0, s>>>(tiles, nt);
    scan_apply_kernel<<<(unsigned) nt, kScanThreads, 0, s>>>(in, n, tiles, out);
    if (launches) *launches += 3;
    return cudaGetLastError();
}

template <class T>
int run_peaks(const T *x, long ldx, const int *host_rows, int ntr, int len, double thr, int dist, PeakWS &ws,
              cudaStream_t s, long long *launches, long long *host_peak_off, std::string &err,
              const FusedSlots<T> *fused, const unsigned *flags, int fwords)
{
    ws.npeaks = 0;
    if (ntr <= 0) return 0;
    if (len <= 0)
    {
        for (int t = 0; t <= ntr; ++t) host_peak_off[t] = 0;
        return 0;
    }
    // chunks: kPkChunk lags for the stand-alone scan, one correlator block
    // (fused.S lags) when the correlator gathered the candidates
    const int nchunks = fused ? fused->nblk : (len + kPkChunk - 1) / kPkChunk;
    const size_t nslots = (size_t) ntr * nchunks;
    {
        void *old = ws.row.p;
        MF_TRY(ws.row.ensure(sizeof(int) * ntr));
        if (ws.row.p != old) ws.rows_on_device.clear();  // a new buffer holds no rows
    }
    MF_TRY(ws.trace_beg.ensure(sizeof(long long) * (ntr + 1)));
    MF_TRY(ws.peak_off.ensure(sizeof(long long) * (ntr + 1)));
    MF_TRY(ws.counts.ensure(sizeof(int) * nslots));
    MF_TRY(ws.offs.ensure(sizeof(long long) * (nslots + 1)));
    if (fused) MF_TRY(ws.ht.ensure(nslots));
    else
    {
        MF_TRY(ws.slot_idx.ensure(sizeof(int) * nslots * kPkCap));
        MF_TRY(ws.slot_val.ensure(sizeof(T) * nslots * kPkCap));
    }
    MF_TRY(ws.counter.ensure(4 * sizeof(int)));  // [0] undecided after the last round, [1] overflow
    // the rows rarely change between calls: upload only when they do (an
    // upload queues behind any large host-to-device copy in flight)
    if (ws.rows_on_device.size() != (size_t) ntr ||
        !std::equal(host_rows, host_rows + ntr, ws.rows_on_device.begin()))
    {
        MF_TRY(cudaMemcpyAsync(ws.row.p, host_rows, sizeof(int) * ntr, cudaMemcpyHostToDevice, s));
        MF_TRY(cudaStreamSynchronize(s));  // host_rows may be a temporary
        ws.rows_on_device.assign(host_rows, host_rows + ntr);
    }
    int *undecided = ws.counter.as<int>(), *overflow = ws.counter.as<int>() + 1;
    const long long *ncand_dev = ws.offs.as<long long>() + nslots;

    PeakTraces<T> tr;
    tr.x = x; tr.ldx = ldx; tr.row = ws.row.as<int>(); tr.len = len; tr.thr = (T) thr;
    tr.flags = fused ? nullptr : flags; tr.fwords = fwords;
    const dim3 grid(nchunks, ntr);
    const bool prune = dist > 0;
    for (int attempt = 0; attempt < 4; ++attempt)
    {
        const long long cap = ws.cand_cap;
        MF_TRY(ws.cidx.ensure(sizeof(int) * cap));
        MF_TRY(ws.cval.ensure(sizeof(T) * cap));
        MF_TRY(ws.ctr.ensure(sizeof(int) * cap));
        MF_TRY(ws.state.ensure((size_t) cap));
        MF_TRY(ws.flags.ensure(sizeof(int) * cap));
        MF_TRY(ws.pos.ensure(sizeof(long long) * (cap + 1)));
        MF_TRY(ws.peaks.ensure(sizeof(int) * cap));
        MF_TRY(ws.tiles.ensure(sizeof(long long) * (scan_tiles_needed(std::max<long>((long) nslots, (long) cap) + 1) + 8)));
        MF_TRY(cudaMemsetAsync(ws.counter.p, 0, 4 * sizeof(int), s));

        if (fused)
            peak_seam_kernel<T><<<(unsigned) ((nslots + 255) / 256), 256, 0, s>>>(tr, ntr, *fused, ws.counts.as<int>(),
                                                                                ws.ht.as<unsigned char>());
        else
            peak_cand_kernel<T><<<grid, kPkThreads, 0, s>>>(tr, nchunks, ws.counts.as<int>(), ws.slot_idx.as<int>(),
                                                            ws.slot_val.as<T>());
        ++*launches;
        MF_TRY(cudaGetLastError());
        MF_TRY(device_excl_scan(ws.counts.as<int>(), (long) nslots, ws.offs.as<long long>(),
                                ws.tiles.as<long long>(), s, launches));
        peak_trace_beg_kernel<<<(ntr + 1 + 127) / 128, 128, 0, s>>>(ntr, nchunks, ws.offs.as<long long>(), cap,
                                                                    ws.trace_beg.as<long long>());
        if (fused)
            peak_gather_fused_kernel<T><<<dim3((nchunks + kPkThreads / 32 * kPkGatherSpan - 1) /
                                                   (kPkThreads / 32 * kPkGatherSpan),
                                               ntr),
                                          kPkThreads, 0, s>>>(
                tr, *fused, ws.counts.as<int>(), ws.ht.as<unsigned char>(), ws.offs.as<long long>(), ws.cidx.as<int>(),
                ws.cval.as<T>(), ws.ctr.as<int>(), cap, overflow);
        else
            peak_gather_kernel<T><<<grid, kPkThreads, 0, s>>>(tr, nchunks, ws.counts.as<int>(),
                                                              ws.offs.as<long long>(), ws.slot_idx.as<int>(),
                                                              ws.slot_val.as<T>(), ws.cidx.as<int>(), ws.cval.as<T>(),
                                                              ws.ctr.as<int>(), cap, overflow);
        *launches += 2;
        MF_TRY(cudaGetLastError());
        const unsigned gblocks = (unsigned) ((cap + kPkThreads - 1) / kPkThreads);
        if (prune) MF_TRY(cudaMemsetAsync(ws.state.p, PK_UNDECIDED, (size_t) cap, s));
        // Pruning rounds, checked in batches: every round accepts at least
        // the highest-priority undecided candidate of each trace.
        long long rounds_done = 0;
        int left = 0;
        long long ncand = 0;
        int ovf = 0;
        for (;;)
        {
            if (prune)
            {
                const int batch = rounds_done == 0 ? 6 : 16;
                for (int r = 0; r < batch; ++r)
                {
                    MF_TRY(cudaMemsetAsync(undecided, 0, sizeof(int), s));
                    peak_decide_kernel<T><<<gblocks, kPkThreads, 0, s>>>(
                        ncand_dev, cap, ws.cidx.as<int>(), ws.cval.as<T>(), ws.ctr.as<int>(),
                        ws.trace_beg.as<long long>(), ws.state.as<unsigned char>(), dist, undecided);
                    peak_suppress_kernel<<<gblocks, kPkThreads, 0, s>>>(ncand_dev, cap, ws.cidx.as<int>(),
                                                                        ws.ctr.as<int>(), ws.trace_beg.as<long long>(),
                                                                        ws.state.as<unsigned char>(), dist);
                    *launches += 2;
                }
                rounds_done += batch;
                MF_TRY(cudaGetLastError());
            }
            peak_flags_kernel<<<gblocks, kPkThreads, 0, s>>>(ncand_dev, cap, ws.state.as<unsigned char>(),
                                                             prune ? 0 : 1, ws.flags.as<int>());
            ++*launches;
            MF_TRY(device_excl_scan(ws.flags.as<int>(), (long) cap, ws.pos.as<long long>(), ws.tiles.as<long long>(),
                                    s, launches));
            peak_compact_kernel<<<gblocks, kPkThreads, 0, s>>>(ncand_dev, cap, ws.flags.as<int>(),
                                                               ws.pos.as<long long>(), ws.cidx.as<int>(),
                                                               ws.peaks.as<int>());
            peak_trace_offsets_kernel<<<(ntr + 1 + 127) / 128, 128, 0, s>>>(ntr, ws.trace_beg.as<long long>(),
                                                                            ws.pos.as<long long>(),
                                                                            ws.peak_off.as<long long>());
            *launches += 2;
            MF_TRY(cudaGetLastError());
            MF_TRY(cudaMemcpyAsync(host_peak_off, ws.peak_off.p, sizeof(long long) * (ntr + 1),
                                   cudaMemcpyDeviceToHost, s));
            MF_TRY(cudaMemcpyAsync(&ncand, ncand_dev, sizeof(long long), cudaMemcpyDeviceToHost, s));
            MF_TRY(cudaMemcpyAsync(&left, undecided, sizeof(int), cudaMemcpyDeviceToHost, s));
            MF_TRY(cudaMemcpyAsync(&ovf, overflow, sizeof(int), cudaMemcpyDeviceToHost, s));
            MF_TRY(cudaStreamSynchronize(s));
            if (ovf || ncand > cap) break;
            if (!prune || left == 0) break;
            if (rounds_done > ncand + 16)
            {
                err = "peak pruning did not converge";
                return -1;
            }
        }
        if (ovf || ncand > cap)
        {
            ws.cand_cap = std::max<long long>(2 * cap, ncand + ncand / 4 + 1024);
            continue;
        }
        ws.npeaks = host_peak_off[ntr];
        return 0;
    }
    err = "peak candidate capacity could not be sized";
    return -1;
}
template int run_peaks<float>(const float *, long, const int *, int, int, double, int, PeakWS &, cudaStream_t,
                              long long *, long long *, std::string &, const FusedSlots<float> *,
                              const unsigned *, int);
template int run_peaks<double>(const double *, long, const int *, int, int, double, int, PeakWS &, cudaStream_t,
                               long long *, long long *, std::string &, const FusedSlots<double> *,
                               const unsigned *, int);

int run_dbscan(int n, int nf, const double *X, const double *w, double eps, int min_obs, int nseg,
               const int *seg_off_host, int *labels_host, int *nclusters_host, DbWS &ws, cudaStream_t s,
               long long *launches, std::string &err)
{
    if (n <= 0)
    {
        for (int i = 0; i < nseg; ++i) nclusters_host[i] = 0;
        return 0;
    }
    MF_TRY(ws.X.ensure(sizeof(double) * (size_t) n * nf));
    MF_TRY(ws.w.ensure(sizeof(double) * (size_t) n));
    MF_TRY(ws.seg_of.ensure(sizeof(int) * (size_t) n));
    MF_TRY(ws.seg_off.ensure(sizeof(int) * (size_t) (nseg + 1)));
    MF_TRY(ws.parent.ensure(sizeof(int) * (size_t) n));
    MF_TRY(ws.is_root.ensure(sizeof(int) * (size_t) n));
    MF_TRY(ws.labels.ensure(sizeof(int) * (size_t) n));
    MF_TRY(ws.nclusters.ensure(sizeof(int) * (size_t) nseg));
    MF_TRY(ws.core.ensure((size_t) n));
    MF_TRY(ws.pos.ensure(sizeof(long long) * (size_t) (n + 1)));
    MF_TRY(ws.tiles.ensure(sizeof(long long) * (scan_tiles_needed(n + 1) + 8)));

    std::vector<int> seg_of(n);
    for (int sg = 0; sg < nseg; ++sg)
        for (int i = seg_off_host[sg]; i < seg_off_host[sg + 1]; ++i) seg_of[i] = sg;
    // one feature: every segment's points sorted by (x, index), so each point
    // visits its neighbourhood only (Db1Sorted).  A NaN has no order and no
    // neighbour; data holding one keeps the full scans.
    bool sorted1 = nf == 1;
    for (int i = 0; sorted1 && i < n; ++i) sorted1 = !std::isnan(X[i]);
    std::vector<double> xs;
    std::vector<int> perm, rank;
    if (sorted1)
    {
        xs.resize(n);
        perm.resize(n);
        rank.resize(n);
        for (int i = 0; i < n; ++i) perm[i] = i;
        for (int sg = 0; sg < nseg; ++sg)
            std::sort(perm.begin() + seg_off_host[sg], perm.begin() + seg_off_host[sg + 1],
                      [&](int a, int b) { return X[a] < X[b] || (X[a] == X[b] && a < b); });
        for (int r = 0; r < n; ++r)
        {
            xs[r] = X[perm[r]];
            rank[perm[r]] = r;
        }
        MF_TRY(ws.xs.ensure(sizeof(double) * (size_t) n));
        MF_TRY(ws.perm.ensure(sizeof(int) * (size_t) n));
        MF_TRY(ws.rank.ensure(sizeof(int) * (size_t) n));
        MF_TRY(cudaMemcpyAsync(ws.xs.p, xs.data(), sizeof(double) * (size_t) n, cudaMemcpyHostToDevice, s));
        MF_TRY(cudaMemcpyAsync(ws.perm.p, perm.data(), sizeof(int) * (size_t) n, cudaMemcpyHostToDevice, s));
        MF_TRY(cudaMemcpyAsync(ws.rank.p, rank.data(), sizeof(int) * (size_t) n, cudaMemcpyHostToDevice, s));
    }
    MF_TRY(cudaMemcpyAsync(ws.X.p, X, sizeof(double) * (size_t) n * nf, cudaMemcpyHostToDevice, s));
    if (w) MF_TRY(cudaMemcpyAsync(ws.w.p, w, sizeof(double) * (size_t) n, cudaMemcpyHostToDevice, s));
    MF_TRY(cudaMemcpyAsync(ws.seg_of.p, seg_of.data(), sizeof(int) * (size_t) n, cudaMemcpyHostToDevice, s));
    MF_TRY(cudaMemcpyAsync(ws.seg_off.p, seg_off_host, sizeof(int) * (size_t) (nseg + 1), cudaMemcpyHostToDevice,
                           s));

    DbParams p;
    p.X = ws.X.as<double>(); p.nf = nf; p.w = w ? ws.w.as<double>() : nullptr; p.eps = eps;
    p.min_obs = (double) min_obs; p.seg_of = ws.seg_of.as<int>(); p.seg_off = ws.seg_off.as<int>(); p.n = n;
    const unsigned blocks = (unsigned) ((n + kDbThreads - 1) / kDbThreads);   // one thread per point
    const unsigned wblocks = (unsigned) ((n + kDbWarps - 1) / kDbWarps);      // one warp per point
    Db1Sorted q{ws.xs.as<double>(), ws.perm.as<int>(), ws.rank.as<int>()};
    if (sorted1)
    {
        db1_core_kernel<<<wblocks, kDbThreads, 0, s>>>(p, q, ws.core.as<unsigned char>(), ws.parent.as<int>());
        db1_union_kernel<<<wblocks, kDbThreads, 0, s>>>(p, q, ws.core.as<unsigned char>(), ws.parent.as<int>());
    }
    else
    {
        db_core_kernel<<<wblocks, kDbThreads, 0, s>>>(p, ws.core.as<unsigned char>(), ws.parent.as<int>());
        db_union_kernel<<<wblocks, kDbThreads, 0, s>>>(p, ws.core.as<unsigned char>(), ws.parent.as<int>());
    }
    db_roots_kernel<<<blocks, kDbThreads, 0, s>>>(n, ws.core.as<unsigned char>(), ws.parent.as<int>(),
                                                  ws.is_root.as<int>());
    *launches += 3;
    MF_TRY(cudaGetLastError());
    MF_TRY(device_excl_scan(ws.is_root.as<int>(), n, ws.pos.as<long long>(), ws.tiles.as<long long>(), s,
                            launches));
    if (sorted1)
        db1_label_kernel<<<wblocks, kDbThreads, 0, s>>>(p, q, ws.core.as<unsigned char>(), ws.parent.as<int>(),
                                                       ws.pos.as<long long>(), ws.labels.as<int>());
    else
        db_label_kernel<<<wblocks, kDbThreads, 0, s>>>(p, ws.core.as<unsigned char>(), ws.parent.as<int>(),
                                                      ws.pos.as<long long>(), ws.labels.as<int>());
    db_count_kernel<<<(nseg + 127) / 128, 128, 0, s>>>(nseg, ws.seg_off.as<int>(), ws.pos.as<long long>(),
                                                       ws.nclusters.as<int>());
    *launches += 2;
    MF_TRY(cudaGetLastError());
    MF_TRY(cudaMemcpyAsync(labels_host, ws.labels.p, sizeof(int) * (size_t) n, cudaMemcpyDeviceToHost, s));
    MF_TRY(cudaMemcpyAsync(nclusters_host, ws.nclusters.p, sizeof(int) * (size_t) nseg, cudaMemcpyDeviceToHost, s));
    // the host vectors above must outlive the copies
    MF_TRY(cudaStreamSynchronize(s));
    return 0;
}

}  // namespace mfgpu
