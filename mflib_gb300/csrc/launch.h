// launch.h -- host-side launchers for the device kernels (one definition per
// sample type lives in mf_f32.cu / mf_f64.cu; peaks and DBSCAN in
// peaks_dbscan.cu).  Used by the C ABI in api.cu.
#pragma once
#include <cstddef>
#include <mutex>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include "kernels_mf.cuh"
#include "kernels_util.cuh"
#include "tc_params.h"
#include "fix_params.h"
#include "mfgpu.h"

namespace mfgpu {

// Supported range of log2(N/2) for the overlap-save correlator.
template <class T> struct fft_limits;
template <> struct fft_limits<float> { static constexpr int lo = 5, hi = 12; };   // N = 64 .. 8192
template <> struct fft_limits<double> { static constexpr int lo = 5, hi = 11; };  // N = 64 .. 4096

// mode: 0 whole CTA, 1 whole CTA + spectrum prefetch, 2 two teams (shared
// length, normalisation rows from den_kernel), 3 two teams (shared length,
// normalisation computed in the CTA; shared_den false), 4 two 256-thread
// teams in a 512-thread CTA (several lengths, each team normalising its own
// templates; FP32, P >= 2048; shared_den false)
template <class T> size_t xcorr_smem_bytes(int log2p, bool shared_den, int mode, int S);
template <class T> cudaError_t launch_xcorr(int log2p, bool shared_den, int mode, const XcorrParams<T> &p,
                                            int nblocks, int ngroups, cudaStream_t s);
template <class T> cudaError_t launch_spectra(int log2p, const SpecParams<T> &p, int nt, cudaStream_t s);
// per-channel normalisation for template length L over nblocks * den_lags_per_cta(L) lags
template <class T> cudaError_t launch_den(const T *x, long ldx, int L, T *den, long ldd, T tol, int nblocks, int nch,
                                          cudaStream_t s);
// twiddle table of the FFT plan for P = 2^log2p (FftPlan layout)
template <class T> void twiddle_table(int log2p, std::vector<cx<T>> &out);
// the pass twiddles in the split layout (FftPlan::tws_off; correlator mode 4)
template <class T> void twiddle_split(int log2p, std::vector<cx<T>> &out);
// dead-trace flags of nch channels (rows of n samples, stride ldx): two
// launches; pmin/pmax are scratch of nch * nchunks entries each; range
// (optional) receives max - min per channel
template <class T> cudaError_t launch_dead(const T *x, long ldx, int nch, long n, unsigned char *dead, T *pmin,
                                           T *pmax, int nchunks, cudaStream_t s, float *range = nullptr);
// tensor-core correlator (FP32, one template length): shared memory per CTA,
// the template bank in MMA layout (ngroups * Gp slots), the persistent launch
size_t tc_smem_bytes(int Kp, int Gp);
// bf16: operands split into BF16 hi + lo instead of FP16 (precision comparison)
cudaError_t launch_tc_bank(const double *tmpl, const long *toff, const int *tlen, const int *grp_tid, int ngroups,
                           int Gp, int Kp, __half *B, float *bscale, bool bf16, cudaStream_t s);
cudaError_t launch_tc_xcorr(const TcParams &p, int nctas, bool bf16, cudaStream_t s);
// FP32 accuracy safeguards (kernels_fix.cuh): cancellation-free window
// variances with per-run statistics (float4 per 32 lags, row stride ldrs;
// den optional) and per-chunk statistics (float2 per 32 samples, row stride
// ldc), the per-run error bounds of the FFT and tensor-core
// correlators (flagged runs listed once each: a bit per run, the list and its
// count), and the fix-up of the listed runs.
cudaError_t launch_den_robust(const float *x, long ldx, int L, float *den, long ldd, float tol, float4 *rstat,
                              long ldrs, float2 *cst, long ldc, int nblocks, int nch, cudaStream_t s);
cudaError_t launch_fix_flag_fft(const float2 *cst, long ldc, long nchunks, int S, int N, int nblocks, int nch,
                                const float4 *rstat, long ldrs, int nruns, const int *dlags, const unsigned char *dead,
                                unsigned *fbits, int *flist, int *fcount, float coef2, cudaStream_t s);
cudaError_t launch_fix_flag_tc(const float *x, long ldx, int L, const float4 *rstat, long ldrs, int nruns,
                               const int *dlags, int tiles, int nch, const unsigned char *dead, const float *xrange,
                               float *off, unsigned *fbits, int *flist, int *fcount, float c1, float c2, float tau,
                               cudaStream_t s);
// *p = v in stream order
cudaError_t launch_set_int(int *p, int v, cudaStream_t s);
// warps per fix-up CTA whose sample rows (templates up to Lmax) fit dev_smem
// bytes (0: none fits)
template <class T> int fixup_warps(int Lmax, int dev_smem);
template <class T>
cudaError_t launch_fix_prep(const double *tmpl, const long *toff, const int *tlen, const int *btid, const long *boff,
                            const int *bL, int nbatch, T *bco, T *bsum, cudaStream_t s);
template <class T> cudaError_t launch_fixup(const FixParams<T> &p, int nctas, int warps, cudaStream_t s);
template <class T>
cudaError_t launch_fix_rescan(const T *rho, long ldr, int nt, int pk_stride, const unsigned char *dirty,
                              const int *row_S, const int *row_nblk, int S0, int nblk0, const int *nvalid, int pk_len,
                              T thr, int *cnt, int *idx, T *val, cudaStream_t s);
// single-channel detector (kernels_detect.cuh): reduction across templates,
// per-template transformed traces, per-detection refinement and amplitudes
template <class T>
cudaError_t launch_det_reduce(const T *rho, long ldr, int nt, long len, int use_abs, T *det, int *id, cudaStream_t s);
template <class T>
cudaError_t launch_det_single(const T *rho, long ldr, int nt, long len, int use_abs, T *out, cudaStream_t s);
template <class T>
cudaError_t launch_det_refine(const T *rho, long ldr, const T *x, long ldx, const struct DetectParams &q,
                              cudaStream_t s);
template <class T>
cudaError_t launch_amp(const double *b, int L, const T *y, long ld, int nw, double *gr, double *sr, int *valid,
                       cudaStream_t s);
// reference debug spectrum of one prepared template at FFT length nfft
template <class T> cudaError_t launch_ref_spectrum(const double *tmpl, int L, int nfft, T *out, cudaStream_t s);
// shift and stack (src/matchedFilter.cpp:1319-1364)
template <class T> cudaError_t launch_stack(const T *rho, long ldr, int nt, const int *shifts, const T *weights,
                                            int stack_abs, int outlen, T *out, cudaStream_t s);

// ---------------------------------------------------------------------------
// Dynamic shared-memory cap of one kernel, raised on demand and never
// lowered: objects driven from different host threads may launch the same
// kernel with different sizes at the same time, and lowering the cap between
// another thread's raise and its launch would fail that launch.
struct SmemCap
{
    std::mutex m;
    int cap[16] = {};
};
template <class K> inline cudaError_t raise_smem_cap(K kernel, size_t bytes, SmemCap &c)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(c.m);
    int *cap = dev >= 0 && dev < 16 ? &c.cap[dev] : nullptr;
    if (cap && (int) bytes <= *cap) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) bytes);
    if (e == cudaSuccess && cap) *cap = (int) bytes;
    return e;
}

// ---------------------------------------------------------------------------
// grow-only device buffer
struct DevBuf
{
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t need)
    {
        if (p && need <= bytes) return cudaSuccess;
        release();
        size_t b = (need < 64 ? 64 : need);
        b += b / 4;
        cudaError_t e = cudaMalloc(&p, b);
        if (e == cudaSuccess) bytes = b;
        else p = nullptr;
        return e;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <class U> U *as() const { return static_cast<U *>(p); }
};

// peak finder pipeline over ntr traces (rows of a matrix)
struct PeakWS
{
    DevBuf counts, offs, slot_idx, slot_val, cidx, cval, ctr, state, flags, pos, tiles, trace_beg, peak_off, peaks,
        counter, row, ht;
    long long npeaks = 0;
    long long cand_cap = 1 << 16;  // capacity of the packed candidate arrays
    std::vector<int> rows_on_device;  // the trace rows last uploaded to `row`
    template <class F> void each_buf(F &&f)
    {
        DevBuf *all[] = {&counts, &offs, &slot_idx, &slot_val, &cidx, &cval, &ctr, &state, &flags,
                         &pos, &tiles, &trace_beg, &peak_off, &peaks, &counter, &row, &ht};
        for (DevBuf *d : all) f(*d);
    }
    void release()
    {
        each_buf([](DevBuf &d) { d.release(); });
        npeaks = 0;
        cand_cap = 1 << 16;
        rows_on_device.clear();
    }
};

// Runs candidates + pruning + compaction; on return (stream synchronised)
// ws.peaks / ws.peak_off hold the result and host_peak_off (ntr+1) is filled.
// With `fused`, the candidates the correlator gathered (same threshold and
// trace length) replace the scan over the traces.  Otherwise `flags` (bit
// per 64 lags of each row, fwords words per row; see PeakTraces), when given,
// lets the scan skip the lags no value above the threshold lies in.
template <class T>
int run_peaks(const T *x, long ldx, const int *host_rows, int ntr, int len, double thr, int dist, PeakWS &ws,
              cudaStream_t s, long long *launches, long long *host_peak_off, std::string &err,
              const FusedSlots<T> *fused = nullptr, const unsigned *flags = nullptr, int fwords = 0);

// ---------------------------------------------------------------------------
// DBSCAN over segments
struct DbWS
{
    DevBuf X, w, seg_of, seg_off, parent, is_root, labels, nclusters, core, pos, tiles, xs, perm, rank;
    void release()
    {
        DevBuf *all[] = {&X, &w, &seg_of, &seg_off, &parent, &is_root, &labels, &nclusters, &core, &pos, &tiles,
                         &xs, &perm, &rank};
        for (DevBuf *d : all) d->release();
    }
};

int run_dbscan(int n, int nf, const double *X, const double *w, double eps, int min_obs, int nseg,
               const int *seg_off_host, int *labels_host, int *nclusters_host, DbWS &ws, cudaStream_t s,
               long long *launches, std::string &err);

// message returned by mfgpu_last_error() on the calling thread
void set_last_error(const std::string &msg);
// Status for an exception caught at the C ABI (called inside a catch
// handler): std::bad_alloc -> MFGPU_ENOMEM, std::invalid_argument and
// std::out_of_range -> MFGPU_EINVAL, anything else -> MFGPU_ESTATE, with
// the exception's text as the last error.  Exceptions never cross the ABI.
mfgpu_status status_of_exception() noexcept;

// device scan helper: out[0..n] = exclusive scan of in[0..n) (+ total)
cudaError_t device_excl_scan(const int *in, long n, long long *out, long long *tiles, cudaStream_t s,
                             long long *launches);
inline long scan_tiles_needed(long n) { return (n + kScanTile - 1) / kScanTile + 1; }

}  // namespace mfgpu
