// api.cu -- the C ABI of libmfgpu.so (declared in include/mfgpu.h).
//
// Host-side objects mirror the reference classes: mfgpu_mf is
// MFLib::MatchedFilter<T> (src/matchedFilter.cpp), mfgpu_peaks is
// MFLib::PeakFinder<T> (src/peakFinder.cpp), mfgpu_dbscan is MFLib::DBSCAN
// (src/dbscan.cpp).  Argument checks follow the reference's exceptions:
// std::invalid_argument -> MFGPU_EINVAL, std::runtime_error -> MFGPU_ESTATE.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <string>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <vector>
#include "mfgpu.h"
#include "launch.h"
#include "kernels_detect.cuh"
#include "kernels_ring.cuh"

using namespace mfgpu;

namespace {

thread_local std::string g_err;

mfgpu_status fail(mfgpu_status s, const std::string &msg)
{
    g_err = msg;
    return s;
}

mfgpu_status cuda_fail(cudaError_t e, const char *what)
{
    return fail(e == cudaErrorMemoryAllocation ? MFGPU_ENOMEM : MFGPU_ECUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

#define CU(expr)                                                                                                   \
    do                                                                                                             \
    {                                                                                                              \
        cudaError_t e_ = (expr);                                                                                   \
        if (e_ != cudaSuccess) return cuda_fail(e_, #expr);                                                        \
    } while (0)

struct DeviceGuard
{
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard()
    {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

// computeWindowLength, src/matchedFilterParameters.cpp:47-104 (with the
// guards of computeOptimalFFTAndBlockLength, :371-385).  The operation-count
// table and the candidate lengths are the reference's, so the chosen
// (FFT length, block length) pair is identical.
const double kFftFlops[21] = {18,       59,       138,       303,       660,       1441,     3150,
                              6875,     14952,    32373,     69762,     149647,    319644,   680105,
                              1441974,  3047619,  6422736,   13500637,  28311786,  59244791, 59244791 * 2.09};

// The FFT and block length minimising blocks x flops over the table
// (src/matchedFilterParameters.cpp:47-104, computeWindowLength): the rule
// MatchedFilterParameters::getFFTLength applies, an error only when the
// template is longer than the signal.
mfgpu_status window_length(int nb, int nx, int *nfft, int *L)
{
    if (nb < 1) return fail(MFGPU_EINVAL, "Filter length must be positive");
    if (nb > nx) return fail(MFGPU_EINVAL, "nb = " + std::to_string(nb) + " cannot exceed nx = " + std::to_string(nx));
    int start = -1;
    for (int i = 0; i < 21; ++i)
        if ((uint64_t) 1 << (i + 1) > (uint64_t) (nb - 1)) { start = i; break; }
    if (start < 0)
    {
        int p = 1;
        if (nx > 1) p = (int) std::pow(2.0, std::ceil(std::log2((double) nx)));
        *nfft = p;
        *L = p - (nb - 1);
        return MFGPU_OK;
    }
    double best = std::numeric_limits<double>::max();
    int bn = 0, bl = 0;
    for (int i = start; i < 21; ++i)
    {
        int len = 1 << (i + 1);
        int lt = len - (nb - 1);
        double obj = std::ceil((double) nx / (double) lt) * kFftFlops[i];
        if (obj < best) { best = obj; bn = len; bl = lt; }
    }
    *nfft = bn;
    *L = bl;
    return MFGPU_OK;
}

// computeOptimalFFTAndBlockLength (src/matchedFilterParameters.cpp:371-385):
// the signal must be longer than the filter
mfgpu_status fft_sizes(int nb, int nx, int *nfft, int *L)
{
    if (nb < 1) return fail(MFGPU_EINVAL, "Filter length must be positive");
    if (nx <= nb)
        return fail(MFGPU_EINVAL, "Signal length = " + std::to_string(nx) + " must exceed filter length = " +
                                      std::to_string(nb));
    return window_length(nb, nx, nfft, L);
}

}  // namespace

void mfgpu::set_last_error(const std::string &msg) { g_err = msg; }

mfgpu_status mfgpu::status_of_exception() noexcept
{
    mfgpu_status st = MFGPU_ESTATE;
    const char *what = "unknown exception";
    try
    {
        throw;
    }
    catch (const std::bad_alloc &e)
    {
        st = MFGPU_ENOMEM;
        what = e.what();
    }
    catch (const std::invalid_argument &e)
    {
        st = MFGPU_EINVAL;
        what = e.what();
    }
    catch (const std::out_of_range &e)
    {
        st = MFGPU_EINVAL;
        what = e.what();
    }
    catch (const std::exception &e)
    {
        what = e.what();
    }
    catch (...)
    {
    }
    try
    {
        g_err = std::string("host exception: ") + what;
    }
    catch (...)
    {
        // no memory for the message either: keep the status
    }
    return st;
}

// ============================================================================
// Overlap-save plan of one length bucket beside the primary plan (the
// templates of a mixed-length bank split by length, each bucket with its own
// FFT length, block length, organisation, spectra and work groups).
struct MfBucket
{
    int log2p = 0, nfft = 0, S = 0, nblocks = 0, mode = 0, ngroups = 0, ntemplates = 0;
    DevBuf Bc, tw, tws, grp_chan, grp_tb, grp_te, tids;
    template <class F> void each_buf(F &&f)
    {
        DevBuf *all[] = {&Bc, &tw, &tws, &grp_chan, &grp_tb, &grp_te, &tids};
        for (DevBuf *d : all) f(*d);
    }
};

struct mfgpu_mf
{
    int prec = 4;
    int dev = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    bool initialized = false, have = false, timed = false;
    int mode = MFGPU_MULTI_CHANNEL, nt = 0, n = 0, maxLen = 0, minLen = 0, nch = 0;
    std::vector<int> lens, tchan, nvalid;
    std::vector<double> tmpl;
    std::vector<long> toff;
    bool can_stack = false;
    std::vector<int> shifts;
    std::vector<double> weights;
    int stack_abs = 1;
    bool ref_layout = true;
    // overlap-save plan
    int nfft = 0, log2p = 0, S = 0, nblocks = 0, ngroups = 0, maxvalid = 0;
    bool shared_den = false;
    int mode_x = 0;  // correlator organisation (launch_xcorr mode)
    // staged upload (mfgpu_mf_stage_channel_signals): copies run on
    // copy_stream into xstage; the next apply (or any other signal access)
    // waits for copy_done and swaps xstage in for x.  x_ev / xstage_ev mark
    // the end of the last apply that read each buffer.
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copy_done = nullptr, x_ev = nullptr, xstage_ev = nullptr;
    bool staged = false;
    // tensor-core correlator (correlator_variant 4): template groups of Gp
    // slots, K padded to Kp, tiles of 1024 lags per group
    bool tc = false;
    int tc_Kp = 0, tc_Gp = 0, tc_groups = 0, tc_tiles = 0, tc_cols = 0, n_sm = 0;
    long ldx = 0, ldr = 0;
    int dead_chunks = 1;
    // device buffers
    DevBuf x, rho, Bc, tw, grp_chan, grp_tb, grp_te, tids, tlen_d, nvalid_d, dead, err, tmpl_d, toff_d, pmin, pmax,
        chan_list, stackbuf, shifts_d, weights_d, specbuf, den, xstage, xrange, tc_B, tc_bscale, tc_grp_chan,
        tc_grp_tid;
    long ldd = 0;
    int nden = 0;
    PeakWS pk;
    std::vector<long long> pk_off;
    bool have_peaks = false;
    // candidates gathered by the correlator (mfgpu_mf_set_peak_threshold)
    double pk_req = -1;         // requested threshold, < 0: off
    bool pk_fused = false;      // slots hold the current apply's candidates
    double pk_fused_thr = 0;
    int pk_fused_len = 0;
    DevBuf pk_cnt, pk_idx, pk_val;
    DevBuf pk_flags;   // tensor-core correlator: candidate flags per 64 lags
    int pk_words = 0;
    // FP32 accuracy safeguards (kernels_fix.cuh): per-run window statistics
    // (rstat, row stride ldrs), per-chunk statistics (cst, row stride ldc,
    // nchunks valid), run flags, the tensor-core strips' operand offsets, the
    // fix-up batches (channel, templates, coefficient offsets and lengths,
    // coefficients, coefficient sums) and the candidate slots to recount
    bool fx_on = false;
    int fx_L = 0, fx_nden = 0, fx_nruns = 0, fx_nbatch = 0;
    long ldrs = 0, ldc = 0, fx_nchunks = 0;
    DevBuf rstat, cst, fxbits, fxlist, fxcount, tc_off, fx_btid, fx_boff, fx_bL, fx_bco, fx_bsum, pk_dirty,
        fx_cb0, fx_cnb;
    int fx_nbmax = 0, fx_lmax = 0;
    // templates longer than any FFT plan takes: correlated directly (batches
    // dir_b0 .. dir_b0 + dir_nb - 1 of the fix-up tables)
    int n_direct = 0, dir_b0 = 0, dir_nb = 0, dir_lmax = 0;
    int fLen = 0;  // longest template of the FFT plans (their shared length when all are equal)
    int fMin = 0;  // shortest template of the FFT plans
    // lags backed by data for the FFT plans' shortest template (device int
    // read by the error-bound kernels), smaller while a request window
    // shorter than the signal is loaded (win_active)
    DevBuf dlags;
    bool win_active = false;
    DevBuf fx_bch;
    DevBuf tws;  // pass twiddles in the split layout (correlator mode 4)
    DevBuf tickets;  // one persistent-launch ticket per correlator launch of an apply
    // length buckets beside the primary plan (longest templates); per
    // template its bucket's block length and block count, and the slot row
    // stride of the gathered candidates (the largest block count)
    std::vector<std::unique_ptr<MfBucket>> xb;
    // single-channel detector: reduced trace and argmax (or transformed
    // traces), detection rows and results
    DevBuf det_buf, det_id, det_rows, det_out, tchan_d;
    std::vector<mfgpu_detection> dets;
    // apply replayed as a CUDA graph (mfgpu_mf_set_graph): one executable
    // per input buffer and peak-gathering setup; captured on the second
    // apply with the same setup (the first sizes every buffer)
    struct ApplyGraph
    {
        cudaGraphExec_t exec = nullptr;
        const void *x = nullptr, *pk_cnt = nullptr, *pk_flags = nullptr;
        double pk_req = -2;
        bool pk_fused = false;
        double pk_fused_thr = 0;
        int pk_fused_len = 0, pk_words = 0;
        long long launches = 0;
        bool same(const ApplyGraph &o) const
        {
            return x == o.x && pk_cnt == o.pk_cnt && pk_flags == o.pk_flags && pk_req == o.pk_req;
        }
    };
    bool use_graph = false;
    ApplyGraph graphs[2];
    int graph_next = 0;
    ApplyGraph last_direct[2];  // setups of the last direct applies (one per input buffer)
    int direct_next = 0;
    long long graph_launches = 0;  // replays of captured applies
    void drop_graphs()
    {
        for (ApplyGraph &g : graphs)
        {
            if (g.exec) cudaGraphExecDestroy(g.exec);
            g = ApplyGraph();
        }
        last_direct[0] = last_direct[1] = ApplyGraph();
    }
    int ntemplates0 = 0;
    DevBuf row_S, row_nblk;
    int pk_stride = 0;
    long long launches = 0;
    float last_xcorr_ms = 0, last_apply_ms = 0;
    bool test_wait_timeout = false;  // mfgpu_mf_test_wait_timeout: the next apply only
    int dev_smem = 0;                // opt-in shared memory per block of the device
    bool persistent = false;         // FFT correlator as a persistent work-queue launch (option)
    bool tc_bf16 = false;            // tensor-core operands split into BF16 instead of FP16 (option)
    float tc_maxb = 0.f;             // largest coefficient of the unit-norm templates (tensor-core path)
    bool test_skip_fixup = false;    // mfgpu_mf_test_skip_fixup: flag runs but do not recompute them

    size_t esz() const { return (size_t) prec; }
    template <class F> void each_buf(F &&f)
    {
        DevBuf *all[] = {&x,      &rho,      &Bc,   &tw,  &grp_chan, &grp_tb, &grp_te, &tids,      &tlen_d,
                         &nvalid_d, &dead,   &err,  &tmpl_d, &toff_d, &pmin, &pmax,  &chan_list, &stackbuf,
                         &shifts_d, &weights_d, &specbuf, &den, &pk_cnt, &pk_idx, &pk_val, &xstage,
                         &xrange,   &tc_B,   &tc_bscale, &tc_grp_chan, &tc_grp_tid, &pk_flags,
                         &rstat,    &cst,    &fxbits, &fxlist, &fxcount, &tc_off, &fx_btid, &fx_boff,
                         &fx_bL,    &fx_cb0, &fx_cnb, &fx_bch, &dlags,
                         &fx_bco,   &fx_bsum, &pk_dirty, &tws, &tickets};
        for (DevBuf *d : all) f(*d);
        pk.each_buf(f);
        f(row_S);
        f(row_nblk);
        f(det_buf);
        f(det_id);
        f(det_rows);
        f(det_out);
        f(tchan_d);
        for (auto &b : xb) b->each_buf(f);
    }
    void release_device()
    {
        each_buf([](DevBuf &d) { d.release(); });
        pk.release();
    }
    size_t device_bytes()
    {
        size_t b = 0;
        each_buf([&](DevBuf &d) { b += d.bytes; });
        return b;
    }
    void reset()
    {
        drop_graphs();
        if (copy_stream) cudaStreamSynchronize(copy_stream);
        if (stream) cudaStreamSynchronize(stream);
        staged = false;
        release_device();
        initialized = have = timed = have_peaks = pk_fused = false;
        pk_req = -1;
        nt = n = maxLen = minLen = nch = 0;
        xb.clear();
        dets.clear();
        ntemplates0 = pk_stride = 0;
        lens.clear(); tchan.clear(); nvalid.clear(); tmpl.clear(); toff.clear();
        shifts.clear(); weights.clear(); pk_off.clear();
        can_stack = false;
        nfft = log2p = S = nblocks = ngroups = maxvalid = 0;
        ldx = ldr = 0;
        fx_on = false;
        fx_L = fx_nden = fx_nruns = fx_nbatch = 0;
        fx_nbmax = fx_lmax = n_direct = dir_b0 = dir_nb = dir_lmax = fLen = fMin = 0;
        win_active = false;
        ldrs = ldc = fx_nchunks = 0;
    }
};

// Waits for the object's compute stream (and, with `copies`, for a staged
// upload in flight).  Results on the device never depend on the staged
// copy, which only feeds the next apply (that apply waits for it on the
// device), so reading results does not wait for the next step's upload.
static mfgpu_status mf_sync(mfgpu_mf *mf, bool copies = false)
{
    if (copies && mf->copy_stream) CU(cudaStreamSynchronize(mf->copy_stream));
    CU(cudaStreamSynchronize(mf->stream));
    if (mf->initialized && mf->err.p)
    {
        int e = 0;
        CU(cudaMemcpy(&e, mf->err.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (e != 0)
        {
            CU(cudaMemset(mf->err.p, 0, sizeof(int)));
            mf->have = false;
            return fail(e == KERR_TMA_TIMEOUT ? MFGPU_ETIMEOUT : MFGPU_ECUDA,
                        "device kernel reported error code " + std::to_string(e));
        }
    }
    if (mf->timed)
    {
        if (cudaEventElapsedTime(&mf->last_xcorr_ms, mf->ev[1], mf->ev[2]) != cudaSuccess ||
            cudaEventElapsedTime(&mf->last_apply_ms, mf->ev[0], mf->ev[3]) != cudaSuccess)
        {
            (void) cudaGetLastError();  // timings unavailable: not an error of the work
            mf->last_xcorr_ms = mf->last_apply_ms = 0.f;
        }
        mf->timed = false;
    }
    return MFGPU_OK;
}


const char *mfgpu_last_error(void) { return g_err.c_str(); }

int mfgpu_version(void) { return 100; }

mfgpu_status mfgpu_device_count(int *count)
try
{
    if (!count) return fail(MFGPU_EINVAL, "count is NULL");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) n = 0;
    *count = n;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_fft_sizes(int nb, int nx, int *fft_length, int *block_length)
try
{
    if (!fft_length || !block_length) return fail(MFGPU_EINVAL, "output is NULL");
    return fft_sizes(nb, nx, fft_length, block_length);
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_window_length(int nb, int nx, int *fft_length, int *block_length)
try
{
    if (!fft_length || !block_length) return fail(MFGPU_EINVAL, "output is NULL");
    return window_length(nb, nx, fft_length, block_length);
}
catch (...)
{
    return mfgpu::status_of_exception();
}

// ---------------------------------------------------------------------------
mfgpu_status mfgpu_mf_create(int precision, mfgpu_mf **out)
try
{
    if (!out) return fail(MFGPU_EINVAL, "mf is NULL");
    if (precision != MFGPU_FLOAT32 && precision != MFGPU_FLOAT64)
        return fail(MFGPU_EINVAL, "precision must be MFGPU_FLOAT32 or MFGPU_FLOAT64");
    auto *mf = new mfgpu_mf();
    mf->prec = precision;
    cudaError_t e = cudaGetDevice(&mf->dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&mf->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&mf->copy_stream, cudaStreamNonBlocking);
    for (int i = 0; i < 4 && e == cudaSuccess; ++i) e = cudaEventCreate(&mf->ev[i]);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&mf->copy_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&mf->x_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&mf->xstage_ev, cudaEventDisableTiming);
    if (e != cudaSuccess)
    {
        delete mf;
        return cuda_fail(e, "mfgpu_mf_create");
    }
    *out = mf;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_destroy(mfgpu_mf *mf)
try
{
    if (!mf) return MFGPU_OK;
    {
        DeviceGuard g(mf->dev);
        mf->reset();
        for (auto &e : mf->ev)
            if (e) cudaEventDestroy(e);
        for (cudaEvent_t e : {mf->copy_done, mf->x_ev, mf->xstage_ev})
            if (e) cudaEventDestroy(e);
        if (mf->copy_stream) cudaStreamDestroy(mf->copy_stream);
        if (mf->stream) cudaStreamDestroy(mf->stream);
    }
    delete mf;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_clear(mfgpu_mf *mf)
try
{
    if (!mf) return fail(MFGPU_EINVAL, "mf is NULL");
    DeviceGuard g(mf->dev);
    mf->reset();
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

// twiddles and resident template spectra of one plan (every template's
// spectrum at the plan's FFT length; the plan reads its bucket's rows)
template <class T>
static mfgpu_status mf_upload_tables(mfgpu_mf *mf, int log2p, DevBuf &twb, DevBuf &Bc, DevBuf *tws = nullptr)
{
    std::vector<cx<T>> tw;
    twiddle_table<T>(log2p, tw);
    CU(twb.ensure(sizeof(cx<T>) * tw.size()));
    CU(cudaMemcpyAsync(twb.p, tw.data(), sizeof(cx<T>) * tw.size(), cudaMemcpyHostToDevice, mf->stream));
    if (tws)
    {
        // mode 4 copies the pass twiddles in the split layout
        std::vector<cx<T>> ts;
        twiddle_split<T>(log2p, ts);
        CU(tws->ensure(sizeof(cx<T>) * ts.size()));
        CU(cudaMemcpyAsync(tws->p, ts.data(), sizeof(cx<T>) * ts.size(), cudaMemcpyHostToDevice, mf->stream));
    }
    CU(Bc.ensure(sizeof(cx<T>) * (size_t) mf->nt * ((1L << log2p) + 2)));
    SpecParams<T> sp;
    sp.tmpl = mf->tmpl_d.as<double>();
    sp.toff = mf->toff_d.as<long>();
    sp.tlen = mf->tlen_d.as<int>();
    sp.Bc = Bc.as<cx<T>>();
    sp.ldb = (1L << log2p) + 2;
    sp.twt = twb.as<cx<T>>();
    CU(launch_spectra<T>(log2p, sp, mf->nt, mf->stream));
    ++mf->launches;
    return MFGPU_OK;
}

template <class T> static int plan_limit_lo() { return fft_limits<T>::lo; }
template <class T> static int plan_limit_hi() { return fft_limits<T>::hi; }

mfgpu_status mfgpu_mf_initialize(mfgpu_mf *mf, const mfgpu_mf_params *p)
try
{
    if (!mf) return fail(MFGPU_EINVAL, "mf is NULL");
    DeviceGuard g(mf->dev);
    mf->reset();
    if (!p) return fail(MFGPU_EINVAL, "Parameters are invalid: NULL");
    if (p->n_templates < 1) return fail(MFGPU_EINVAL, "Parameters are invalid: no templates");
    if (p->signal_size < 1) return fail(MFGPU_EINVAL, "Parameters are invalid: signal size not set");
    if (!p->template_lengths || !p->templates) return fail(MFGPU_EINVAL, "Parameters are invalid: templates NULL");
    if (p->detection_mode != MFGPU_SINGLE_CHANNEL && p->detection_mode != MFGPU_MULTI_CHANNEL)
        return fail(MFGPU_EINVAL, "invalid detection mode");
    const int nt = p->n_templates, n = p->signal_size;
    int maxLen = 0, minLen = std::numeric_limits<int>::max();
    for (int t = 0; t < nt; ++t)
    {
        if (p->template_lengths[t] < 1 || !p->templates[t])
            return fail(MFGPU_EINVAL, "template " + std::to_string(t) + " has no signal");
        maxLen = std::max(maxLen, p->template_lengths[t]);
        minLen = std::min(minLen, p->template_lengths[t]);
    }
    // MatchedFilter::initialize sizes the reference's FFT from (maxLen, n+maxLen-1)
    // and throws when the signal is not longer than that (src/matchedFilter.cpp:522-525).
    int rn = 0, rl = 0;
    mfgpu_status st = fft_sizes(maxLen, n + maxLen - 1, &rn, &rl);
    if (st != MFGPU_OK) return st;

    int nch;
    std::vector<int> tchan(nt);
    bool ref_layout = p->n_channels <= 0;
    if (ref_layout)
    {
        nch = p->detection_mode == MFGPU_MULTI_CHANNEL ? nt : 1;
        for (int t = 0; t < nt; ++t) tchan[t] = p->detection_mode == MFGPU_MULTI_CHANNEL ? t : 0;
    }
    else
    {
        if (!p->template_channel) return fail(MFGPU_EINVAL, "template_channel is NULL");
        nch = p->n_channels;
        for (int t = 0; t < nt; ++t)
        {
            if (p->template_channel[t] < 0 || p->template_channel[t] >= nch)
                return fail(MFGPU_EINVAL, "template_channel[" + std::to_string(t) + "] out of range");
            tchan[t] = p->template_channel[t];
        }
    }
    if (nch > 65535 * 64) return fail(MFGPU_EINVAL, "too many channels");

    mf->mode = p->detection_mode;
    mf->nt = nt; mf->n = n; mf->maxLen = maxLen; mf->minLen = minLen; mf->nch = nch;
    mf->ref_layout = ref_layout;
    mf->tchan = tchan;
    mf->lens.assign(p->template_lengths, p->template_lengths + nt);
    mf->nvalid.resize(nt);
    int maxvalid = 0;
    for (int t = 0; t < nt; ++t)
    {
        mf->nvalid[t] = std::max(0, n - mf->lens[t] + 1);
        maxvalid = std::max(maxvalid, mf->nvalid[t]);
    }
    mf->maxvalid = maxvalid;
    mf->toff.resize(nt);
    long tot = 0;
    for (int t = 0; t < nt; ++t) { mf->toff[t] = tot; tot += mf->lens[t]; }
    mf->tmpl.resize(tot);
    for (int t = 0; t < nt; ++t)
        std::memcpy(&mf->tmpl[mf->toff[t]], p->templates[t], sizeof(double) * mf->lens[t]);
    mf->stack_abs = p->stack_absolute_values ? 1 : 0;
    if (p->stack_shifts && p->stack_weights)
    {
        mf->can_stack = true;
        mf->shifts.assign(p->stack_shifts, p->stack_shifts + nt);
        mf->weights.assign(p->stack_weights, p->stack_weights + nt);
    }

    // Templates longer than the longest FFT plan takes (S >= 32 lags per
    // block: N - 31 samples) are correlated directly in the time domain
    // (fixup_kernel in direct mode); the FFT plan below covers the others.
    const int lcap = (2 << (mf->prec == 4 ? plan_limit_hi<float>() : plan_limit_hi<double>())) - 31;
    std::vector<char> is_direct(nt, 0);
    int ndirect = 0, fMax = 0, fMin = std::numeric_limits<int>::max();
    for (int t = 0; t < nt; ++t)
    {
        if (mf->lens[t] > lcap)
        {
            is_direct[t] = 1;
            ++ndirect;
        }
        else
        {
            fMax = std::max(fMax, mf->lens[t]);
            fMin = std::min(fMin, mf->lens[t]);
        }
    }
    const int ntf = nt - ndirect;
    mf->n_direct = ndirect;
    mf->fLen = ntf > 0 ? fMax : 0;
    mf->fMin = ntf > 0 ? fMin : 0;
    mf->persistent = p->persistent != 0;
    mf->tc_bf16 = p->tc_bf16 != 0;
    if (ndirect > 0)
    {
        if (p->correlator_variant == 4)
            return fail(MFGPU_EINVAL, "correlator_variant 4 (tensor cores) takes templates of at most " +
                                          std::to_string(lcap) + " samples");
        int dev_smem0 = 0;
        CU(cudaDeviceGetAttribute(&dev_smem0, cudaDevAttrMaxSharedMemoryPerBlockOptin, mf->dev));
        if ((mf->prec == 4 ? fixup_warps<float>(maxLen, dev_smem0) : fixup_warps<double>(maxLen, dev_smem0)) < 1)
            return fail(MFGPU_EINVAL, "template length " + std::to_string(maxLen) +
                                          " exceeds the supported maximum of the direct correlator");
    }
    // the FFT plan sees its own templates only
    maxLen = ntf > 0 ? fMax : 0;
    minLen = ntf > 0 ? fMin : 0;
    const int maxvalid_f = ntf > 0 ? n - fMin + 1 : 0;

    // ---- plan: FFT length (autotuned unless given), lags per block, groups
    std::vector<int> per_chan(nch, 0);
    for (int t = 0; t < nt; ++t)
        if (!is_direct[t]) per_chan[tchan[t]]++;
    int used_ch = 0, max_tpc = 0;
    for (int c = 0; c < nch; ++c) if (per_chan[c]) { ++used_ch; max_tpc = std::max(max_tpc, per_chan[c]); }
    const double tpc = (double) nt / std::max(1, used_ch);
    const int lo = mf->prec == 4 ? plan_limit_lo<float>() : plan_limit_lo<double>();
    const int hi = mf->prec == 4 ? plan_limit_hi<float>() : plan_limit_hi<double>();
    bool all_equal = ntf > 0 && minLen == maxLen;
    mf->shared_den = all_equal;
    // mode 3 normalises inside the CTA: no per-channel rows
    auto smem_of = [&](int l2p, int mode, int S) {
        const bool sd = all_equal && mode != 3 && mode != 4;
        return mf->prec == 4 ? xcorr_smem_bytes<float>(l2p, sd, mode, S)
                             : xcorr_smem_bytes<double>(l2p, sd, mode, S);
    };
    // correlator_variant: 1..3 -> modes 0..2, 5 -> mode 3, 4 tensor cores
    const int v = p->correlator_variant;
    const int forced_mode = v >= 1 && v <= 3 ? v - 1 : v == 5 ? 3 : v == 6 ? 4 : -1;
    if (v < 0 || v > 6) return fail(MFGPU_EINVAL, "correlator_variant must be 0..6");
    if (v == 6 && (mf->prec != 4 || all_equal))
        return fail(MFGPU_EINVAL, "correlator_variant 6 (two 256-thread teams) needs FP32 data and templates of "
                                  "several lengths");
    if ((forced_mode == 2 || forced_mode == 3) && !all_equal)
        return fail(MFGPU_EINVAL, "correlator_variant " + std::to_string(v) + " (teams) needs templates of one length");
    mf->tc = p->correlator_variant == 4;
    if (mf->tc && (mf->prec != 4 || !all_equal))
        return fail(MFGPU_EINVAL, "correlator_variant 4 (tensor cores) needs FP32 data and templates of one length");
    // per-bucket overrides: FFT length and organisation (mode) of bucket b
    if (p->n_bucket_plans < 0) return fail(MFGPU_EINVAL, "n_bucket_plans must be >= 0");
    bool bucket_forced = false;
    for (int b = 0; b < p->n_bucket_plans; ++b)
    {
        const int F = p->bucket_fft_lengths ? p->bucket_fft_lengths[b] : 0;
        const int bv = p->bucket_variants ? p->bucket_variants[b] : 0;
        if (F < 0 || (F > 0 && (F & (F - 1)) != 0))
            return fail(MFGPU_EINVAL, "bucket_fft_lengths[" + std::to_string(b) + "] = " + std::to_string(F) +
                                          " is not 0 or a power of two");
        if (!(bv == 0 || bv == 1 || bv == 2 || ((bv == 3 || bv == 5) && all_equal) ||
              (bv == 6 && !all_equal && mf->prec == 4)))
            return fail(MFGPU_EINVAL, "bucket_variants[" + std::to_string(b) + "] = " + std::to_string(bv) +
                                          (all_equal ? " must be 0, 1, 2, 3 or 5" : " must be 0, 1 or 2 (several template lengths)"));
        bucket_forced = bucket_forced || F > 0 || bv > 0;
    }
    auto bucket_nfft = [&](int b) {
        return b < p->n_bucket_plans && p->bucket_fft_lengths ? p->bucket_fft_lengths[b] : 0;
    };
    auto bucket_mode = [&](int b) {
        const int bv = b < p->n_bucket_plans && p->bucket_variants ? p->bucket_variants[b] : 0;
        return bv == 0 ? -1 : bv == 5 ? 3 : bv == 6 ? 4 : bv - 1;
    };
    const bool tc_candidate = mf->tc || (p->correlator_variant == 0 && mf->prec == 4 && all_equal &&
                                         p->fft_length == 0 && !bucket_forced && ndirect == 0);
    int dev_smem = 0, sm_smem = 0;
    CU(cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, mf->dev));
    CU(cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, mf->dev));
    mf->dev_smem = dev_smem;
    // CTAs per SM for a given shared-memory size (the register budget caps
    // the FP32 kernels at 2 per SM for P <= 2048 and 1 above, FP64 at 1)
    auto occupancy = [&](int l2p, size_t bytes) {
        int cap = (mf->prec == 4 && l2p <= 11) ? 2 : 1;
        int occ = (int) (sm_smem / (bytes + 1024));
        return std::min(cap, occ);
    };
    // best plan for templates of lengths up to Lb, the longest trace mv lags:
    // FFT length, lags per block, organisation and the cost in seconds per
    // template of the whole trace
    struct PlanPick
    {
        int l2p = -1, S = 0, mode = 0;
        double cost = 0;
    };
    // f_nfft / f_mode: a bucket's plan override (0 / -1: automatic)
    auto plan_for = [&](int Lb, int mv, bool eq, int f_nfft = 0, int f_mode = -1) {
        PlanPick best;
        for (int l2p = lo; l2p <= hi; ++l2p)
        {
            int N = 2 << l2p;
            if (p->fft_length > 0 && p->fft_length != N) continue;
            if (f_nfft > 0 && f_nfft != N) continue;
            int S = ((N - Lb + 1) / 32) * 32;
            if (S < 32) continue;
            // organisation: forced, else two teams for a shared length when
            // they keep the occupancy (measured 16% faster than the whole-CTA
            // loop at N = 4096 and 5% at N = 2048, 2% slower at N = 8192),
            // else spectrum prefetch when it keeps the occupancy
            int mode;
            if (f_mode >= 0) mode = f_mode;
            else if (forced_mode >= 0) mode = forced_mode;
            else
            {
                size_t b0 = smem_of(l2p, 0, S), b1 = smem_of(l2p, 1, S);
                int occ0 = occupancy(l2p, b0), occ1 = (int) b1 <= dev_smem ? occupancy(l2p, b1) : 0;
                mode = (occ1 >= occ0 && occ1 > 0) ? 1 : 0;
                if (eq && l2p <= 11)
                {
                    size_t b2 = smem_of(l2p, 2, S);
                    int occ2 = (int) b2 <= dev_smem ? occupancy(l2p, b2) : 0;
                    if (occ2 >= std::max(occ0, occ1) && occ2 > 0) mode = 2;
                }
                // several lengths at N = 8192 (FP32): two 256-thread teams
                // when the block's two normalisation rows fit (measured 12 %
                // faster than the whole-CTA organisation on the 2,000-template
                // bank)
                if (!eq && mf->prec == 4 && l2p == 12 && (int) smem_of(l2p, 4, S) <= dev_smem) mode = 4;
            }
            if (mode == 4)
            {
                // two normalisation rows: the block may have to be shorter
                // than the longest that the FFT length allows
                if (l2p < 11) continue;
                while (S > 32 && (int) smem_of(l2p, 4, S) > dev_smem) S -= 32;
            }
            size_t bytes = smem_of(l2p, mode, S);
            if ((int) bytes > dev_smem) continue;
            // a 512-thread mode-4 CTA holds as many warps as two others
            int occ = mode == 4 ? 2 : occupancy(l2p, bytes);
            if (occ < 1) continue;
            // seconds per (template, block), measured on GB300.  One template
            // length (normalisation rows precomputed): 8.4 ns at P = 2048 (N =
            // 4096, two CTAs per SM), ratios 0.70 at N = 2048 and 2.86 at N =
            // 8192 (one CTA per SM).  Several lengths (normalisation inside the
            // CTA for each template): 18.8 ns at N = 4096 and 35.2 ns at N =
            // 8192 (2,000-template bank).  Shorter transforms scale as N log N.
            double rel, base;
            if (eq)
            {
                base = 8.4e-9;
                rel = l2p == 11 ? 1.0 : l2p == 12 ? 2.86 : 0.70 * std::ldexp(1.0, l2p - 10) * (l2p + 1) / 11.0;
                if (l2p <= 11 && occ < 2) rel *= 1.4;
            }
            else
            {
                base = 18.8e-9;
                rel = l2p == 12 ? 1.87 : std::ldexp(1.0, l2p - 11) * (l2p + 1) / 12.0;
                if (mode == 4) rel *= 0.88;
            }
            const double nb = std::ceil((double) std::max(1, mv) / S);
            const double cost = nb * rel * base;
            if (best.l2p < 0 || cost < best.cost) best = PlanPick{l2p, S, mode, cost};
        }
        return best;
    };
    // Length buckets for a mixed-length bank (automatic FFT length, whole-CTA
    // organisations): the templates sorted by length split into at most
    // length_buckets (default 3) contiguous buckets, each with its own plan,
    // minimising the summed plan cost plus, when the limit is automatic,
    // 20 us per extra launch.  Cut positions are taken from 64 quantiles of
    // the sorted lengths.
    std::vector<int> order(nt);
    for (int t = 0; t < nt; ++t) order[t] = t;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return mf->lens[a] < mf->lens[b]; });
    std::vector<int> cuts{0, ntf};
    const int maxb = p->length_buckets > 0 ? p->length_buckets : 3;
    if (p->length_buckets < 0) return fail(MFGPU_EINVAL, "length_buckets must be >= 0");
    if (!all_equal && p->fft_length == 0 && (forced_mode <= 1 || forced_mode == 4) && maxb > 1)
    {
        std::vector<int> pos{0};
        for (int q = 1; q < 64; ++q)
        {
            const int i = (int) ((long) q * ntf / 64);
            if (i > pos.back() && i < ntf && mf->lens[order[i]] != mf->lens[order[i - 1]]) pos.push_back(i);
        }
        pos.push_back(ntf);
        const int M = (int) pos.size();
        std::vector<double> bc((size_t) M * M, 1e300);
        for (int a = 0; a < M; ++a)
            for (int b = a + 1; b < M; ++b)
            {
                const int Lb = mf->lens[order[pos[b] - 1]], mv = n - mf->lens[order[pos[a]]] + 1;
                const PlanPick pk = plan_for(Lb, mv, false);
                if (pk.l2p >= 0) bc[(size_t) a * M + b] = pk.cost * (pos[b] - pos[a]);
            }
        // an explicit bucket limit splits wherever the plans get cheaper
        const double launch_cost = p->length_buckets == 0 ? 20e-6 : 0.0;
        // dp[k][b]: best cost of positions [0, b) in k buckets
        std::vector<std::vector<double>> dp(maxb + 1, std::vector<double>(M, 1e300));
        std::vector<std::vector<int>> from(maxb + 1, std::vector<int>(M, -1));
        dp[0][0] = 0;
        for (int k = 1; k <= maxb; ++k)
            for (int b = 1; b < M; ++b)
                for (int a = 0; a < b; ++a)
                {
                    const double c = dp[k - 1][a] + bc[(size_t) a * M + b] + (k > 1 ? launch_cost : 0.0);
                    if (c < dp[k][b]) { dp[k][b] = c; from[k][b] = a; }
                }
        int bk = 1;
        for (int k = 2; k <= maxb; ++k)
            if (dp[k][M - 1] < dp[bk][M - 1]) bk = k;
        // automatic: split only for a predicted saving above 15 % (on the
        // 2,000-template bank the model predicted 10 % for two buckets at N =
        // 8192 and GB300 measured 1 %; for three, 10 % and -4 %)
        if (p->length_buckets == 0 && dp[bk][M - 1] > 0.85 * dp[1][M - 1]) bk = 1;
        if (dp[bk][M - 1] < 1e299 && bk > 1)
        {
            cuts.assign(1, ntf);
            for (int k = bk, b = M - 1; k > 0; b = from[k][b], --k) cuts.push_back(pos[from[k][b]]);
            std::reverse(cuts.begin(), cuts.end());
        }
    }
    const int nbk = (int) cuts.size() - 1;  // bucket nbk - 1 (longest templates) is the primary plan
    std::vector<int> bucket_of(nt, nbk - 1);
    for (int b = 0; b < nbk; ++b)
        for (int i = cuts[b]; i < cuts[b + 1]; ++i) bucket_of[order[i]] = b;
    for (int t = 0; t < nt; ++t)
        if (is_direct[t]) bucket_of[t] = -1;  // in no FFT plan
    const int mv0 = ntf > 0 ? n - mf->lens[order[cuts[nbk - 1]]] + 1 : 0;
    const PlanPick best =
        plan_for(maxLen, nbk > 1 ? mv0 : maxvalid_f, all_equal, bucket_nfft(nbk - 1), bucket_mode(nbk - 1));
    if (best.l2p < 0 && (bucket_nfft(nbk - 1) > 0 || bucket_mode(nbk - 1) >= 0))
        return fail(MFGPU_EINVAL, "the plan override of bucket " + std::to_string(nbk - 1) + " does not fit");
    const int best_l2p = best.l2p, best_S = best.S, best_mode = best.mode;
    const double best_cost = best.cost;
    mf->mode_x = best_mode;
    if (best_mode == 3) mf->shared_den = false;
    // seconds per template-lag of the chosen FFT plan
    const double fft_cost_per_lag = best_l2p >= 0 ? best_cost / std::max(1, maxvalid_f) : 1e30;
    if (best_l2p < 0)
    {
        if (p->fft_length > 0)
            return fail(MFGPU_EINVAL, "fft_length " + std::to_string(p->fft_length) +
                                          " is not a supported power of two for templates of length " +
                                          std::to_string(maxLen));
        return fail(MFGPU_EINVAL, "template length " + std::to_string(maxLen) + " exceeds the supported maximum (" +
                                      std::to_string((2 << hi) - 31) + ")");
    }
    mf->log2p = best_l2p;
    mf->nfft = 2 << best_l2p;
    mf->S = best_S;
    mf->nblocks = ((nbk > 1 ? mv0 : maxvalid_f) + best_S - 1) / best_S;
    for (int b = 0; b + 1 < nbk; ++b)
    {
        const int Lb = mf->lens[order[cuts[b + 1] - 1]], mv = n - mf->lens[order[cuts[b]]] + 1;
        const PlanPick pk = plan_for(Lb, mv, false, bucket_nfft(b), bucket_mode(b));
        if (pk.l2p < 0) return fail(MFGPU_EINVAL, "the plan override of bucket " + std::to_string(b) + " does not fit");
        auto xb = std::make_unique<MfBucket>();
        xb->log2p = pk.l2p;
        xb->nfft = 2 << pk.l2p;
        xb->S = pk.S;
        xb->mode = pk.mode;
        xb->nblocks = (mv + pk.S - 1) / pk.S;
        xb->ntemplates = cuts[b + 1] - cuts[b];
        mf->xb.push_back(std::move(xb));
    }
    mf->ntemplates0 = cuts[nbk] - cuts[nbk - 1];
    mf->ldx = ((long) mf->nblocks * best_S + mf->nfft + 63) / 64 * 64;
    for (auto &xb : mf->xb) mf->ldx = std::max<long>(mf->ldx, ((long) xb->nblocks * xb->S + xb->nfft + 63) / 64 * 64);
    mf->ldx = std::max<long>(mf->ldx, (n + 63) / 64 * 64);
    mf->ldr = ((long) std::max(1, maxvalid) + 63) / 64 * 64;
    if (all_equal)
    {
        // per-channel normalisation rows read by the correlator (S lags per
        // block) and written by den_kernel (den_lags_per_cta lags per CTA,
        // reading 32 * den_tail_runs samples past them)
        const long lpc = den_lags_per_cta(maxLen);
        mf->nden = (int) ((std::max(1, maxvalid) + lpc - 1) / lpc);
        mf->ldd = (std::max<long>((long) mf->nblocks * best_S + 32, (long) mf->nden * lpc) + 63) / 64 * 64;
        mf->ldx = std::max<long>(mf->ldx, ((long) mf->nden * lpc + 32L * den_tail_runs(maxLen) + 63) / 64 * 64);
    }
    std::vector<std::vector<int>> chan_t(nch);
    for (int t = 0; t < nt; ++t) chan_t[tchan[t]].push_back(t);
    std::vector<int> tc_gch, tc_gtid;
    if (tc_candidate)
    {
        // Hankel GEMM plan: K = L + 7 (8 phases) padded to 16; as many
        // templates per group (even, at most 16: the wide MMA has N = 16 per
        // template, at most 256) as fit the shared memory beside the strips
        const int Kp = (maxLen + 7 + 15) / 16 * 16;
        const long room = (long) dev_smem - (long) tc_smem_bytes(Kp, 0);
        const int gmax = (int) std::min<long>(16, room / (32L * Kp)) & ~1;
        if (gmax < 2 && mf->tc)
            return fail(MFGPU_EINVAL, "template length " + std::to_string(maxLen) +
                                          " is too long for the tensor-core correlator");
        if (p->tc_group != 0 && (p->tc_group < 2 || p->tc_group > gmax || (p->tc_group & 1)))
            return fail(MFGPU_EINVAL, "tc_group = " + std::to_string(p->tc_group) +
                                          " must be even and in [2, " + std::to_string(std::max(2, gmax)) +
                                          "] for templates of " + std::to_string(maxLen) + " samples");
        // balanced groups: the busiest channel splits into ngc equal groups
        const int ngc = gmax >= 2 ? (max_tpc + gmax - 1) / gmax : 1;
        const int Gp = p->tc_group ? p->tc_group
                                   : gmax >= 2 ? std::min(gmax, ((max_tpc + ngc - 1) / ngc + 1) & ~1) : 2;
        // automatic choice: seconds per template-lag measured on GB300 (two
        // MMAs per K step), about 3.6e-15 per padded template sample plus
        // 5.7e-12 per tile row shared by the Gp templates of a group, against
        // the FFT plan's estimate
        if (!mf->tc && gmax >= 2)
            mf->tc = 3.6e-15 * Kp + 5.7e-12 / Gp < 0.9 * fft_cost_per_lag;
    }
    if (mf->tc)
    {
        const int Kp = (maxLen + 7 + 15) / 16 * 16;
        const long room = (long) dev_smem - (long) tc_smem_bytes(Kp, 0);
        const int gmax = (int) std::min<long>(16, room / (32L * Kp)) & ~1;
        const int ngc = (max_tpc + gmax - 1) / gmax;
        const int Gp = p->tc_group ? p->tc_group : std::min(gmax, ((max_tpc + ngc - 1) / ngc + 1) & ~1);
        for (int c = 0; c < nch; ++c)
            for (size_t i = 0; i < chan_t[c].size(); i += Gp)
            {
                tc_gch.push_back(c);
                for (int k = 0; k < Gp; ++k)
                    tc_gtid.push_back(i + k < chan_t[c].size() ? chan_t[c][i + k] : -1);
            }
        mf->tc_Kp = Kp;
        // largest coefficient of the demeaned unit-norm templates (the BF16
        // split's error bound scales with it)
        mf->tc_maxb = 0.f;
        for (int t = 0; t < nt; ++t)
        {
            const double *b = &mf->tmpl[mf->toff[t]];
            const int L = mf->lens[t];
            double m = 0, q = 0, mx = 0;
            for (int i = 0; i < L; ++i) m += b[i];
            m /= L;
            for (int i = 0; i < L; ++i) q += (b[i] - m) * (b[i] - m);
            for (int i = 0; i < L; ++i) mx = std::max(mx, std::fabs(b[i] - m));
            if (q > 0) mf->tc_maxb = std::max(mf->tc_maxb, (float) (mx / std::sqrt(q)));
        }
        mf->tc_Gp = Gp;
        mf->tc_groups = (int) tc_gch.size();
        mf->tc_tiles = (std::max(1, maxvalid) + kTcLags - 1) / kTcLags;
        int cols = 32;  // two accumulators of 16 Gp columns each
        while (cols < 32 * Gp) cols *= 2;
        mf->tc_cols = cols;
        CU(cudaDeviceGetAttribute(&mf->n_sm, cudaDevAttrMultiProcessorCount, mf->dev));
        // strips read tiles * 1024 + Kp samples; the normalisation row covers every tile
        const long tl = (long) mf->tc_tiles * kTcLags;
        const long lpc = den_lags_per_cta(maxLen);
        mf->nden = (int) ((std::max<long>(tl, maxvalid) + lpc - 1) / lpc);
        mf->ldd = (std::max<long>(mf->ldd, std::max<long>(tl, (long) mf->nden * lpc)) + 63) / 64 * 64;
        mf->ldx = std::max<long>(mf->ldx, (tl + Kp + 63) / 64 * 64);
        mf->ldx = std::max<long>(mf->ldx, ((long) mf->nden * lpc + 32L * den_tail_runs(maxLen) + 63) / 64 * 64);
    }
    if (mf->tc) mf->shared_den = true;  // the tensor-core epilogue reads den_kernel's rows
    if (ndirect > 0)
    {
        // the direct correlator stages L + 31 samples from the start of every run
        mf->fx_nruns = (std::max(1, maxvalid) + 31) / 32;
        mf->ldx = std::max<long>(mf->ldx, ((long) mf->fx_nruns * 32 + mf->maxLen + 32 + 63) / 64 * 64);
    }
    if (mf->prec == 4 && ntf > 0)
    {
        // accuracy safeguards: window statistics of the shared length (the
        // normalisation rows come from the same launch) or, for several
        // lengths, of the shortest one (a longer window starting at the same
        // lag contains it, so its variance is no smaller: the bound stays
        // conservative for every template)
        mf->fx_on = true;
        mf->fx_L = mf->shared_den ? maxLen : minLen;
        const long lpc = den_lags_per_cta(mf->fx_L);
        mf->fx_nruns = (std::max(1, maxvalid) + 31) / 32;
        long cover = (long) mf->fx_nruns * 32;
        if (mf->tc) cover = std::max<long>(cover, (long) mf->tc_tiles * kTcLags);
        mf->fx_nden = mf->shared_den ? mf->nden : (int) ((cover + lpc - 1) / lpc);
        if (mf->shared_den) mf->fx_nden = std::max<int>(mf->nden, (int) ((cover + lpc - 1) / lpc));
        mf->ldrs = ((long) mf->fx_nden * lpc / 32 + 63) / 64 * 64;
        mf->fx_nchunks = (long) mf->fx_nden * lpc / 32 + den_tail_runs(mf->fx_L) + 1;
        mf->ldc = (mf->fx_nchunks + 63) / 64 * 64;
        mf->ldx = std::max<long>(mf->ldx, ((long) mf->fx_nden * lpc + 32L * den_tail_runs(mf->fx_L) + 63) / 64 * 64);
        // the fix-up stages L + 31 samples from the start of every run
        mf->ldx = std::max<long>(mf->ldx, ((long) mf->fx_nruns * 32 + maxLen + 32 + 63) / 64 * 64);
        if (mf->shared_den)
        {
            mf->nden = mf->fx_nden;
            mf->ldd = std::max<long>(mf->ldd, ((long) mf->nden * lpc + 63) / 64 * 64);
        }
    }
    // work groups of one plan: each channel's templates of the bucket, split
    // so the grid has enough CTAs
    struct Groups
    {
        std::vector<int> gch, gtb, gte, tids;
    };
    auto make_groups = [&](int bucket, int nblocks, Groups &gr) {
        std::vector<int> pc(nch, 0);
        int mx = 0;
        for (int t = 0; t < nt; ++t)
            if (bucket_of[t] == bucket) mx = std::max(mx, ++pc[tchan[t]]);
        int G = std::max(1, mx);
        auto count_groups = [&](int gsz) {
            long ng = 0;
            for (int c = 0; c < nch; ++c) ng += (pc[c] + gsz - 1) / gsz;
            return ng;
        };
        while (G > 1 && ((long) nblocks * count_groups(G) < 4L * 152 * 2 || count_groups(G) > 65535)) G = (G + 1) / 2;
        if (count_groups(G) > 65535) return false;
        for (int c = 0; c < nch; ++c)
        {
            std::vector<int> mine;
            for (int t : chan_t[c])
                if (bucket_of[t] == bucket) mine.push_back(t);
            for (size_t i = 0; i < mine.size(); i += G)
            {
                gr.gch.push_back(c);
                gr.gtb.push_back((int) gr.tids.size());
                for (size_t j = i; j < std::min(mine.size(), i + (size_t) G); ++j) gr.tids.push_back(mine[j]);
                gr.gte.push_back((int) gr.tids.size());
            }
        }
        return true;
    };
    Groups g0;
    std::vector<Groups> gx(mf->xb.size());
    if (!make_groups(nbk - 1, mf->nblocks, g0)) return fail(MFGPU_EINVAL, "too many template groups");
    for (size_t b = 0; b < mf->xb.size(); ++b)
    {
        if (!make_groups((int) b, mf->xb[b]->nblocks, gx[b])) return fail(MFGPU_EINVAL, "too many template groups");
        mf->xb[b]->ngroups = (int) gx[b].gch.size();
    }
    const std::vector<int> &gch = g0.gch, &gtb = g0.gtb, &gte = g0.gte, &tids = g0.tids;
    mf->ngroups = (int) gch.size();
    mf->dead_chunks = (int) std::min<long>(1024, std::max<long>(1, (n + 16383) / 16384));

    // ---- device memory
    const size_t es = mf->esz();
    CU(mf->x.ensure(es * (size_t) nch * mf->ldx));
    if (mf->shared_den) CU(mf->den.ensure(es * (size_t) nch * mf->ldd));
    CU(cudaMemsetAsync(mf->x.p, 0, mf->x.bytes, mf->stream));
    CU(mf->rho.ensure(es * (size_t) nt * mf->ldr));
    CU(cudaMemsetAsync(mf->rho.p, 0, mf->rho.bytes, mf->stream));
    CU(mf->grp_chan.ensure(sizeof(int) * gch.size()));
    CU(mf->grp_tb.ensure(sizeof(int) * gch.size()));
    CU(mf->grp_te.ensure(sizeof(int) * gch.size()));
    CU(mf->tids.ensure(sizeof(int) * tids.size()));
    CU(mf->tlen_d.ensure(sizeof(int) * nt));
    CU(mf->nvalid_d.ensure(sizeof(int) * nt));
    CU(mf->dead.ensure((size_t) nch));
    CU(cudaMemsetAsync(mf->dead.p, 0, mf->dead.bytes, mf->stream));
    CU(mf->err.ensure(sizeof(int)));
    CU(cudaMemsetAsync(mf->err.p, 0, sizeof(int), mf->stream));
    CU(mf->tmpl_d.ensure(sizeof(double) * (size_t) tot));
    CU(mf->toff_d.ensure(sizeof(long) * nt));
    CU(mf->pmin.ensure(es * (size_t) nch * mf->dead_chunks));
    CU(mf->pmax.ensure(es * (size_t) nch * mf->dead_chunks));
    CU(mf->chan_list.ensure(sizeof(int) * nch));
    std::vector<int> all_ch(nch);
    for (int c = 0; c < nch; ++c) all_ch[c] = c;
    CU(cudaMemcpyAsync(mf->chan_list.p, all_ch.data(), sizeof(int) * nch, cudaMemcpyHostToDevice, mf->stream));
    CU(cudaMemcpyAsync(mf->grp_chan.p, gch.data(), sizeof(int) * gch.size(), cudaMemcpyHostToDevice, mf->stream));
    CU(cudaMemcpyAsync(mf->grp_tb.p, gtb.data(), sizeof(int) * gtb.size(), cudaMemcpyHostToDevice, mf->stream));
    CU(cudaMemcpyAsync(mf->grp_te.p, gte.data(), sizeof(int) * gte.size(), cudaMemcpyHostToDevice, mf->stream));
    CU(cudaMemcpyAsync(mf->tids.p, tids.data(), sizeof(int) * tids.size(), cudaMemcpyHostToDevice, mf->stream));
    CU(cudaMemcpyAsync(mf->tlen_d.p, mf->lens.data(), sizeof(int) * nt, cudaMemcpyHostToDevice, mf->stream));
    CU(cudaMemcpyAsync(mf->nvalid_d.p, mf->nvalid.data(), sizeof(int) * nt, cudaMemcpyHostToDevice, mf->stream));
    CU(cudaMemcpyAsync(mf->tmpl_d.p, mf->tmpl.data(), sizeof(double) * tot, cudaMemcpyHostToDevice, mf->stream));
    CU(cudaMemcpyAsync(mf->toff_d.p, mf->toff.data(), sizeof(long) * nt, cudaMemcpyHostToDevice, mf->stream));
    CU(mf->tchan_d.ensure(sizeof(int) * nt));
    CU(cudaMemcpyAsync(mf->tchan_d.p, mf->tchan.data(), sizeof(int) * nt, cudaMemcpyHostToDevice, mf->stream));
    CU(mf->xrange.ensure(sizeof(float) * nch));
    CU(cudaMemsetAsync(mf->xrange.p, 0, sizeof(float) * nch, mf->stream));
    mfgpu_status s2 = mf->prec == 4 ? mf_upload_tables<float>(mf, mf->log2p, mf->tw, mf->Bc,
                                                              mf->mode_x == 4 ? &mf->tws : nullptr)
                                    : mf_upload_tables<double>(mf, mf->log2p, mf->tw, mf->Bc);
    if (s2 != MFGPU_OK) return s2;
    for (size_t b = 0; b < mf->xb.size(); ++b)
    {
        MfBucket &xb = *mf->xb[b];
        s2 = mf->prec == 4 ? mf_upload_tables<float>(mf, xb.log2p, xb.tw, xb.Bc, xb.mode == 4 ? &xb.tws : nullptr)
                           : mf_upload_tables<double>(mf, xb.log2p, xb.tw, xb.Bc);
        if (s2 != MFGPU_OK) return s2;
        const Groups &gr = gx[b];
        CU(xb.grp_chan.ensure(sizeof(int) * gr.gch.size()));
        CU(xb.grp_tb.ensure(sizeof(int) * gr.gch.size()));
        CU(xb.grp_te.ensure(sizeof(int) * gr.gch.size()));
        CU(xb.tids.ensure(sizeof(int) * std::max<size_t>(1, gr.tids.size())));
        CU(cudaMemcpyAsync(xb.grp_chan.p, gr.gch.data(), sizeof(int) * gr.gch.size(), cudaMemcpyHostToDevice,
                           mf->stream));
        CU(cudaMemcpyAsync(xb.grp_tb.p, gr.gtb.data(), sizeof(int) * gr.gtb.size(), cudaMemcpyHostToDevice,
                           mf->stream));
        CU(cudaMemcpyAsync(xb.grp_te.p, gr.gte.data(), sizeof(int) * gr.gte.size(), cudaMemcpyHostToDevice,
                           mf->stream));
        CU(cudaMemcpyAsync(xb.tids.p, gr.tids.data(), sizeof(int) * gr.tids.size(), cudaMemcpyHostToDevice,
                           mf->stream));
    }
    // block length and count of every template's plan; slot rows of the
    // gathered peak candidates span the largest count
    mf->pk_stride = mf->nblocks;
    for (auto &xb : mf->xb) mf->pk_stride = std::max(mf->pk_stride, xb->nblocks);
    if (!mf->xb.empty())
    {
        std::vector<int> rs(nt), rn(nt);
        for (int t = 0; t < nt; ++t)
        {
            const int b = bucket_of[t];  // -1: a direct template, slots laid out like the primary plan's
            rs[t] = b < 0 || b == nbk - 1 ? mf->S : mf->xb[b]->S;
            rn[t] = b < 0 || b == nbk - 1 ? mf->nblocks : mf->xb[b]->nblocks;
        }
        CU(mf->row_S.ensure(sizeof(int) * nt));
        CU(mf->row_nblk.ensure(sizeof(int) * nt));
        CU(cudaMemcpyAsync(mf->row_S.p, rs.data(), sizeof(int) * nt, cudaMemcpyHostToDevice, mf->stream));
        CU(cudaMemcpyAsync(mf->row_nblk.p, rn.data(), sizeof(int) * nt, cudaMemcpyHostToDevice, mf->stream));
        // the host vectors above must outlive the copies
        CU(cudaStreamSynchronize(mf->stream));
    }
    if (mf->tc)
    {
        const size_t slots = (size_t) mf->tc_groups * mf->tc_Gp;
        CU(mf->tc_grp_chan.ensure(sizeof(int) * tc_gch.size()));
        CU(mf->tc_grp_tid.ensure(sizeof(int) * slots));
        CU(mf->tc_bscale.ensure(sizeof(float) * slots));
        CU(mf->tc_B.ensure(sizeof(__half) * 16 * slots * mf->tc_Kp));
        CU(cudaMemcpyAsync(mf->tc_grp_chan.p, tc_gch.data(), sizeof(int) * tc_gch.size(), cudaMemcpyHostToDevice,
                           mf->stream));
        CU(cudaMemcpyAsync(mf->tc_grp_tid.p, tc_gtid.data(), sizeof(int) * slots, cudaMemcpyHostToDevice, mf->stream));
        CU(launch_tc_bank(mf->tmpl_d.as<double>(), mf->toff_d.as<long>(), mf->tlen_d.as<int>(),
                          mf->tc_grp_tid.as<int>(), mf->tc_groups, mf->tc_Gp, mf->tc_Kp, mf->tc_B.as<__half>(),
                          mf->tc_bscale.as<float>(), mf->tc_bf16, mf->stream));
        ++mf->launches;
    }
    if (mf->fx_on || ndirect > 0)
    {
        // Template batches, kFixBatch templates of one channel each,
        // coefficients interleaved [i][kFixBatch]: first every channel's FFT
        // templates sorted by length (the FP32 fix-up), then every channel's
        // direct templates (the time-domain correlator)
        std::vector<int> btid, bL, bch, cb0(nch, 0), cnb(nch, 0);
        std::vector<long> boff;
        long tot_co = 0;
        mf->fx_nbmax = 0;
        mf->fx_lmax = 0;
        mf->dir_lmax = 0;
        auto add_batches = [&](int c, bool direct) {
            std::vector<int> ts;
            for (int t : chan_t[c])
                if ((bool) is_direct[t] == direct) ts.push_back(t);
            std::stable_sort(ts.begin(), ts.end(), [&](int a, int b) { return mf->lens[a] < mf->lens[b]; });
            for (size_t i = 0; i < ts.size(); i += kFixBatch)
            {
                int lb = 0;
                for (int k = 0; k < kFixBatch; ++k)
                {
                    const int t = i + k < ts.size() ? ts[i + k] : -1;
                    btid.push_back(t);
                    if (t >= 0) lb = std::max(lb, mf->lens[t]);
                }
                bL.push_back(lb);
                bch.push_back(c);
                boff.push_back(tot_co);
                tot_co += (long) kFixBatch * lb;
                if (direct) mf->dir_lmax = std::max(mf->dir_lmax, lb);
                else mf->fx_lmax = std::max(mf->fx_lmax, lb);
            }
            return (int) ((ts.size() + kFixBatch - 1) / kFixBatch);
        };
        if (mf->fx_on)
            for (int c = 0; c < nch; ++c)
            {
                cb0[c] = (int) bL.size();
                cnb[c] = add_batches(c, false);
                mf->fx_nbmax = std::max(mf->fx_nbmax, cnb[c]);
            }
        mf->dir_b0 = (int) bL.size();
        for (int c = 0; c < nch && ndirect > 0; ++c) add_batches(c, true);
        mf->dir_nb = (int) bL.size() - mf->dir_b0;
        mf->fx_nbatch = (int) bL.size();
        if (mf->fx_on)
        {
            CU(mf->rstat.ensure(sizeof(float4) * (size_t) nch * mf->ldrs));
            CU(mf->cst.ensure(sizeof(float2) * (size_t) nch * mf->ldc));
            CU(mf->fxbits.ensure(sizeof(unsigned) * (size_t) nch * (mf->ldrs / 32)));
            CU(mf->fxlist.ensure(sizeof(int) * (size_t) nch * mf->ldrs));
            CU(mf->fxcount.ensure(sizeof(int)));
            CU(cudaMemsetAsync(mf->fxcount.p, 0, sizeof(int), mf->stream));
            CU(mf->dlags.ensure(sizeof(int)));
            CU(launch_set_int(mf->dlags.as<int>(), std::max(0, n - mf->fMin + 1), mf->stream));
            if (mf->tc) CU(mf->tc_off.ensure(sizeof(float) * (size_t) nch * mf->tc_tiles));
        }
        CU(mf->fx_btid.ensure(sizeof(int) * btid.size()));
        CU(mf->fx_boff.ensure(sizeof(long) * boff.size()));
        CU(mf->fx_bL.ensure(sizeof(int) * bL.size()));
        CU(mf->fx_bch.ensure(sizeof(int) * bch.size()));
        CU(mf->fx_bco.ensure(es * (size_t) std::max<long>(1, tot_co)));
        CU(mf->fx_bsum.ensure(es * nt));
        CU(mf->fx_cb0.ensure(sizeof(int) * nch));
        CU(mf->fx_cnb.ensure(sizeof(int) * nch));
        CU(cudaMemcpyAsync(mf->fx_cb0.p, cb0.data(), sizeof(int) * nch, cudaMemcpyHostToDevice, mf->stream));
        CU(cudaMemcpyAsync(mf->fx_cnb.p, cnb.data(), sizeof(int) * nch, cudaMemcpyHostToDevice, mf->stream));
        CU(cudaMemcpyAsync(mf->fx_btid.p, btid.data(), sizeof(int) * btid.size(), cudaMemcpyHostToDevice, mf->stream));
        CU(cudaMemcpyAsync(mf->fx_boff.p, boff.data(), sizeof(long) * boff.size(), cudaMemcpyHostToDevice, mf->stream));
        CU(cudaMemcpyAsync(mf->fx_bL.p, bL.data(), sizeof(int) * bL.size(), cudaMemcpyHostToDevice, mf->stream));
        CU(cudaMemcpyAsync(mf->fx_bch.p, bch.data(), sizeof(int) * bch.size(), cudaMemcpyHostToDevice, mf->stream));
        if (mf->prec == 4)
            CU(launch_fix_prep<float>(mf->tmpl_d.as<double>(), mf->toff_d.as<long>(), mf->tlen_d.as<int>(),
                                      mf->fx_btid.as<int>(), mf->fx_boff.as<long>(), mf->fx_bL.as<int>(), mf->fx_nbatch,
                                      mf->fx_bco.as<float>(), mf->fx_bsum.as<float>(), mf->stream));
        else
            CU(launch_fix_prep<double>(mf->tmpl_d.as<double>(), mf->toff_d.as<long>(), mf->tlen_d.as<int>(),
                                       mf->fx_btid.as<int>(), mf->fx_boff.as<long>(), mf->fx_bL.as<int>(),
                                       mf->fx_nbatch, mf->fx_bco.as<double>(), mf->fx_bsum.as<double>(), mf->stream));
        ++mf->launches;
        if (!mf->n_sm) CU(cudaDeviceGetAttribute(&mf->n_sm, cudaDevAttrMultiProcessorCount, mf->dev));
        // the host vectors above must outlive the copies
        CU(cudaStreamSynchronize(mf->stream));
    }
    CU(cudaStreamSynchronize(mf->stream));
    CU(cudaGetLastError());
    mf->initialized = true;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

#define MF_CHECK_INIT(mf)                                                                                          \
    do                                                                                                             \
    {                                                                                                              \
        if (!(mf)) return fail(MFGPU_EINVAL, "mf is NULL");                                                        \
        if (!(mf)->initialized) return fail(MFGPU_ESTATE, "Class not initialized");                                \
    } while (0)

mfgpu_status mfgpu_mf_is_initialized(const mfgpu_mf *mf, int *flag)
try
{
    if (!mf || !flag) return fail(MFGPU_EINVAL, "NULL argument");
    *flag = mf->initialized ? 1 : 0;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_number_of_templates(const mfgpu_mf *mf, int *n)
try
{
    MF_CHECK_INIT(mf);
    if (!n) return fail(MFGPU_EINVAL, "n is NULL");
    *n = mf->nt;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_signal_length(const mfgpu_mf *mf, int *n)
try
{
    MF_CHECK_INIT(mf);
    if (!n) return fail(MFGPU_EINVAL, "n is NULL");
    *n = mf->n;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_filtered_signal_length(const mfgpu_mf *mf, int *n)
try
{
    MF_CHECK_INIT(mf);
    if (!n) return fail(MFGPU_EINVAL, "n is NULL");
    *n = mf->n - mf->maxLen + 1;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_plan(const mfgpu_mf *mf, int *fft_length, int *lags_per_block, int *n_blocks)
try
{
    MF_CHECK_INIT(mf);
    if (fft_length) *fft_length = mf->nfft;
    if (lags_per_block) *lags_per_block = mf->S;
    if (n_blocks) *n_blocks = mf->nblocks;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_correlator(const mfgpu_mf *mf, int *variant, int *tc_group, int *tc_k)
try
{
    MF_CHECK_INIT(mf);
    if (variant) *variant = mf->tc ? 4 : mf->mode_x == 3 ? 5 : mf->mode_x == 4 ? 6 : mf->mode_x + 1;
    if (tc_group) *tc_group = mf->tc ? mf->tc_Gp : 0;
    if (tc_k) *tc_k = mf->tc ? mf->tc_Kp : 0;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_buckets(const mfgpu_mf *mf, int max, int *fft_lengths, int *n_templates, int *count)
try
{
    MF_CHECK_INIT(mf);
    const int nb = (int) mf->xb.size() + 1;
    if (count) *count = nb;
    for (int b = 0; b < nb && b < max; ++b)
    {
        const bool prim = b == nb - 1;
        if (fft_lengths) fft_lengths[b] = prim ? mf->nfft : mf->xb[b]->nfft;
        if (n_templates) n_templates[b] = prim ? mf->ntemplates0 : mf->xb[b]->ntemplates;
    }
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_bucket_plans(const mfgpu_mf *mf, int max, int *lags_per_block, int *variants, int *count)
try
{
    MF_CHECK_INIT(mf);
    const int nb = (int) mf->xb.size() + 1;
    if (count) *count = nb;
    auto variant_of = [](int mode) { return mode == 3 ? 5 : mode == 4 ? 6 : mode + 1; };
    for (int b = 0; b < nb && b < max; ++b)
    {
        const bool prim = b == nb - 1;
        if (lags_per_block) lags_per_block[b] = prim ? mf->S : mf->xb[b]->S;
        if (variants) variants[b] = prim ? (mf->tc ? 4 : variant_of(mf->mode_x)) : variant_of(mf->xb[b]->mode);
    }
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

// Records, in stream order, how many samples of every row carry data
// (ndata; the rest is zero tail): the error bounds list no run past the lags
// those samples back.  Cheap, and skipped while nothing changes.
static mfgpu_status mf_set_data_length(mfgpu_mf *mf, int ndata)
{
    if (!mf->fx_on) return MFGPU_OK;
    const bool window = ndata < mf->n;
    if (!window && !mf->win_active) return MFGPU_OK;
    CU(launch_set_int(mf->dlags.as<int>(), std::max(0, ndata - mf->fMin + 1), mf->stream));
    mf->win_active = window;
    return MFGPU_OK;
}

static mfgpu_status mf_channel_of(mfgpu_mf *mf, int it, int *c)
{
    if (it < 0 || it >= mf->nt)
        return fail(MFGPU_EINVAL, "it = " + std::to_string(it) + " must be in the range [0," +
                                      std::to_string(mf->nt - 1) + "]");
    if (mf->ref_layout && mf->mode == MFGPU_SINGLE_CHANNEL && it != 0)
        return fail(MFGPU_EINVAL, "single-channel mode has one signal: it must be 0");
    *c = mf->tchan[it];
    return MFGPU_OK;
}

// Makes staged signals current: the compute stream waits for the staged
// copy, the buffers swap and the dead-trace flags of every channel are
// recomputed.
static mfgpu_status mf_resolve_stage(mfgpu_mf *mf)
{
    if (!mf->staged) return MFGPU_OK;
    mf->staged = false;
    mf->have = false;
    mf->have_peaks = false;
    mf->pk_fused = false;
    CU(cudaStreamWaitEvent(mf->stream, mf->copy_done, 0));
    std::swap(mf->x, mf->xstage);
    std::swap(mf->x_ev, mf->xstage_ev);
    if (mf->prec == 4)
        CU(launch_dead<float>(mf->x.as<float>(), mf->ldx, mf->nch, mf->n, mf->dead.as<unsigned char>(),
                              mf->pmin.as<float>(), mf->pmax.as<float>(), mf->dead_chunks, mf->stream,
                              mf->xrange.as<float>()));
    else
        CU(launch_dead<double>(mf->x.as<double>(), mf->ldx, mf->nch, mf->n, mf->dead.as<unsigned char>(),
                               mf->pmin.as<double>(), mf->pmax.as<double>(), mf->dead_chunks, mf->stream));
    mf->launches += 2;
    return MFGPU_OK;
}

mfgpu_status mfgpu_mf_stage_channel_signals(mfgpu_mf *mf, int n, const void *x, long ld)
try
{
    MF_CHECK_INIT(mf);
    DeviceGuard g(mf->dev);
    if (n != mf->n)
        return fail(MFGPU_EINVAL, "Number of samples = " + std::to_string(n) + " must equal" + std::to_string(mf->n));
    if (!x) return fail(MFGPU_EINVAL, "x is NULL");
    if (mf->nch > 1 && ld < n) return fail(MFGPU_EINVAL, "row stride is smaller than the number of samples");
    const size_t es = mf->esz();
    const size_t need = es * (size_t) mf->nch * mf->ldx;  // both buffers hold at least this
    if (!mf->xstage.p || mf->xstage.bytes < need)
    {
        // a fresh staging buffer: no apply has read it; zero row tails like x
        CU(cudaStreamSynchronize(mf->copy_stream));
        CU(mf->xstage.ensure(need));
        CU(cudaMemsetAsync(mf->xstage.p, 0, mf->xstage.bytes, mf->copy_stream));
    }
    // full rows from the next apply on (after a shorter request window)
    mfgpu_status ds = mf_set_data_length(mf, mf->n);
    if (ds != MFGPU_OK) return ds;
    // the buffer is free once the last apply that read it has finished
    CU(cudaStreamWaitEvent(mf->copy_stream, mf->xstage_ev, 0));
    if (mf->nch == 1) CU(cudaMemcpyAsync(mf->xstage.p, x, es * (size_t) n, cudaMemcpyHostToDevice, mf->copy_stream));
    else
        CU(cudaMemcpy2DAsync(mf->xstage.p, es * (size_t) mf->ldx, x, es * (size_t) ld, es * (size_t) n,
                             (size_t) mf->nch, cudaMemcpyHostToDevice, mf->copy_stream));
    CU(cudaEventRecord(mf->copy_done, mf->copy_stream));
    mf->staged = true;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

// Copies nch channel rows (n samples each, source row stride ld samples)
// into channels [c0, c0 + nch) and recomputes their dead-trace flags.
static mfgpu_status mf_store_signals(mfgpu_mf *mf, int c0, int nch, int n, const void *x, long ld,
                                     cudaMemcpyKind kind)
{
    if (n != mf->n)
        return fail(MFGPU_EINVAL, "Number of samples = " + std::to_string(n) + " must equal" + std::to_string(mf->n));
    if (!x) return fail(MFGPU_EINVAL, "x is NULL");
    if (nch > 1 && ld < n) return fail(MFGPU_EINVAL, "row stride is smaller than the number of samples");
    mfgpu_status rs = mf_resolve_stage(mf);
    if (rs != MFGPU_OK) return rs;
    rs = mf_set_data_length(mf, mf->n);
    if (rs != MFGPU_OK) return rs;
    mf->have = false;
    mf->have_peaks = false;
    const size_t es = mf->esz();
    char *row = mf->x.as<char>() + es * (size_t) c0 * mf->ldx;
    if (nch == 1) CU(cudaMemcpyAsync(row, x, es * (size_t) n, kind, mf->stream));
    else
        CU(cudaMemcpy2DAsync(row, es * (size_t) mf->ldx, x, es * (size_t) ld, es * (size_t) n, (size_t) nch, kind,
                             mf->stream));
    unsigned char *dflag = mf->dead.as<unsigned char>() + c0;
    const size_t poff = (size_t) c0 * mf->dead_chunks;
    if (mf->prec == 4)
        CU(launch_dead<float>(reinterpret_cast<const float *>(row), mf->ldx, nch, mf->n, dflag,
                              mf->pmin.as<float>() + poff, mf->pmax.as<float>() + poff, mf->dead_chunks, mf->stream,
                              mf->xrange.as<float>() + c0));
    else
        CU(launch_dead<double>(reinterpret_cast<const double *>(row), mf->ldx, nch, mf->n, dflag,
                               mf->pmin.as<double>() + poff, mf->pmax.as<double>() + poff, mf->dead_chunks,
                               mf->stream));
    mf->launches += 2;
    // the reference copies the caller's samples before returning
    CU(cudaStreamSynchronize(mf->stream));
    return MFGPU_OK;
}

static mfgpu_status mf_store_signal(mfgpu_mf *mf, int c, int n, const void *x, cudaMemcpyKind kind)
{
    return mf_store_signals(mf, c, 1, n, x, n, kind);
}

mfgpu_status mfgpu_mf_set_signal(mfgpu_mf *mf, int it, int n, const void *x)
try
{
    MF_CHECK_INIT(mf);
    DeviceGuard g(mf->dev);
    int c;
    mfgpu_status st = mf_channel_of(mf, it, &c);
    if (st != MFGPU_OK) return st;
    return mf_store_signal(mf, c, n, x, cudaMemcpyHostToDevice);
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_set_channel_signal(mfgpu_mf *mf, int channel, int n, const void *x)
try
{
    MF_CHECK_INIT(mf);
    DeviceGuard g(mf->dev);
    if (channel < 0 || channel >= mf->nch) return fail(MFGPU_EINVAL, "channel out of range");
    return mf_store_signal(mf, channel, n, x, cudaMemcpyHostToDevice);
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_set_channel_signals(mfgpu_mf *mf, int first_channel, int n_channels, int n, const void *x,
                                          long ld)
try
{
    MF_CHECK_INIT(mf);
    DeviceGuard g(mf->dev);
    if (n_channels < 1 || first_channel < 0 || first_channel + n_channels > mf->nch)
        return fail(MFGPU_EINVAL, "channel range out of range");
    return mf_store_signals(mf, first_channel, n_channels, n, x, ld, cudaMemcpyHostToDevice);
}
catch (...)
{
    return mfgpu::status_of_exception();
}

// Checks and state shared by the window setters: n_src source rows, n
// samples; the caller then fills rows [0, n_src) of x with the window.
static mfgpu_status mf_window_begin(mfgpu_mf *mf, int n_src, int n)
{
    if (n_src < 1 || n_src > mf->nch)
        return fail(MFGPU_EINVAL, "n_src = " + std::to_string(n_src) + " must be in [1, " + std::to_string(mf->nch) + "]");
    if (n < 1 || n > mf->n)
        return fail(MFGPU_EINVAL, "window length " + std::to_string(n) + " must be in [1, " + std::to_string(mf->n) + "]");
    mfgpu_status rs = mf_resolve_stage(mf);
    if (rs != MFGPU_OK) return rs;
    rs = mf_set_data_length(mf, n);
    if (rs != MFGPU_OK) return rs;
    mf->have = false;
    mf->have_peaks = false;
    return MFGPU_OK;
}

// After the window's rows are in place: zero tail, channels c >= n_src
// repeating channel c % n_src, dead-trace flags over the window; waits.
static mfgpu_status mf_window_end(mfgpu_mf *mf, int n_src, int n)
{
    const size_t es = mf->esz(), pitch = es * (size_t) mf->ldx;
    char *x0 = mf->x.as<char>();
    if (n < mf->n)
        CU(cudaMemset2DAsync(x0 + es * (size_t) n, pitch, 0, es * (size_t) (mf->n - n), (size_t) n_src, mf->stream));
    for (int c0 = n_src; c0 < mf->nch; c0 += n_src)
        CU(cudaMemcpy2DAsync(x0 + pitch * (size_t) c0, pitch, x0, pitch, es * (size_t) mf->n,
                             (size_t) std::min(n_src, mf->nch - c0), cudaMemcpyDeviceToDevice, mf->stream));
    if (mf->prec == 4)
        CU(launch_dead<float>(mf->x.as<float>(), mf->ldx, mf->nch, n, mf->dead.as<unsigned char>(),
                              mf->pmin.as<float>(), mf->pmax.as<float>(), mf->dead_chunks, mf->stream,
                              mf->xrange.as<float>()));
    else
        CU(launch_dead<double>(mf->x.as<double>(), mf->ldx, mf->nch, n, mf->dead.as<unsigned char>(),
                               mf->pmin.as<double>(), mf->pmax.as<double>(), mf->dead_chunks, mf->stream));
    mf->launches += 2;
    CU(cudaStreamSynchronize(mf->stream));
    return MFGPU_OK;
}

mfgpu_status mfgpu_mf_set_window(mfgpu_mf *mf, int n_src, int n, const void *x, long ld)
try
{
    MF_CHECK_INIT(mf);
    DeviceGuard g(mf->dev);
    if (!x) return fail(MFGPU_EINVAL, "x is NULL");
    if (n_src > 1 && ld < n) return fail(MFGPU_EINVAL, "row stride is smaller than the number of samples");
    mfgpu_status rs = mf_window_begin(mf, n_src, n);
    if (rs != MFGPU_OK) return rs;
    const size_t es = mf->esz(), pitch = es * (size_t) mf->ldx;
    CU(cudaMemcpy2DAsync(mf->x.as<char>(), pitch, x, es * (size_t) (n_src > 1 ? ld : n), es * (size_t) n,
                         (size_t) n_src, cudaMemcpyHostToDevice, mf->stream));
    return mf_window_end(mf, n_src, n);
}
catch (...)
{
    return mfgpu::status_of_exception();
}

// ---- device ring of recent samples per channel (no reference counterpart)
struct mfgpu_ring
{
    int dev = 0, prec = 4, nch = 0;
    long cap = 0;          // samples kept per channel
    long long head = 0;    // samples appended so far: sample s of channel c at c * cap + s mod cap
    DevBuf buf;
    cudaStream_t stream = nullptr;
    std::mutex mu;         // appends and window reads
    size_t esz() const { return (size_t) prec; }
};

mfgpu_status mfgpu_ring_create(int precision, int n_channels, long capacity, mfgpu_ring **out)
try
{
    if (!out) return fail(MFGPU_EINVAL, "ring is NULL");
    if (precision != MFGPU_FLOAT32 && precision != MFGPU_FLOAT64)
        return fail(MFGPU_EINVAL, "precision must be MFGPU_FLOAT32 or MFGPU_FLOAT64");
    if (n_channels < 1) return fail(MFGPU_EINVAL, "n_channels must be positive");
    if (capacity < 1) return fail(MFGPU_EINVAL, "capacity must be positive");
    auto *r = new mfgpu_ring();
    r->prec = precision;
    r->nch = n_channels;
    r->cap = capacity;
    const size_t bytes = r->esz() * (size_t) n_channels * (size_t) capacity;
    cudaError_t e = cudaGetDevice(&r->dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&r->buf.p, bytes);  // exact size: no growth margin for a ring
    if (e == cudaSuccess) r->buf.bytes = bytes;
    if (e == cudaSuccess) e = cudaMemsetAsync(r->buf.p, 0, bytes, r->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(r->stream);
    if (e != cudaSuccess)
    {
        mfgpu_ring_destroy(r);
        return cuda_fail(e, "mfgpu_ring_create");
    }
    *out = r;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_ring_destroy(mfgpu_ring *r)
try
{
    if (!r) return MFGPU_OK;
    {
        DeviceGuard g(r->dev);
        if (r->stream) cudaStreamSynchronize(r->stream);
        r->buf.release();
        if (r->stream) cudaStreamDestroy(r->stream);
    }
    delete r;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_ring_append(mfgpu_ring *r, int n, const void *x, long ld)
try
{
    if (!r) return fail(MFGPU_EINVAL, "ring is NULL");
    if (n < 1) return fail(MFGPU_EINVAL, "n must be positive");
    if (!x) return fail(MFGPU_EINVAL, "x is NULL");
    if (r->nch > 1 && ld < n) return fail(MFGPU_EINVAL, "row stride is smaller than the number of samples");
    DeviceGuard g(r->dev);
    std::lock_guard<std::mutex> lk(r->mu);
    const size_t es = r->esz();
    const long keep = std::min<long>(n, r->cap);  // older samples of the chunk would be overwritten at once
    const long skip = n - keep;
    long long s = r->head + skip;
    long done = 0;
    while (done < keep)
    {
        const long pos = (long) (s % r->cap);
        const long len = std::min<long>(keep - done, r->cap - pos);
        CU(cudaMemcpy2DAsync(r->buf.as<char>() + es * (size_t) pos, es * (size_t) r->cap,
                             static_cast<const char *>(x) + es * (size_t) (skip + done), es * (size_t) (r->nch > 1 ? ld : n),
                             es * (size_t) len, (size_t) r->nch, cudaMemcpyHostToDevice, r->stream));
        done += len;
        s += len;
    }
    CU(cudaStreamSynchronize(r->stream));
    r->head += n;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_ring_get_head(mfgpu_ring *r, long long *appended)
try
{
    if (!r || !appended) return fail(MFGPU_EINVAL, "ring or appended is NULL");
    std::lock_guard<std::mutex> lk(r->mu);
    *appended = r->head;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_set_window_ring(mfgpu_mf *mf, mfgpu_ring *r, int n_src, const int *channels, long long end,
                                      int n)
try
{
    MF_CHECK_INIT(mf);
    if (!r) return fail(MFGPU_EINVAL, "ring is NULL");
    if (r->dev != mf->dev) return fail(MFGPU_EINVAL, "the ring and the object are on different devices");
    if (r->prec != mf->prec) return fail(MFGPU_EINVAL, "the ring and the object have different precisions");
    if (n_src < 1 || n_src > kRingMaxRows)
        return fail(MFGPU_EINVAL, "n_src must be in [1, " + std::to_string(kRingMaxRows) + "]");
    RingRows rr;
    for (int i = 0; i < n_src; ++i)
    {
        const int c = channels ? channels[i] : i;
        if (c < 0 || c >= r->nch)
            return fail(MFGPU_EINVAL, "ring channel " + std::to_string(c) + " must be in [0, " + std::to_string(r->nch) + ")");
        rr.src[i] = c;
    }
    if (n < 1 || n > r->cap)
        return fail(MFGPU_EINVAL, "window length " + std::to_string(n) + " must be in [1, " + std::to_string(r->cap) + "]");
    DeviceGuard g(mf->dev);
    std::lock_guard<std::mutex> lk(r->mu);  // no append overwrites the window while it is read
    if (end > r->head || end - n < 0 || end - n < r->head - r->cap)
        return fail(MFGPU_EINVAL, "window [" + std::to_string(end - n) + ", " + std::to_string(end) +
                                      ") is not in the ring (samples [" + std::to_string(std::max<long long>(0, r->head - r->cap)) +
                                      ", " + std::to_string(r->head) + "))");
    mfgpu_status rs = mf_window_begin(mf, n_src, n);
    if (rs != MFGPU_OK) return rs;
    const dim3 grid((unsigned) std::min<long>(64, (n + 255) / 256), (unsigned) n_src);
    if (mf->prec == 4)
        ring_gather_kernel<float><<<grid, 256, 0, mf->stream>>>(r->buf.as<float>(), r->cap, rr, end - n, n,
                                                                mf->x.as<float>(), mf->ldx);
    else
        ring_gather_kernel<double><<<grid, 256, 0, mf->stream>>>(r->buf.as<double>(), r->cap, rr, end - n, n,
                                                                 mf->x.as<double>(), mf->ldx);
    CU(cudaGetLastError());
    ++mf->launches;
    return mf_window_end(mf, n_src, n);  // waits: the window has been read before the lock is released
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_device_bytes(const mfgpu_mf *cmf, unsigned long long *bytes)
try
{
    auto *mf = const_cast<mfgpu_mf *>(cmf);
    if (!mf) return fail(MFGPU_EINVAL, "mf is NULL");
    if (!bytes) return fail(MFGPU_EINVAL, "bytes is NULL");
    *bytes = mf->device_bytes();
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_set_channel_signal_device(mfgpu_mf *mf, int channel, int n, const void *dx)
try
{
    MF_CHECK_INIT(mf);
    DeviceGuard g(mf->dev);
    if (channel < 0 || channel >= mf->nch) return fail(MFGPU_EINVAL, "channel out of range");
    return mf_store_signal(mf, channel, n, dx, cudaMemcpyDeviceToDevice);
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_zero_signal(mfgpu_mf *mf, int it)
try
{
    MF_CHECK_INIT(mf);
    DeviceGuard g(mf->dev);
    int c;
    mfgpu_status st = mf_channel_of(mf, it, &c);
    if (st != MFGPU_OK) return st;
    st = mf_resolve_stage(mf);
    if (st != MFGPU_OK) return st;
    mf->have = false;
    mf->have_peaks = false;
    const size_t es = mf->esz();
    CU(cudaMemsetAsync(mf->x.as<char>() + es * (size_t) c * mf->ldx, 0, es * (size_t) mf->n, mf->stream));
    CU(cudaMemsetAsync(mf->dead.as<unsigned char>() + c, 1, 1, mf->stream));
    CU(cudaStreamSynchronize(mf->stream));
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_signal(const mfgpu_mf *cmf, int it, int maxn, void *dst)
try
{
    auto *mf = const_cast<mfgpu_mf *>(cmf);
    MF_CHECK_INIT(mf);
    DeviceGuard g(mf->dev);
    int c;
    mfgpu_status st = mf_channel_of(mf, it, &c);
    if (st != MFGPU_OK) return st;
    if (!dst || maxn < mf->n) return fail(MFGPU_EINVAL, "destination too small");
    st = mf_resolve_stage(mf);
    if (st != MFGPU_OK) return st;
    const size_t es = mf->esz();
    CU(cudaMemcpyAsync(dst, mf->x.as<char>() + es * (size_t) c * mf->ldx, es * (size_t) mf->n,
                       cudaMemcpyDeviceToHost, mf->stream));
    CU(cudaStreamSynchronize(mf->stream));
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

// Records ev on the object's stream.  While apply is being captured into a
// graph the record must be external, or the replays would not record it
// (the staging buffers' reuse and the timings depend on these events).
static cudaError_t mf_record(mfgpu_mf *mf, cudaEvent_t ev)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(mf->stream, &cs);
    if (e != cudaSuccess) return e;
    return cudaEventRecordWithFlags(ev, mf->stream,
                                    cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault);
}

template <class T> static mfgpu_status mf_launch_xcorr(mfgpu_mf *mf)
{
    XcorrParams<T> p{};
    p.x = mf->x.as<T>(); p.ldx = mf->ldx;
    p.Bc = mf->Bc.as<cx<T>>(); p.ldb = (1L << mf->log2p) + 2;
    p.rho = mf->rho.as<T>(); p.ldr = mf->ldr;
    p.grp_chan = mf->grp_chan.as<int>(); p.grp_tb = mf->grp_tb.as<int>(); p.grp_te = mf->grp_te.as<int>();
    p.tids = mf->tids.as<int>();
    p.tlen = mf->tlen_d.as<int>(); p.nvalid = mf->nvalid_d.as<int>();
    p.dead = mf->dead.as<unsigned char>();
    p.twt = mf->tw.as<cx<T>>();
    p.twt_split = mf->tws.as<cx<T>>();
    p.S = mf->S;
    p.tol = sizeof(T) == 4 ? (T) 1.e-6 : (T) 1.e-12;  // src/matchedFilter.cpp:1287 / :1115
    p.err = mf->err.as<int>();
    p.den = mf->den.as<T>();
    p.ldd = mf->ldd;
    p.test_skip_copy = mf->test_wait_timeout && !mf->tc ? 1 : 0;
    mf->test_wait_timeout = false;
    if constexpr (sizeof(T) == 4)
    {
        if (mf->fx_on)
        {
            // normalisation rows (one length) and window statistics, then the
            // per-run error bounds of the chosen correlator
            CU(launch_den_robust(mf->x.as<float>(), mf->ldx, mf->fx_L, mf->shared_den ? mf->den.as<float>() : nullptr,
                                 mf->ldd, (float) p.tol, mf->rstat.as<float4>(), mf->ldrs, mf->cst.as<float2>(),
                                 mf->ldc, mf->fx_nden, mf->nch, mf->stream));
            CU(cudaMemsetAsync(mf->fxbits.p, 0, sizeof(unsigned) * (size_t) mf->nch * (mf->ldrs / 32), mf->stream));
            CU(cudaMemsetAsync(mf->fxcount.p, 0, sizeof(int), mf->stream));
            ++mf->launches;
            if (mf->tc)
            {
                CU(launch_fix_flag_tc(mf->x.as<float>(), mf->ldx, mf->fLen, mf->rstat.as<float4>(), mf->ldrs,
                                      mf->fx_nruns, mf->dlags.as<int>(), mf->tc_tiles, mf->nch,
                                      mf->dead.as<unsigned char>(),
                                      mf->xrange.as<float>(), mf->tc_off.as<float>(),
                                      mf->fxbits.as<unsigned>(), mf->fxlist.as<int>(), mf->fxcount.as<int>(),
                                      mf->tc_bf16 ? kFixTcC1 + kFixTcC1Bf16Per * mf->tc_maxb : kFixTcC1,
                                      mf->tc_bf16 ? kFixTcC2Bf16 : kFixTcC2,
                                      kFixTol, mf->stream));
                ++mf->launches;
            }
            else
            {
                const float coef = kFixFftK * 0x1p-24f / kFixTol;
                CU(launch_fix_flag_fft(mf->cst.as<float2>(), mf->ldc, mf->fx_nchunks, mf->S, mf->nfft, mf->nblocks,
                                       mf->nch, mf->rstat.as<float4>(), mf->ldrs, mf->fx_nruns, mf->dlags.as<int>(),
                                       mf->dead.as<unsigned char>(), mf->fxbits.as<unsigned>(), mf->fxlist.as<int>(),
                                       mf->fxcount.as<int>(), coef * coef,
                                       mf->stream));
                ++mf->launches;
                for (auto &xb : mf->xb)
                {
                    if (xb->ngroups == 0) continue;
                    CU(launch_fix_flag_fft(mf->cst.as<float2>(), mf->ldc, mf->fx_nchunks, xb->S, xb->nfft, xb->nblocks,
                                           mf->nch, mf->rstat.as<float4>(), mf->ldrs, mf->fx_nruns,
                                           mf->dlags.as<int>(), mf->dead.as<unsigned char>(), mf->fxbits.as<unsigned>(),
                                           mf->fxlist.as<int>(), mf->fxcount.as<int>(),
                                           coef * coef, mf->stream));
                    ++mf->launches;
                }
            }
        }
    }
    if (mf->shared_den && !(sizeof(T) == 4 && mf->fx_on))
    {
        CU(launch_den<T>(mf->x.as<T>(), mf->ldx, mf->fLen, mf->den.as<T>(), mf->ldd, p.tol, mf->nden, mf->nch,
                         mf->stream));
        ++mf->launches;
    }
    // fused peak candidates
    mf->pk_fused = false;
    p.pk_on = 0;
    p.pk_stride = mf->pk_stride;
    if (mf->pk_req >= 0 && !mf->tc)
    {
        const size_t nslot = (size_t) mf->nt * mf->pk_stride;
        CU(mf->pk_cnt.ensure(sizeof(int) * nslot));
        CU(mf->pk_idx.ensure(sizeof(int) * nslot * kPkCap));
        CU(mf->pk_val.ensure(sizeof(T) * nslot * kPkCap));
        CU(cudaMemsetAsync(mf->pk_cnt.p, 0, sizeof(int) * nslot, mf->stream));
        p.pk_on = 1;
        p.pk_len = mf->n - mf->maxLen + 1;
        p.pk_thr = (T) mf->pk_req;
        p.pk_cnt = mf->pk_cnt.as<int>();
        p.pk_idx = mf->pk_idx.as<int>();
        p.pk_val = mf->pk_val.as<T>();
    }
    CU(mf_record(mf, mf->ev[1]));
    if constexpr (sizeof(T) == 4)
    {
        if (mf->tc)
        {
            TcParams q{};
            q.x = mf->x.as<float>(); q.ldx = mf->ldx;
            q.B = mf->tc_B.as<__half>(); q.bscale = mf->tc_bscale.as<float>();
            q.grp_chan = mf->tc_grp_chan.as<int>(); q.grp_tid = mf->tc_grp_tid.as<int>();
            q.xrange = mf->xrange.as<float>(); q.dead = mf->dead.as<unsigned char>();
            q.off = mf->tc_off.as<float>();
            q.den = mf->den.as<float>(); q.ldd = mf->ldd;
            q.rho = mf->rho.as<float>(); q.ldr = mf->ldr;
            q.nv = mf->maxvalid; q.Kp = mf->tc_Kp; q.Gp = mf->tc_Gp; q.tmem_cols = mf->tc_cols;
            q.ngroups = mf->tc_groups; q.tiles = mf->tc_tiles; q.err = mf->err.as<int>();
            q.pk_flags = nullptr; q.pk_words = 0; q.pk_thr = 0.f;
            if (mf->pk_req >= 0)
            {
                // candidate flags: one bit per 64 lags, cleared per apply
                q.pk_words = (mf->tc_tiles * (kTcLags / 64) + 31) / 32;
                const size_t fb = sizeof(unsigned) * (size_t) mf->nt * q.pk_words;
                CU(mf->pk_flags.ensure(fb));
                CU(cudaMemsetAsync(mf->pk_flags.p, 0, fb, mf->stream));
                q.pk_flags = mf->pk_flags.as<unsigned>();
                q.pk_thr = (float) mf->pk_req;
            }
            const long work = (long) q.ngroups * q.tiles;
            CU(launch_tc_xcorr(q, (int) std::min<long>(mf->n_sm, work), mf->tc_bf16, mf->stream));
            ++mf->launches;
            if (q.pk_flags)
            {
                mf->pk_fused = true;
                mf->pk_fused_thr = mf->pk_req;
                mf->pk_fused_len = mf->n - mf->maxLen + 1;
                mf->pk_words = q.pk_words;
            }
            return MFGPU_OK;
        }
    }
    // persistent launches (an option): one ticket per correlator launch,
    // zeroed per apply; the FP32 two-team organisations at P >= 2048 only
    auto persist = [&](int mode, int log2p) {
        return mf->persistent && sizeof(T) == 4 && log2p >= 11 && (mode == 4 || (mode == 2 && mf->shared_den));
    };
    if (mf->persistent)
    {
        CU(mf->tickets.ensure(sizeof(int) * (1 + mf->xb.size())));
        CU(cudaMemsetAsync(mf->tickets.p, 0, sizeof(int) * (1 + mf->xb.size()), mf->stream));
    }
    p.ticket = persist(mf->mode_x, mf->log2p) ? mf->tickets.as<int>() : nullptr;
    p.nblk = mf->nblocks;
    p.ntiles = mf->nblocks * mf->ngroups;
    CU(launch_xcorr<T>(mf->log2p, mf->shared_den, mf->mode_x, p, mf->nblocks, mf->ngroups, mf->stream));
    ++mf->launches;
    // the other length buckets, one launch each
    for (auto &xb : mf->xb)
    {
        if (xb->ngroups == 0) continue;
        XcorrParams<T> q = p;
        q.Bc = xb->Bc.as<cx<T>>(); q.ldb = (1L << xb->log2p) + 2;
        q.grp_chan = xb->grp_chan.as<int>(); q.grp_tb = xb->grp_tb.as<int>(); q.grp_te = xb->grp_te.as<int>();
        q.tids = xb->tids.as<int>();
        q.twt = xb->tw.as<cx<T>>();
        q.twt_split = xb->tws.as<cx<T>>();
        q.S = xb->S;
        q.ticket = persist(xb->mode, xb->log2p) ? mf->tickets.as<int>() + 1 + (&xb - &mf->xb[0]) : nullptr;
        q.nblk = xb->nblocks;
        q.ntiles = xb->nblocks * xb->ngroups;
        CU(launch_xcorr<T>(xb->log2p, false, xb->mode, q, xb->nblocks, xb->ngroups, mf->stream));
        ++mf->launches;
    }
    if (p.pk_on)
    {
        mf->pk_fused = true;
        mf->pk_fused_thr = mf->pk_req;
        mf->pk_fused_len = p.pk_len;
    }
    return MFGPU_OK;
}

// After the correlator: the FP32 fix-up of the runs the error bounds listed
// (every template of the run's channel), and the direct time-domain
// correlation of templates longer than any FFT plan takes (every run); then
// the fused peak candidates of the blocks either touched are recounted.  The
// fix-up reads the list's length from device memory, so the host never
// waits for the bounds; with no listed run it returns at once.
template <class T> static mfgpu_status mf_launch_fixup(mfgpu_mf *mf)
{
    FixParams<T> f{};
    f.x = mf->x.as<T>(); f.ldx = mf->ldx;
    f.rho = mf->rho.as<T>(); f.ldr = mf->ldr;
    f.ldf = mf->ldrs; f.nruns = mf->fx_nruns;
    f.bch = mf->fx_bch.as<int>(); f.dead = mf->dead.as<unsigned char>();
    f.btid = mf->fx_btid.as<int>(); f.boff = mf->fx_boff.as<long>();
    f.bL = mf->fx_bL.as<int>(); f.bco = mf->fx_bco.as<T>(); f.bsum = mf->fx_bsum.as<T>();
    f.tlen = mf->tlen_d.as<int>(); f.nvalid = mf->nvalid_d.as<int>();
    f.tol = sizeof(T) == 4 ? (T) 1.e-6 : (T) 1.e-12;  // src/matchedFilter.cpp:1287 / :1115
    const bool fused = mf->pk_fused && !mf->tc;
    if (mf->pk_fused && mf->tc)
    {
        f.pk_flags = mf->pk_flags.as<unsigned>();
        f.pk_words = mf->pk_words;
        f.pk_thr = (T) mf->pk_fused_thr;
        f.pk_len = mf->pk_fused_len;
    }
    if (fused)
    {
        const size_t ns = (size_t) mf->nt * mf->pk_stride;
        CU(mf->pk_dirty.ensure(ns));
        CU(cudaMemsetAsync(mf->pk_dirty.p, 0, ns, mf->stream));
        f.pk_dirty = mf->pk_dirty.as<unsigned char>();
        f.pk_stride = mf->pk_stride;
        f.row_S = mf->xb.empty() ? nullptr : mf->row_S.as<int>();
        f.S0 = mf->S;
    }
    const int nctas = 4 * std::max(1, mf->n_sm);
    if (mf->fx_on && mf->nblocks > 0 && !mf->test_skip_fixup)
    {
        FixParams<T> g = f;
        g.flist = mf->fxlist.as<int>(); g.fcount = mf->fxcount.as<int>();
        g.nbmax = mf->fx_nbmax;
        g.chan_b0 = mf->fx_cb0.as<int>(); g.chan_nb = mf->fx_cnb.as<int>();
        g.Lmax = mf->fx_lmax;
        CU(launch_fixup<T>(g, nctas, fixup_warps<T>(g.Lmax, mf->dev_smem), mf->stream));
        ++mf->launches;
    }
    if (mf->n_direct > 0)
    {
        FixParams<T> g = f;
        g.flist = nullptr;
        g.dir_b0 = mf->dir_b0; g.ndir = mf->dir_nb;
        g.Lmax = mf->dir_lmax;
        CU(launch_fixup<T>(g, nctas, fixup_warps<T>(g.Lmax, mf->dev_smem), mf->stream));
        ++mf->launches;
    }
    if (fused)
    {
        CU(launch_fix_rescan<T>(mf->rho.as<T>(), mf->ldr, mf->nt, mf->pk_stride, mf->pk_dirty.as<unsigned char>(),
                                mf->xb.empty() ? nullptr : mf->row_S.as<int>(),
                                mf->xb.empty() ? nullptr : mf->row_nblk.as<int>(), mf->S, mf->nblocks,
                                mf->nvalid_d.as<int>(), mf->pk_fused_len, (T) mf->pk_fused_thr, mf->pk_cnt.as<int>(),
                                mf->pk_idx.as<int>(), mf->pk_val.as<T>(), mf->stream));
        ++mf->launches;
    }
    return MFGPU_OK;
}

// the stream work of one apply (events, normalisation, correlators)
static mfgpu_status mf_apply_body(mfgpu_mf *mf)
{
    CU(mf_record(mf, mf->ev[0]));
    if (mf->nblocks > 0)
    {
        // records ev[1] between the normalisation and the correlator
        mfgpu_status st = mf->prec == 4 ? mf_launch_xcorr<float>(mf) : mf_launch_xcorr<double>(mf);
        if (st != MFGPU_OK) return st;
    }
    else
    {
        CU(mf_record(mf, mf->ev[1]));
    }
    CU(mf_record(mf, mf->ev[2]));
    if ((mf->nblocks > 0 && mf->fx_on) || mf->n_direct > 0)
    {
        mfgpu_status st = mf->prec == 4 ? mf_launch_fixup<float>(mf) : mf_launch_fixup<double>(mf);
        if (st != MFGPU_OK) return st;
    }
    CU(mf_record(mf, mf->ev[3]));
    CU(mf_record(mf, mf->x_ev));  // the last read of x by this apply
    return MFGPU_OK;
}

mfgpu_status mfgpu_mf_apply(mfgpu_mf *mf)
try
{
    if (!mf) return fail(MFGPU_EINVAL, "mf is NULL");
    if (!mf->initialized) return fail(MFGPU_ESTATE, "Class is not initialized");
    DeviceGuard g(mf->dev);
    mfgpu_status rs = mf_resolve_stage(mf);
    if (rs != MFGPU_OK) return rs;
    mf->have = false;
    mf->have_peaks = false;
    if (mf->use_graph && !mf->test_wait_timeout)
    {
        mfgpu_mf::ApplyGraph key;
        key.x = mf->x.p;
        key.pk_cnt = mf->pk_cnt.p;
        key.pk_flags = mf->pk_flags.p;
        key.pk_req = mf->pk_req;
        for (mfgpu_mf::ApplyGraph &gr : mf->graphs)
            if (gr.exec && gr.same(key))
            {
                CU(cudaGraphLaunch(gr.exec, mf->stream));
                mf->pk_fused = gr.pk_fused;
                mf->pk_fused_thr = gr.pk_fused_thr;
                mf->pk_fused_len = gr.pk_fused_len;
                mf->pk_words = gr.pk_words;
                mf->launches += gr.launches;
                ++mf->graph_launches;
                mf->timed = true;
                mf->have = true;
                return MFGPU_OK;
            }
        if (mf->last_direct[0].same(key) || mf->last_direct[1].same(key))
        {
            // every buffer of this setup is sized: capture the stream work
            const long long l0 = mf->launches;
            CU(cudaStreamBeginCapture(mf->stream, cudaStreamCaptureModeThreadLocal));
            mfgpu_status st = mf_apply_body(mf);
            cudaGraph_t graph = nullptr;
            cudaError_t e = cudaStreamEndCapture(mf->stream, &graph);
            if (st != MFGPU_OK)
            {
                if (graph) cudaGraphDestroy(graph);
                return st;
            }
            if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
            cudaGraphExec_t exec = nullptr;
            e = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
            mfgpu_mf::ApplyGraph &slot = mf->graphs[mf->graph_next];
            mf->graph_next ^= 1;
            if (slot.exec) cudaGraphExecDestroy(slot.exec);
            slot = key;
            slot.exec = exec;
            slot.pk_fused = mf->pk_fused;
            slot.pk_fused_thr = mf->pk_fused_thr;
            slot.pk_fused_len = mf->pk_fused_len;
            slot.pk_words = mf->pk_words;
            slot.launches = mf->launches - l0;
            CU(cudaGraphLaunch(exec, mf->stream));
            ++mf->graph_launches;
            mf->timed = true;
            mf->have = true;
            return MFGPU_OK;
        }
    }
    const bool testing = mf->test_wait_timeout;
    mfgpu_status st = mf_apply_body(mf);
    if (st != MFGPU_OK) return st;
    if (mf->use_graph && !testing)
    {
        // the direct run may have resized buffers: the setup is taken after it
        mfgpu_mf::ApplyGraph &d = mf->last_direct[mf->direct_next];
        mf->direct_next ^= 1;
        d = mfgpu_mf::ApplyGraph();
        d.x = mf->x.p;
        d.pk_cnt = mf->pk_cnt.p;
        d.pk_flags = mf->pk_flags.p;
        d.pk_req = mf->pk_req;
    }
    mf->timed = true;
    mf->have = true;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_set_graph(mfgpu_mf *mf, int enable)
try
{
    if (!mf) return fail(MFGPU_EINVAL, "mf is NULL");
    DeviceGuard g(mf->dev);
    if (mf->copy_stream) CU(cudaStreamSynchronize(mf->copy_stream));
    CU(cudaStreamSynchronize(mf->stream));
    mf->drop_graphs();
    mf->use_graph = enable != 0;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_graph_launches(const mfgpu_mf *mf, long long *count)
try
{
    if (!mf || !count) return fail(MFGPU_EINVAL, "NULL argument");
    *count = mf->graph_launches;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_synchronize(mfgpu_mf *mf)
try
{
    if (!mf) return fail(MFGPU_EINVAL, "mf is NULL");
    DeviceGuard g(mf->dev);
    return mf_sync(mf, true);
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_have_matched_filtered_signals(const mfgpu_mf *mf, int *flag)
try
{
    if (!mf || !flag) return fail(MFGPU_EINVAL, "NULL argument");
    *flag = mf->have ? 1 : 0;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_last_timings(mfgpu_mf *mf, float *xcorr_ms, float *apply_ms)
try
{
    if (!mf) return fail(MFGPU_EINVAL, "mf is NULL");
    DeviceGuard g(mf->dev);
    mfgpu_status st = mf_sync(mf);
    if (st != MFGPU_OK) return st;
    if (xcorr_ms) *xcorr_ms = mf->last_xcorr_ms;
    if (apply_ms) *apply_ms = mf->last_apply_ms;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_launch_count(const mfgpu_mf *mf, long long *count)
try
{
    if (!mf || !count) return fail(MFGPU_EINVAL, "NULL argument");
    *count = mf->launches;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_test_skip_fixup(mfgpu_mf *mf, int skip)
try
{
    if (!mf) return fail(MFGPU_EINVAL, "mf is NULL");
    DeviceGuard g(mf->dev);
    if (mf->copy_stream) CU(cudaStreamSynchronize(mf->copy_stream));
    CU(cudaStreamSynchronize(mf->stream));
    mf->drop_graphs();  // captured applies hold the old setting
    mf->test_skip_fixup = skip != 0;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_test_wait_timeout(mfgpu_mf *mf)
try
{
    if (!mf) return fail(MFGPU_EINVAL, "mf is NULL");
    if (!mf->initialized) return fail(MFGPU_ESTATE, "Class is not initialized");
    if (mf->tc) return fail(MFGPU_EINVAL, "the wait test runs on the FFT correlator");
    mf->test_wait_timeout = true;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_fixup_runs(mfgpu_mf *mf, long long *runs)
try
{
    if (!mf || !runs) return fail(MFGPU_EINVAL, "NULL argument");
    if (!mf->initialized) return fail(MFGPU_ESTATE, "Class is not initialized");
    DeviceGuard g(mf->dev);
    *runs = 0;
    mfgpu_status st = mf_sync(mf);
    if (st != MFGPU_OK) return st;
    if (!mf->fx_on || !mf->have) return MFGPU_OK;
    int k = 0;
    CU(cudaMemcpy(&k, mf->fxcount.p, sizeof(int), cudaMemcpyDeviceToHost));
    *runs = k;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_stream(const mfgpu_mf *mf, void **stream)
try
{
    if (!mf || !stream) return fail(MFGPU_EINVAL, "NULL argument");
    *stream = (void *) mf->stream;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

static mfgpu_status mf_check_template(mfgpu_mf *mf, int it)
{
    if (it < 0 || it >= mf->nt)
        return fail(MFGPU_EINVAL, "it = " + std::to_string(it) + " must be in the range [0," +
                                      std::to_string(mf->nt - 1) + "]");
    return MFGPU_OK;
}

static mfgpu_status mf_copy_rho(mfgpu_mf *mf, int it, int count, int maxn, void *dst, int *nout)
{
    if (!mf->have) return fail(MFGPU_ESTATE, "Matched filtering not yet applied");
    mfgpu_status st = mf_check_template(mf, it);
    if (st != MFGPU_OK) return st;
    st = mf_sync(mf);
    if (st != MFGPU_OK) return st;
    count = std::max(0, count);
    if (count > 0 && (!dst || maxn < count))
        return fail(MFGPU_EINVAL, "maxn = " + std::to_string(maxn) + " must be at least " + std::to_string(count));
    const size_t es = mf->esz();
    if (count > 0)
        CU(cudaMemcpy(dst, mf->rho.as<char>() + es * (size_t) it * mf->ldr, es * (size_t) count,
                      cudaMemcpyDeviceToHost));
    if (nout) *nout = count;
    return MFGPU_OK;
}

mfgpu_status mfgpu_mf_get_matched_filtered_signal(mfgpu_mf *mf, int it, int maxn, void *dst, int *nout)
try
{
    MF_CHECK_INIT(mf);
    DeviceGuard g(mf->dev);
    return mf_copy_rho(mf, it, mf->n - mf->maxLen + 1, maxn, dst, nout);
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_valid_signal(mfgpu_mf *mf, int it, int maxn, void *dst, int *nout)
try
{
    MF_CHECK_INIT(mf);
    DeviceGuard g(mf->dev);
    mfgpu_status st = mf_check_template(mf, it);
    if (st != MFGPU_OK) return st;
    return mf_copy_rho(mf, it, mf->nvalid[it], maxn, dst, nout);
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_device_signal(mfgpu_mf *mf, int it, const void **dptr, int *nvalid)
try
{
    MF_CHECK_INIT(mf);
    mfgpu_status st = mf_check_template(mf, it);
    if (st != MFGPU_OK) return st;
    if (!dptr) return fail(MFGPU_EINVAL, "dptr is NULL");
    *dptr = mf->rho.as<char>() + mf->esz() * (size_t) it * mf->ldr;
    if (nvalid) *nvalid = mf->nvalid[it];
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

template <class T> static mfgpu_status mf_stack(mfgpu_mf *mf, int maxn, void *dst, int *nout)
{
    const int nfilt = mf->n - mf->maxLen + 1;
    int smax = mf->shifts[0];
    T xnorm = 0;
    for (int t = 0; t < mf->nt; ++t)
    {
        smax = std::max(smax, mf->shifts[t]);
        xnorm = xnorm + (T) mf->weights[t];
    }
    if (xnorm > 0) xnorm = 1 / xnorm;
    const int outlen = nfilt - smax;
    if (nout) *nout = std::max(0, outlen);
    if (outlen <= 0) return MFGPU_OK;
    if (!dst || maxn < outlen)
        return fail(MFGPU_EINVAL, "maxn = " + std::to_string(maxn) + " must be at least " + std::to_string(outlen));
    std::vector<T> w(mf->nt);
    for (int t = 0; t < mf->nt; ++t) w[t] = xnorm * (T) mf->weights[t];
    CU(mf->shifts_d.ensure(sizeof(int) * mf->nt));
    CU(mf->weights_d.ensure(sizeof(T) * mf->nt));
    CU(mf->stackbuf.ensure(sizeof(T) * (size_t) outlen));
    CU(cudaMemcpyAsync(mf->shifts_d.p, mf->shifts.data(), sizeof(int) * mf->nt, cudaMemcpyHostToDevice, mf->stream));
    CU(cudaMemcpyAsync(mf->weights_d.p, w.data(), sizeof(T) * mf->nt, cudaMemcpyHostToDevice, mf->stream));
    CU(launch_stack<T>(mf->rho.as<T>(), mf->ldr, mf->nt, mf->shifts_d.as<int>(), mf->weights_d.as<T>(),
                       mf->stack_abs, outlen, mf->stackbuf.as<T>(), mf->stream));
    ++mf->launches;
    CU(cudaMemcpyAsync(dst, mf->stackbuf.p, sizeof(T) * (size_t) outlen, cudaMemcpyDeviceToHost, mf->stream));
    CU(cudaStreamSynchronize(mf->stream));
    return MFGPU_OK;
}

mfgpu_status mfgpu_mf_shift_and_stack(mfgpu_mf *mf, int maxn, void *dst, int *nout)
try
{
    MF_CHECK_INIT(mf);
    DeviceGuard g(mf->dev);
    if (!mf->have) return fail(MFGPU_ESTATE, "Matched filtered signals not yet computed");
    if (!mf->can_stack) return fail(MFGPU_ESTATE, "Templates missing info - can't shift");
    mfgpu_status st = mf_sync(mf);
    if (st != MFGPU_OK) return st;
    return mf->prec == 4 ? mf_stack<float>(mf, maxn, dst, nout) : mf_stack<double>(mf, maxn, dst, nout);
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_spectra_of_template(mfgpu_mf *mf, int it, int maxn, void *dst, int *nout)
try
{
    MF_CHECK_INIT(mf);
    DeviceGuard g(mf->dev);
    mfgpu_status st = mf_check_template(mf, it);
    if (st != MFGPU_OK) return st;
    int rn = 0, rl = 0;
    st = fft_sizes(mf->maxLen, mf->n + mf->maxLen - 1, &rn, &rl);
    if (st != MFGPU_OK) return st;
    const int ns = rn / 2 + 1;
    if (!dst || maxn < 2 * ns) return fail(MFGPU_EINVAL, "maxn must be at least 2*(nfft/2+1)");
    const size_t es = mf->esz();
    CU(mf->specbuf.ensure(es * 2 * (size_t) ns));
    const double *tp = mf->tmpl_d.as<double>() + mf->toff[it];
    if (mf->prec == 4) CU(launch_ref_spectrum<float>(tp, mf->lens[it], rn, mf->specbuf.as<float>(), mf->stream));
    else CU(launch_ref_spectrum<double>(tp, mf->lens[it], rn, mf->specbuf.as<double>(), mf->stream));
    ++mf->launches;
    CU(cudaMemcpyAsync(dst, mf->specbuf.p, es * 2 * (size_t) ns, cudaMemcpyDeviceToHost, mf->stream));
    CU(cudaStreamSynchronize(mf->stream));
    if (nout) *nout = 2 * ns;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_find_peaks(mfgpu_mf *mf, double threshold, int min_distance, int trace_length)
try
{
    MF_CHECK_INIT(mf);
    DeviceGuard g(mf->dev);
    if (!mf->have) return fail(MFGPU_ESTATE, "Matched filtering not yet applied");
    if (threshold < 0 || threshold > 1)
        return fail(MFGPU_EINVAL, "Threshold = " + std::to_string(threshold) + " must be in the range [0,1]");
    int len = trace_length > 0 ? trace_length : mf->n - mf->maxLen + 1;
    if (len > mf->maxvalid) return fail(MFGPU_EINVAL, "trace_length exceeds the valid lags");
    mfgpu_status st = mf_sync(mf);
    if (st != MFGPU_OK) return st;
    mf->have_peaks = false;
    std::vector<int> rows(mf->nt);
    for (int t = 0; t < mf->nt; ++t) rows[t] = t;
    mf->pk_off.assign(mf->nt + 1, 0);
    std::string err;
    // candidates of the last apply when it gathered them for this threshold and length
    const bool match = mf->pk_fused && threshold == mf->pk_fused_thr && len <= mf->pk_fused_len;
    // the FFT correlator gathered the candidates (same trace length); the
    // tensor-core correlator flagged the 64-lag chunks above the threshold
    const bool fused = match && !mf->tc && len == mf->pk_fused_len;
    const unsigned *flags = match && mf->tc ? mf->pk_flags.as<unsigned>() : nullptr;
    FusedSlots<float> ff{mf->pk_cnt.as<int>(), mf->pk_idx.as<int>(), mf->pk_val.as<float>(), mf->pk_stride, mf->S,
                         mf->row_S.as<int>(), mf->row_nblk.as<int>()};
    FusedSlots<double> fd{mf->pk_cnt.as<int>(), mf->pk_idx.as<int>(), mf->pk_val.as<double>(), mf->pk_stride, mf->S,
                          mf->row_S.as<int>(), mf->row_nblk.as<int>()};
    int rc = mf->prec == 4
                 ? run_peaks<float>(mf->rho.as<float>(), mf->ldr, rows.data(), mf->nt, len, threshold, min_distance,
                                    mf->pk, mf->stream, &mf->launches, mf->pk_off.data(), err, fused ? &ff : nullptr,
                                    flags, mf->pk_words)
                 : run_peaks<double>(mf->rho.as<double>(), mf->ldr, rows.data(), mf->nt, len, threshold,
                                     min_distance, mf->pk, mf->stream, &mf->launches, mf->pk_off.data(), err,
                                     fused ? &fd : nullptr);
    if (rc != 0) return fail(MFGPU_ECUDA, err);
    mf->have_peaks = true;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

template <class T> static mfgpu_status mf_detect(mfgpu_mf *mf, const mfgpu_detect_params *dp, long len)
{
    const double thr = std::min(1.0, std::max(0.0, dp->threshold));
    const int nt = mf->nt;
    const T *rho = mf->rho.as<T>();
    std::vector<int> rows_host;
    std::vector<long long> off(nt + 1, 0);
    std::string err;
    int ndet = 0;
    mf->have_peaks = false;  // the peak workspace is reused below
    if (!dp->single)
    {
        CU(mf->det_buf.ensure(sizeof(T) * (size_t) len));
        CU(mf->det_id.ensure(sizeof(int) * (size_t) len));
        CU(launch_det_reduce<T>(rho, mf->ldr, nt, len, dp->absolute_maximum, mf->det_buf.as<T>(),
                                mf->det_id.as<int>(), mf->stream));
        ++mf->launches;
        const int row0 = 0;
        if (run_peaks<T>(mf->det_buf.as<T>(), 0, &row0, 1, (int) len, thr, dp->min_distance, mf->pk, mf->stream,
                         &mf->launches, off.data(), err) != 0)
            return fail(MFGPU_ECUDA, err);
        ndet = (int) off[1];
        rows_host.assign(ndet, -1);
    }
    else
    {
        CU(mf->det_buf.ensure(sizeof(T) * (size_t) nt * mf->ldr));
        CU(launch_det_single<T>(rho, mf->ldr, nt, len, dp->absolute_maximum, mf->det_buf.as<T>(), mf->stream));
        ++mf->launches;
        std::vector<int> rows(nt);
        for (int t = 0; t < nt; ++t) rows[t] = t;
        if (run_peaks<T>(mf->det_buf.as<T>(), mf->ldr, rows.data(), nt, (int) len, thr, dp->min_distance, mf->pk,
                         mf->stream, &mf->launches, off.data(), err) != 0)
            return fail(MFGPU_ECUDA, err);
        ndet = (int) off[nt];
        rows_host.resize(ndet);
        for (int t = 0; t < nt; ++t)
            for (long long i = off[t]; i < off[t + 1]; ++i) rows_host[i] = t;
    }
    mf->dets.clear();
    if (ndet == 0) return MFGPU_OK;
    CU(mf->det_rows.ensure(sizeof(int) * (size_t) ndet));
    CU(mf->det_out.ensure(sizeof(DetectOut) * (size_t) ndet));
    CU(mf->det_id.ensure(sizeof(int)));
    CU(cudaMemcpyAsync(mf->det_rows.p, rows_host.data(), sizeof(int) * ndet, cudaMemcpyHostToDevice, mf->stream));
    DetectParams q{};
    q.peak = mf->pk.peaks.as<int>();
    q.row = mf->det_rows.as<int>();
    q.id = mf->det_id.as<int>();
    q.ndet = ndet;
    q.len = len;
    q.use_abs = dp->absolute_maximum;
    q.interp = dp->interpolation;
    q.alpha = dp->lanczos_alpha;
    q.nrefine = dp->lanczos_points;
    q.dt = 1.0 / dp->sampling_rate;
    q.amplitudes = dp->amplitudes;
    q.tmpl = mf->tmpl_d.as<double>();
    q.toff = mf->toff_d.as<long>();
    q.tlen = mf->tlen_d.as<int>();
    q.tchan = mf->tchan_d.as<int>();
    q.n = mf->n;
    q.out = mf->det_out.as<DetectOut>();
    CU(launch_det_refine<T>(rho, mf->ldr, mf->x.as<T>(), mf->ldx, q, mf->stream));
    ++mf->launches;
    std::vector<DetectOut> out(ndet);
    CU(cudaMemcpyAsync(out.data(), mf->det_out.p, sizeof(DetectOut) * ndet, cudaMemcpyDeviceToHost, mf->stream));
    CU(cudaStreamSynchronize(mf->stream));
    const double dt = 1.0 / dp->sampling_rate;
    mf->dets.resize(ndet);
    for (int i = 0; i < ndet; ++i)
    {
        const DetectOut &o = out[i];
        mfgpu_detection &d = mf->dets[i];
        d.template_index = o.tmpl;
        d.sample = o.sample;
        d.correlation = o.xc;
        d.detection_time = o.sample * dt;
        d.interpolated_time = d.detection_time + o.shift;
        d.sign = o.sign;
        d.have_amplitude = o.have_amp;
        d.gibbons_ringdal = o.gr;
        d.schaff_richards = o.sr;
    }
    if (dp->single)
        std::stable_sort(mf->dets.begin(), mf->dets.end(), [](const mfgpu_detection &a, const mfgpu_detection &b) {
            return a.detection_time < b.detection_time;
        });
    return MFGPU_OK;
}

mfgpu_status mfgpu_mf_detect(mfgpu_mf *mf, const mfgpu_detect_params *dp, int *n_detections)
try
{
    MF_CHECK_INIT(mf);
    DeviceGuard g(mf->dev);
    if (!dp) return fail(MFGPU_EINVAL, "params is NULL");
    if (!mf->have) return fail(MFGPU_EINVAL, "Matched filtered signals not computed");
    if (dp->interpolation < 0 || dp->interpolation > 2) return fail(MFGPU_EINVAL, "invalid interpolation type");
    if (dp->interpolation == 0 && (dp->lanczos_alpha < 1 || dp->lanczos_points < 1))
        return fail(MFGPU_EINVAL, "Lanczos alpha and points must be positive");
    if (!(dp->sampling_rate > 0)) return fail(MFGPU_EINVAL, "sampling rate must be positive");
    const long len = (long) mf->n - mf->maxLen + 1;  // getFilteredSignalLength
    if (len < 1) return fail(MFGPU_EINVAL, "Matched filtered signal length is 0");
    mfgpu_status st = mf_sync(mf);
    if (st != MFGPU_OK) return st;
    st = mf->prec == 4 ? mf_detect<float>(mf, dp, len) : mf_detect<double>(mf, dp, len);
    if (st != MFGPU_OK) return st;
    if (n_detections) *n_detections = (int) mf->dets.size();
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_detections(mfgpu_mf *mf, int max, mfgpu_detection *out, int *n)
try
{
    MF_CHECK_INIT(mf);
    const int nd = (int) mf->dets.size();
    if (n) *n = nd;
    if (max > 0 && !out) return fail(MFGPU_EINVAL, "out is NULL");
    for (int i = 0; i < nd && i < max; ++i) out[i] = mf->dets[i];
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_relative_amplitudes(int precision, int L, const double *templ, int n_windows, const void *windows,
                                       long ld, double *gr, double *sr, int *valid)
try
{
    if (precision != MFGPU_FLOAT32 && precision != MFGPU_FLOAT64)
        return fail(MFGPU_EINVAL, "precision must be MFGPU_FLOAT32 or MFGPU_FLOAT64");
    if (L < 1 || n_windows < 0) return fail(MFGPU_EINVAL, "L must be positive and n_windows non-negative");
    if (!templ || (n_windows > 0 && (!windows || !gr || !sr || !valid))) return fail(MFGPU_EINVAL, "NULL argument");
    if (n_windows > 1 && ld < L) return fail(MFGPU_EINVAL, "row stride is smaller than the window length");
    if (n_windows == 0) return MFGPU_OK;
    const size_t es = (size_t) precision, rows = (size_t) n_windows;
    const long ldd = n_windows > 1 ? ld : L;
    struct Scratch  // released on every return
    {
        DevBuf b[5];
        ~Scratch()
        {
            for (DevBuf &d : b) d.release();
        }
    } tmp;
    DevBuf &db = tmp.b[0], &dy = tmp.b[1], &dg = tmp.b[2], &ds = tmp.b[3], &dv = tmp.b[4];
    cudaStream_t s = cudaStreamPerThread;
    CU(db.ensure(sizeof(double) * L));
    CU(dy.ensure(es * (size_t) ldd * rows));
    CU(dg.ensure(sizeof(double) * rows));
    CU(ds.ensure(sizeof(double) * rows));
    CU(dv.ensure(sizeof(int) * rows));
    CU(cudaMemcpyAsync(db.p, templ, sizeof(double) * L, cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(dy.p, windows, es * (size_t) ldd * (rows - 1) + es * L, cudaMemcpyHostToDevice, s));
    if (precision == MFGPU_FLOAT32)
        CU(launch_amp<float>(db.as<double>(), L, dy.as<float>(), ldd, n_windows, dg.as<double>(), ds.as<double>(),
                             dv.as<int>(), s));
    else
        CU(launch_amp<double>(db.as<double>(), L, dy.as<double>(), ldd, n_windows, dg.as<double>(),
                              ds.as<double>(), dv.as<int>(), s));
    CU(cudaMemcpyAsync(gr, dg.p, sizeof(double) * rows, cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(sr, ds.p, sizeof(double) * rows, cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(valid, dv.p, sizeof(int) * rows, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_set_peak_threshold(mfgpu_mf *mf, double threshold)
try
{
    if (!mf) return fail(MFGPU_EINVAL, "mf is NULL");
    if (threshold > 1) return fail(MFGPU_EINVAL, "Threshold = " + std::to_string(threshold) + " must be at most 1");
    mf->pk_req = threshold < 0 ? -1.0 : threshold;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_peak_threshold(const mfgpu_mf *mf, double *threshold, int *active)
try
{
    if (!mf || !threshold) return fail(MFGPU_EINVAL, "NULL argument");
    *threshold = mf->pk_req;
    if (active) *active = mf->pk_fused ? 1 : 0;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_peaks(mfgpu_mf *mf, int it, int maxn, int *dst, int *nout)
try
{
    MF_CHECK_INIT(mf);
    DeviceGuard g(mf->dev);
    if (!mf->have_peaks) return fail(MFGPU_ESTATE, "peaks not computed");
    mfgpu_status st = mf_check_template(mf, it);
    if (st != MFGPU_OK) return st;
    long long cnt = mf->pk_off[it + 1] - mf->pk_off[it];
    if (cnt > 0 && (!dst || maxn < cnt)) return fail(MFGPU_EINVAL, "destination too small");
    if (cnt > 0)
        CU(cudaMemcpy(dst, mf->pk.peaks.as<int>() + mf->pk_off[it], sizeof(int) * (size_t) cnt,
                      cudaMemcpyDeviceToHost));
    if (nout) *nout = (int) cnt;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_mf_get_all_peaks(mfgpu_mf *mf, int nt, int *counts, int max_total, int *indices, int *total)
try
{
    MF_CHECK_INIT(mf);
    DeviceGuard g(mf->dev);
    if (!mf->have_peaks) return fail(MFGPU_ESTATE, "peaks not computed");
    if (nt != mf->nt || !counts) return fail(MFGPU_EINVAL, "counts must hold one entry per template");
    long long tot = mf->pk_off[mf->nt];
    if (total) *total = (int) tot;
    for (int t = 0; t < mf->nt; ++t) counts[t] = (int) (mf->pk_off[t + 1] - mf->pk_off[t]);
    if (tot > 0 && indices == nullptr && max_total == 0) return MFGPU_OK;  // size query
    if (tot > 0)
    {
        if (!indices || max_total < tot) return fail(MFGPU_EINVAL, "indices too small");
        CU(cudaMemcpy(indices, mf->pk.peaks.p, sizeof(int) * (size_t) tot, cudaMemcpyDeviceToHost));
    }
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}


// ============================================================================
struct mfgpu_peaks
{
    int prec = 4;
    int dev = 0;
    cudaStream_t stream = nullptr;
    double thr = 0.7;  // DEFAULT_THRESH, src/peakFinder.cpp:24
    int dist = 0;      // src/peakFinder.cpp:167
    int n = 0;
    DevBuf x;
    PeakWS ws;
    std::vector<int> peaks;
    int npeaks = 0;
    long long launches = 0;
};


mfgpu_status mfgpu_peaks_create(int precision, mfgpu_peaks **out)
try
{
    if (!out) return fail(MFGPU_EINVAL, "pf is NULL");
    if (precision != MFGPU_FLOAT32 && precision != MFGPU_FLOAT64)
        return fail(MFGPU_EINVAL, "precision must be MFGPU_FLOAT32 or MFGPU_FLOAT64");
    auto *pf = new mfgpu_peaks();
    pf->prec = precision;
    cudaError_t e = cudaGetDevice(&pf->dev);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&pf->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess)
    {
        delete pf;
        return cuda_fail(e, "mfgpu_peaks_create");
    }
    *out = pf;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_peaks_destroy(mfgpu_peaks *pf)
try
{
    if (!pf) return MFGPU_OK;
    {
        DeviceGuard g(pf->dev);
        cudaStreamSynchronize(pf->stream);
        pf->x.release();
        pf->ws.release();
        cudaStreamDestroy(pf->stream);
    }
    delete pf;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_peaks_clear(mfgpu_peaks *pf)
try
{
    if (!pf) return fail(MFGPU_EINVAL, "pf is NULL");
    DeviceGuard g(pf->dev);
    cudaStreamSynchronize(pf->stream);
    pf->x.release();
    pf->ws.release();
    pf->thr = 0.7;
    pf->dist = 0;
    pf->n = 0;
    pf->npeaks = 0;
    pf->peaks.clear();
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_peaks_set_threshold(mfgpu_peaks *pf, double threshold)
try
{
    if (!pf) return fail(MFGPU_EINVAL, "pf is NULL");
    pf->npeaks = 0;
    if (threshold < 0 || threshold > 1)
        return fail(MFGPU_EINVAL, "Threshold = " + std::to_string(threshold) + " must be in the range [0,1]");
    pf->thr = threshold;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_peaks_get_threshold(const mfgpu_peaks *pf, double *threshold)
try
{
    if (!pf || !threshold) return fail(MFGPU_EINVAL, "NULL argument");
    *threshold = pf->thr;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_peaks_set_minimum_peak_distance(mfgpu_peaks *pf, int min_distance)
try
{
    if (!pf) return fail(MFGPU_EINVAL, "pf is NULL");
    pf->npeaks = 0;
    pf->dist = min_distance;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_peaks_get_minimum_peak_distance(const mfgpu_peaks *pf, int *min_distance)
try
{
    if (!pf || !min_distance) return fail(MFGPU_EINVAL, "NULL argument");
    *min_distance = pf->dist;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_peaks_set_signal(mfgpu_peaks *pf, int n, const void *x)
try
{
    if (!pf) return fail(MFGPU_EINVAL, "pf is NULL");
    pf->npeaks = 0;
    if (n < 1) return fail(MFGPU_EINVAL, "No points in x");
    if (!x) return fail(MFGPU_EINVAL, "x is NULL");
    DeviceGuard g(pf->dev);
    // the candidate scan reads 16-sample vectors: pad to a multiple of 16
    CU(pf->x.ensure((size_t) pf->prec * ((n + 15) / 16 * 16)));
    CU(cudaMemcpyAsync(pf->x.p, x, (size_t) pf->prec * n, cudaMemcpyHostToDevice, pf->stream));
    CU(cudaStreamSynchronize(pf->stream));
    pf->n = n;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_peaks_apply(mfgpu_peaks *pf)
try
{
    if (!pf) return fail(MFGPU_EINVAL, "pf is NULL");
    DeviceGuard g(pf->dev);
    pf->npeaks = 0;
    pf->peaks.clear();
    if (pf->n < 1) return MFGPU_OK;
    int row = 0;
    long long off[2] = {0, 0};
    std::string err;
    int rc = pf->prec == 4 ? run_peaks<float>(pf->x.as<float>(), 0, &row, 1, pf->n, pf->thr, pf->dist, pf->ws,
                                              pf->stream, &pf->launches, off, err)
                           : run_peaks<double>(pf->x.as<double>(), 0, &row, 1, pf->n, pf->thr, pf->dist, pf->ws,
                                               pf->stream, &pf->launches, off, err);
    if (rc != 0) return fail(MFGPU_ECUDA, err);
    pf->npeaks = (int) (off[1] - off[0]);
    pf->peaks.resize(pf->npeaks);
    if (pf->npeaks > 0)
        CU(cudaMemcpy(pf->peaks.data(), pf->ws.peaks.p, sizeof(int) * pf->npeaks, cudaMemcpyDeviceToHost));
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_peaks_get_number_of_peaks(const mfgpu_peaks *pf, int *n)
try
{
    if (!pf || !n) return fail(MFGPU_EINVAL, "NULL argument");
    *n = pf->npeaks;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_peaks_get_peak_indices(const mfgpu_peaks *pf, int maxn, int *dst)
try
{
    if (!pf) return fail(MFGPU_EINVAL, "pf is NULL");
    if (maxn < pf->npeaks)
        return fail(MFGPU_EINVAL, "maxx = " + std::to_string(maxn) + " must be at least = " +
                                      std::to_string(pf->npeaks));
    if (!dst) return fail(MFGPU_EINVAL, "peaks is NULL");
    if (pf->npeaks > 0) std::memcpy(dst, pf->peaks.data(), sizeof(int) * pf->npeaks);
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}


// ============================================================================
struct mfgpu_dbscan
{
    int dev = 0;
    cudaStream_t stream = nullptr;
    double eps = 3;     // src/dbscan.cpp:56
    int min_obs = 5;    // src/dbscan.cpp:58
    bool init = false, have_data = false, have_labels = false, have_weights = false;
    int nobs = 0, nf = 0, ncl = 0;
    std::vector<double> X, w;
    std::vector<int> labels;
    DbWS ws;
    long long launches = 0;
};


mfgpu_status mfgpu_dbscan_create(mfgpu_dbscan **out)
try
{
    if (!out) return fail(MFGPU_EINVAL, "db is NULL");
    auto *db = new mfgpu_dbscan();
    cudaError_t e = cudaGetDevice(&db->dev);
    // the highest stream priority: clustering is small latency-bound work
    // that typically runs beside a matched filter's long correlator launch,
    // whose waiting CTAs should not hold it back
    int least = 0, greatest = 0;
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&db->stream, cudaStreamNonBlocking, greatest);
    if (e != cudaSuccess)
    {
        delete db;
        return cuda_fail(e, "mfgpu_dbscan_create");
    }
    *out = db;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_dbscan_destroy(mfgpu_dbscan *db)
try
{
    if (!db) return MFGPU_OK;
    {
        DeviceGuard g(db->dev);
        cudaStreamSynchronize(db->stream);
        db->ws.release();
        cudaStreamDestroy(db->stream);
    }
    delete db;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_dbscan_clear(mfgpu_dbscan *db)
try
{
    if (!db) return fail(MFGPU_EINVAL, "db is NULL");
    db->eps = 3;
    db->min_obs = 5;
    db->init = db->have_data = db->have_labels = db->have_weights = false;
    db->nobs = db->nf = db->ncl = 0;
    db->X.clear(); db->w.clear(); db->labels.clear();
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_dbscan_initialize(mfgpu_dbscan *db, double epsilon, int min_observations)
try
{
    if (!db) return fail(MFGPU_EINVAL, "db is NULL");
    mfgpu_dbscan_clear(db);
    if (epsilon < 0) return fail(MFGPU_EINVAL, "epsilon = " + std::to_string(epsilon) + " must be non-negative");
    if (min_observations < 1)
        return fail(MFGPU_EINVAL, "minObservations = " + std::to_string(min_observations) + " must be positive");
    db->eps = epsilon;
    db->min_obs = min_observations;
    db->init = true;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

static mfgpu_status db_set(mfgpu_dbscan *db, int n_obs, int n_features, const double *X, const double *w)
{
    if (!db) return fail(MFGPU_EINVAL, "db is NULL");
    db->have_data = db->have_labels = db->have_weights = false;
    if (!db->init) return fail(MFGPU_ESTATE, "Class not initialized");
    if (n_obs < 1) return fail(MFGPU_EINVAL, "No observations");
    if (n_features < 1) return fail(MFGPU_EINVAL, "No features");
    if (!X) return fail(MFGPU_EINVAL, "X is NULL");
    if (w)
    {
        double mn = *std::min_element(w, w + n_obs);
        if (!(mn > 0)) return fail(MFGPU_EINVAL, "All weights must be positive");
    }
    db->X.assign(X, X + (size_t) n_obs * n_features);
    if (w) db->w.assign(w, w + n_obs);
    else db->w.clear();
    db->nobs = n_obs;
    db->nf = n_features;
    db->have_weights = w != nullptr;
    db->have_data = true;
    return MFGPU_OK;
}

mfgpu_status mfgpu_dbscan_set_data(mfgpu_dbscan *db, int n_obs, int n_features, const double *X)
try
{
    return db_set(db, n_obs, n_features, X, nullptr);
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_dbscan_set_weighted_data(mfgpu_dbscan *db, int n_obs, int n_features, const double *X,
                                            const double *weights)
try
{
    return db_set(db, n_obs, n_features, X, weights);
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_dbscan_cluster(mfgpu_dbscan *db)
try
{
    if (!db) return fail(MFGPU_EINVAL, "db is NULL");
    db->have_labels = false;
    db->labels.clear();
    if (!db->init) return fail(MFGPU_ESTATE, "Class not initialized");
    if (!db->have_data) return fail(MFGPU_ESTATE, "Data not yet set");
    DeviceGuard g(db->dev);
    int seg[2] = {0, db->nobs};
    db->labels.resize(db->nobs);
    std::string err;
    int rc = run_dbscan(db->nobs, db->nf, db->X.data(), db->have_weights ? db->w.data() : nullptr, db->eps,
                        db->min_obs, 1, seg, db->labels.data(), &db->ncl, db->ws, db->stream, &db->launches, err);
    if (rc != 0) return fail(MFGPU_ECUDA, err);
    db->have_labels = true;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_dbscan_get_number_of_clusters(const mfgpu_dbscan *db, int *n)
try
{
    if (!db || !n) return fail(MFGPU_EINVAL, "NULL argument");
    *n = db->ncl;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_dbscan_get_labels(const mfgpu_dbscan *db, int maxn, int *labels)
try
{
    if (!db) return fail(MFGPU_EINVAL, "db is NULL");
    if (!db->have_labels) return fail(MFGPU_ESTATE, "clustering not yet done");
    if (!labels || maxn < (int) db->labels.size()) return fail(MFGPU_EINVAL, "labels too small");
    std::memcpy(labels, db->labels.data(), sizeof(int) * db->labels.size());
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_dbscan_get_launch_count(const mfgpu_dbscan *db, long long *count)
try
{
    if (!db || !count) return fail(MFGPU_EINVAL, "NULL argument");
    *count = db->launches;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_dbscan_is_initialized(const mfgpu_dbscan *db, int *flag)
try
{
    if (!db || !flag) return fail(MFGPU_EINVAL, "NULL argument");
    *flag = db->init;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_dbscan_have_data(const mfgpu_dbscan *db, int *flag)
try
{
    if (!db || !flag) return fail(MFGPU_EINVAL, "NULL argument");
    *flag = db->have_data;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_dbscan_have_labels(const mfgpu_dbscan *db, int *flag)
try
{
    if (!db || !flag) return fail(MFGPU_EINVAL, "NULL argument");
    *flag = db->have_labels;
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

mfgpu_status mfgpu_dbscan_segmented(mfgpu_dbscan *db, int n_segments, const int *seg_offsets, int n_features,
                                    const double *X, const double *weights, int *labels, int *n_clusters)
try
{
    if (!db) return fail(MFGPU_EINVAL, "db is NULL");
    if (!db->init) return fail(MFGPU_ESTATE, "Class not initialized");
    if (n_segments < 1 || !seg_offsets || !labels || !n_clusters) return fail(MFGPU_EINVAL, "NULL argument");
    if (n_features < 1) return fail(MFGPU_EINVAL, "No features");
    if (seg_offsets[0] != 0) return fail(MFGPU_EINVAL, "seg_offsets[0] must be 0");
    for (int s = 0; s < n_segments; ++s)
        if (seg_offsets[s + 1] < seg_offsets[s]) return fail(MFGPU_EINVAL, "seg_offsets must be non-decreasing");
    const int n = seg_offsets[n_segments];
    if (n > 0 && !X) return fail(MFGPU_EINVAL, "X is NULL");
    if (weights && n > 0)
    {
        double mn = *std::min_element(weights, weights + n);
        if (!(mn > 0)) return fail(MFGPU_EINVAL, "All weights must be positive");
    }
    DeviceGuard g(db->dev);
    std::string err;
    int rc = run_dbscan(n, n_features, X, weights, db->eps, db->min_obs, n_segments, seg_offsets, labels,
                        n_clusters, db->ws, db->stream, &db->launches, err);
    if (rc != 0) return fail(MFGPU_ECUDA, err);
    return MFGPU_OK;
}
catch (...)
{
    return mfgpu::status_of_exception();
}

