/*
 * mfgpu.h -- C ABI of the GB300 matched-filtering library (libmfgpu.so).
 *
 * The library is a drop-in for mflib's matched-filtering hot path: every
 * entry point below replaces one method of the reference's C++ classes,
 * cited as file:line within the mflib project.  Plain pointers and sizes
 * only; no exception crosses this boundary.  Every function returns an
 * mfgpu_status; on failure mfgpu_last_error() holds a message for the
 * calling thread.  MFGPU_EINVAL maps to the reference's
 * std::invalid_argument, MFGPU_ESTATE to std::runtime_error.
 *
 * Threading: an object (matched filter, peak finder, DBSCAN) is used by one
 * host thread at a time, like the reference classes.  Each object owns its
 * own CUDA stream on the current device.  All host buffers passed in are
 * copied (the reference copies every input, e.g. src/matchedFilter.cpp:896-904).
 *
 * Sample type: a matched filter or peak finder is created for
 * MFGPU_FLOAT32 or MFGPU_FLOAT64 (MFLib::MatchedFilter<float|double>);
 * `const void *` sample arguments point at that type.
 */
#ifndef MFGPU_H
#define MFGPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum
{
    MFGPU_OK = 0,
    MFGPU_EINVAL = 1,   /* invalid argument   (reference: std::invalid_argument) */
    MFGPU_ESTATE = 2,   /* invalid state      (reference: std::runtime_error)    */
    MFGPU_ENOMEM = 3,   /* device or pinned host allocation failed               */
    MFGPU_ECUDA = 4,    /* CUDA runtime error                                    */
    MFGPU_ETIMEOUT = 5  /* a bounded device-side wait gave up                    */
} mfgpu_status;

enum { MFGPU_FLOAT32 = 4, MFGPU_FLOAT64 = 8 };

/* MFLib::MatchedFilterDetectionMode, include/mflib/enums.hpp:24-32 */
enum { MFGPU_SINGLE_CHANNEL = 0, MFGPU_MULTI_CHANNEL = 1 };

/* Message for the last failed call on this thread ("" if none). */
const char *mfgpu_last_error(void);

/* Library version (major*10000 + minor*100 + patch). */
int mfgpu_version(void);

/* Number of visible CUDA devices (0 when none). */
mfgpu_status mfgpu_device_count(int *count);

/* MFLib::computeOptimalFFTAndBlockLength(nb, nx),
 * include/mflib/matchedFilterParameters.hpp:208, src/matchedFilterParameters.cpp:371-385.
 * Returns the reference's FFT length and overlap-add block length. */
mfgpu_status mfgpu_fft_sizes(int nb, int nx, int *fft_length, int *block_length);

/* MFLib::MatchedFilterParameters::getFFTLength / getBlockLength for a longest
 * template of nb samples and a signal of nx (src/matchedFilterParameters.cpp:268-300,
 * computeWindowLength :47-104): the same search as mfgpu_fft_sizes, an error
 * only when nb > nx (a signal as long as the template is accepted). */
mfgpu_status mfgpu_window_length(int nb, int nx, int *fft_length, int *block_length);

/* ------------------------------------------------------------------------ */
/* Matched filter: MFLib::MatchedFilter<T> (include/mflib/matchedFilter.hpp:28-178)
 * and its SINGLE_CHANNEL facade MFLib::SingleChannel::MatchedFilter<T>
 * (include/mflib/singleChannel/matchedFilter.hpp). */
typedef struct mfgpu_mf mfgpu_mf;

/* Everything MatchedFilter<T>::initialize reads from MatchedFilterParameters
 * (src/matchedFilter.cpp:507-593): templates (FP64 samples, as stored by
 * WaveformTemplate), signal size, detection mode, and the per-template
 * shift/weight that shiftAndStack uses (:577-592). */
typedef struct
{
    int detection_mode;             /* MFGPU_SINGLE_CHANNEL or MFGPU_MULTI_CHANNEL */
    int n_templates;                /* >= 1 */
    const int *template_lengths;    /* [n_templates], each >= 1 */
    const double *const *templates; /* [n_templates] pointers to FP64 samples */
    int signal_size;                /* samples per signal, >= 1 */
    /* shift-and-stack inputs, may be NULL: the reference stacks only when
       every template has an onset and a travel time (:581-592) */
    const int *stack_shifts;        /* round((travel - onset) * fs) per template */
    const double *stack_weights;    /* per template weight in [0,1] */
    int stack_absolute_values;      /* MatchedFilterParameters::getStackAbsoluteValues */
    /* Extension (no reference counterpart): share one signal between
       several templates.  n_channels = 0 keeps the reference layout (one
       signal per template in MULTI_CHANNEL, one signal in SINGLE_CHANNEL).
       Otherwise template t reads channel template_channel[t]. */
    int n_channels;
    const int *template_channel;
    /* Extension: FFT length for the overlap-save blocks; 0 = autotune. */
    int fft_length;
    /* Extension: correlator organisation; 0 = automatic, 1 = whole CTA per
       transform, 2 = whole CTA with the next spectrum prefetched by TMA,
       3 = two 128-thread teams per CTA (templates of one length only),
       4 = split-precision (FP16 hi+lo) time-domain correlation on the tensor
       cores (FP32 data, templates of one length), 5 = two teams with the
       normalisation computed inside each CTA instead of by a separate
       per-channel pass (templates of one length), 6 = two 256-thread teams
       in a 512-thread CTA, each normalising its own templates (FP32 data,
       templates of several lengths). */
    int correlator_variant;
    /* Extension: templates of several lengths are split by length into at
       most this many buckets, each with its own FFT length and block length
       (0 = automatic: at most 3, a split must save more than a launch;
       1 = one plan for every template; k > 1: at most k, split wherever the
       plans get cheaper). */
    int length_buckets;
    /* Extension: per-bucket plan overrides, e.g. from a measured autotune.
       Entry b applies to length bucket b (shortest templates first, as
       mfgpu_mf_get_buckets reports them); entries past the bucket count are
       ignored.  bucket_fft_lengths[b]: the bucket's FFT length (0 =
       automatic); bucket_variants[b]: its correlator organisation numbered
       like correlator_variant (0 = automatic; 1, 2 or (FP32) 6 when the
       templates have several lengths, 1, 2, 3 or 5 for one length).  Either array may be
       NULL when n_bucket_plans is 0.  An override whose plan does not fit
       (block too short, shared memory, unsupported length) fails with
       MFGPU_EINVAL.  Any non-zero entry turns off the automatic choice of
       the tensor-core correlator. */
    int n_bucket_plans;
    const int *bucket_fft_lengths;
    const int *bucket_variants;
    /* Extension: 1 = run the FFT correlator as one persistent launch whose
       CTAs take (template group, signal block) tiles from a device ticket
       instead of a static grid (FP32, two-team organisations 3 and 6, FFT
       length >= 4096; ignored otherwise).  0 = the static grid, which
       measured faster on GB300. */
    int persistent;
    /* Extension: 1 = the tensor-core correlator splits its operands into
       BF16 hi + lo (about 16 bits of each FP32 value kept, no range
       scaling needed) instead of FP16 hi + lo (22 bits).  The accuracy
       fix-up's bound grows with the templates' largest coefficient
       (independent roundings summed over the window), so more runs are
       recomputed than with FP16.  0 = FP16. */
    int tc_bf16;
    /* Extension: the tensor-core correlator's tile shape, as templates per
       group Gp (the MMA's N = 16 Gp: the hi and lo columns of each): an even
       number in [2, 16] that fits the shared memory beside the strips for
       the templates' padded length (MFGPU_EINVAL otherwise); 0 = automatic
       (the most that fit, balanced over the busiest channel). */
    int tc_group;
} mfgpu_mf_params;

/* MatchedFilter<T>::MatchedFilter(); precision MFGPU_FLOAT32 | MFGPU_FLOAT64 */
mfgpu_status mfgpu_mf_create(int precision, mfgpu_mf **mf);
/* ~MatchedFilter() */
mfgpu_status mfgpu_mf_destroy(mfgpu_mf *mf);
/* MatchedFilter<T>::initialize, src/matchedFilter.cpp:507-821.  Like the
 * reference (which sizes its FFT up to 2^21, src/matchedFilterParameters.cpp:54-64)
 * any template length is accepted: templates longer than the largest
 * overlap-save plan takes (FP32: 8,161 samples, FP64: 4,065) are correlated
 * directly in the time domain (two-pass Pearson per lag, cost proportional to
 * the template length per lag), beside the FFT plan of the others.  The direct
 * correlator keeps L + 31 samples per warp in shared memory, which bounds L
 * at about 57,000 samples (FP32) or 27,900 (FP64); longer templates fail
 * with MFGPU_EINVAL. */
mfgpu_status mfgpu_mf_initialize(mfgpu_mf *mf, const mfgpu_mf_params *params);
/* MatchedFilter<T>::clear, src/matchedFilter.cpp:501-504 */
mfgpu_status mfgpu_mf_clear(mfgpu_mf *mf);
/* MatchedFilter<T>::isInitialized, src/matchedFilter.cpp:1367-1371 */
mfgpu_status mfgpu_mf_is_initialized(const mfgpu_mf *mf, int *flag);
/* MatchedFilter<T>::getNumberOfTemplates, src/matchedFilter.cpp:1374-1382 */
mfgpu_status mfgpu_mf_get_number_of_templates(const mfgpu_mf *mf, int *n);
/* MatchedFilter<T>::getSignalLength, src/matchedFilter.cpp:1385-1393 */
mfgpu_status mfgpu_mf_get_signal_length(const mfgpu_mf *mf, int *n);
/* MatchedFilter<T>::getFilteredSignalLength (n - maxLen + 1), src/matchedFilter.cpp:1396-1402 */
mfgpu_status mfgpu_mf_get_filtered_signal_length(const mfgpu_mf *mf, int *n);
/* MatchedFilter<T>::setSignal(it, n, x) (host samples), src/matchedFilter.cpp:863-921.
 * MULTI_CHANNEL: signal of template `it`; SINGLE_CHANNEL: it must be 0
 * (SingleChannel::MatchedFilter::setSignal, src/singleChannel/matchedFilter.cpp:62-67). */
mfgpu_status mfgpu_mf_set_signal(mfgpu_mf *mf, int it, int n, const void *x);
/* MatchedFilter<T>::zeroSignal, src/matchedFilter.cpp:824-845 */
mfgpu_status mfgpu_mf_zero_signal(mfgpu_mf *mf, int it);
/* MatchedFilter<T>::getSignalPointer, src/matchedFilter.cpp:924-938: copies the
 * stored signal of `it` (n samples) to host memory `dst` (capacity maxn). */
mfgpu_status mfgpu_mf_get_signal(const mfgpu_mf *mf, int it, int maxn, void *dst);
/* MatchedFilter<T>::apply, src/matchedFilter.cpp:972-1316.  Enqueues the
 * work on the object's stream; getters synchronise. */
mfgpu_status mfgpu_mf_apply(mfgpu_mf *mf);
/* MatchedFilter<T>::haveMatchedFilteredSignals, src/matchedFilter.cpp:1405-1409 */
mfgpu_status mfgpu_mf_have_matched_filtered_signals(const mfgpu_mf *mf, int *flag);
/* MatchedFilter<T>::getMatchedFilteredSignal, src/matchedFilter.cpp:941-948:
 * copies the first getFilteredSignalLength() coefficients of template `it`
 * into `dst` (capacity maxn); *nout receives the count. */
mfgpu_status mfgpu_mf_get_matched_filtered_signal(mfgpu_mf *mf, int it, int maxn, void *dst, int *nout);
/* MatchedFilter<T>::shiftAndStack, src/matchedFilter.cpp:1319-1364 */
mfgpu_status mfgpu_mf_shift_and_stack(mfgpu_mf *mf, int maxn, void *dst, int *nout);
/* MatchedFilter<T>::getSpectraOfTemplate, src/matchedFilter.cpp:1412-1431: the
 * reference's debug view, rfft of the reversed, demeaned, unit-norm template
 * at the reference's FFT length (computed on the device on request);
 * dst holds 2*(nfft/2+1) interleaved re/im values of the object's type. */
mfgpu_status mfgpu_mf_get_spectra_of_template(mfgpu_mf *mf, int it, int maxn, void *dst, int *nout);

/* Extensions (no reference counterpart) --------------------------------- */
/* Signal of channel c (n_channels > 0 layout), host samples. */
mfgpu_status mfgpu_mf_set_channel_signal(mfgpu_mf *mf, int channel, int n, const void *x);
/* Signals of channels [first_channel, first_channel + n_channels) from one
 * host array: row r (n samples) starts at x + r * ld samples.  One copy and
 * one dead-trace pass for all rows; returns when the rows are copied. */
mfgpu_status mfgpu_mf_set_channel_signals(mfgpu_mf *mf, int first_channel, int n_channels, int n, const void *x,
                                          long ld);
/* Asynchronous upload of every channel's signal (row c of x, n samples,
 * row stride ld samples) for the NEXT apply: the copy runs on a separate
 * stream into a second device buffer, so it overlaps the work already
 * enqueued (the current apply, peak finding), and the results of the
 * previous apply stay readable.  The next apply -- or any call that reads
 * or writes the signals -- makes the staged signals current.  Unlike the
 * reference's copying setters, x must stay valid and unchanged until the
 * copy has finished: until a result of that next apply has been read (a
 * getter or find_peaks after it), or until mfgpu_mf_synchronize; pinned host
 * memory makes the copy DMA. */
mfgpu_status mfgpu_mf_stage_channel_signals(mfgpu_mf *mf, int n, const void *x, long ld);
/* Signal of channel c from device memory (same type, n samples). */
mfgpu_status mfgpu_mf_set_channel_signal_device(mfgpu_mf *mf, int channel, int n, const void *dx);
/* Full valid coefficient range of template it: lags 0..n-L_t (n - L_t + 1
 * values), host copy. */
mfgpu_status mfgpu_mf_get_valid_signal(mfgpu_mf *mf, int it, int maxn, void *dst, int *nout);
/* Device pointer to template it's coefficients (lag k at p[k]) and the
 * number of valid lags; valid until the next apply/initialize/clear. */
mfgpu_status mfgpu_mf_get_device_signal(mfgpu_mf *mf, int it, const void **dptr, int *nvalid);
/* Overlap-save plan chosen at initialize. */
mfgpu_status mfgpu_mf_get_plan(const mfgpu_mf *mf, int *fft_length, int *lags_per_block, int *n_blocks);
/* Correlator organisation chosen at initialize, numbered like
 * correlator_variant (1-3, 5 and 6 FFT organisations, 4 tensor cores); for the
 * tensor-core path also the templates per group and the padded K, else 0.
 * Extension: the reference has one CPU correlator and no such query. */
mfgpu_status mfgpu_mf_get_correlator(const mfgpu_mf *mf, int *variant, int *tc_group, int *tc_k);
/* Length buckets chosen at initialize: their number, and for each (up to
 * max, shortest templates first, the primary plan last) the FFT length and
 * the number of templates (templates correlated directly in the time domain
 * belong to no bucket).  Extension: the reference has one FFT length. */
mfgpu_status mfgpu_mf_get_buckets(const mfgpu_mf *mf, int max, int *fft_lengths, int *n_templates, int *count);
/* Per length bucket (same order, up to max): lags per block and the FFT
 * organisation numbered like correlator_variant (4 for the tensor-core
 * correlator, which has one bucket).  Extension. */
mfgpu_status mfgpu_mf_get_bucket_plans(const mfgpu_mf *mf, int max, int *lags_per_block, int *variants, int *count);
/* Request-window upload for a serving loop.  Extension: the reference sets
 * whole-length signals one template at a time (setSignal,
 * src/matchedFilter.cpp:863-921) and has no serving loop.  x holds n_src
 * channel rows (row stride ld samples) of n <= signal-length samples; every
 * channel c of the object receives row c % n_src, zero-filled from n to the
 * signal length; dead-trace flags are decided over the first n samples.
 * Coefficients at lags k <= n - L_t use window samples only.  Copies before
 * returning, like setSignal. */
mfgpu_status mfgpu_mf_set_window(mfgpu_mf *mf, int n_src, int n, const void *x, long ld);
/* ---- Device ring of recent samples per channel.  No reference
 * counterpart: a serving loop keeps each station channel's latest samples
 * on the device, appends only the new samples, and sets a request's window
 * from the ring by a device gather instead of uploading the window from the
 * host.  Sample s (counted from the first append) of channel c lives at
 * c * capacity + s mod capacity; the last `capacity` samples are kept.
 * Appends and window reads of one ring are serialised by the ring. */
typedef struct mfgpu_ring mfgpu_ring;
/* precision MFGPU_FLOAT32 | MFGPU_FLOAT64 (that of the objects it feeds);
 * n_channels rows of capacity samples, zeroed, on the current device */
mfgpu_status mfgpu_ring_create(int precision, int n_channels, long capacity, mfgpu_ring **ring);
mfgpu_status mfgpu_ring_destroy(mfgpu_ring *ring);
/* Appends n samples to every channel from host rows with stride ld (ld is
 * ignored for one channel); copies before returning.  Of a chunk longer
 * than the capacity only its last capacity samples are kept. */
mfgpu_status mfgpu_ring_append(mfgpu_ring *ring, int n, const void *x, long ld);
/* Samples appended per channel so far (the end of the newest window). */
mfgpu_status mfgpu_ring_get_head(mfgpu_ring *ring, long long *appended);
/* mfgpu_mf_set_window with the window read from a ring: samples
 * [end - n, end) of ring channels channels[0 .. n_src) (NULL: 0 .. n_src-1)
 * become the object's source rows; the window must still be in the ring
 * (end <= head, end - n >= head - capacity) and n_src <= 256.  Same
 * precision and device as the object; waits for the gather. */
mfgpu_status mfgpu_mf_set_window_ring(mfgpu_mf *mf, mfgpu_ring *ring, int n_src, const int *channels,
                                      long long end, int n);
/* Device bytes the object holds (its buffers and peak-finder scratch), for
 * admission against a memory budget.  Extension: no reference counterpart. */
mfgpu_status mfgpu_mf_get_device_bytes(const mfgpu_mf *mf, unsigned long long *bytes);
/* ---- single-channel detector (MFLib::SingleChannel::Detector<T>,
 * src/singleChannel/detector.cpp:419-691) over the last apply's traces. */
typedef struct
{
    double threshold;       /* DetectorParameters::setDetectionThreshold, clamped to [0, 1] */
    int min_distance;       /* setMinimumDetectionSpacing (samples) */
    int absolute_maximum;   /* MaximumMatchedFilterPolicy: 0 MAXIMUM, 1 ABSOLUTE_MAXIMUM */
    int single;             /* MatchedFilteredSignalDetectorPolicy: 0 REDUCED, 1 SINGLE */
    int interpolation;      /* DetectionTimeInterpolationType: 0 LANCZOS, 1 QUADRATIC, 2 NONE */
    int lanczos_alpha;      /* DetectionTimeInterpolationParameters (51) */
    int lanczos_points;     /* (100) */
    double sampling_rate;   /* of the templates, Hz */
    int amplitudes;         /* wantAmplitudeScalingFactor */
} mfgpu_detect_params;

typedef struct
{
    int template_index;
    int sample;                   /* lag of the detection */
    double correlation;           /* the template's coefficient there, clamped to [-1, 1] */
    double detection_time;        /* sample / sampling_rate */
    double interpolated_time;     /* detection_time + refinement */
    int sign;                     /* sign of the coefficient (-1, 0, 1): polarity factor */
    int have_amplitude;
    double gibbons_ringdal;       /* amplitude scaling factors of the detected window */
    double schaff_richards;
} mfgpu_detection;

/* Detector::detect: reduce (REDUCED) or keep (SINGLE) the traces, PeakFinder,
 * then per detection the refined time, polarity factor and amplitudes; the
 * detections stay in the object (REDUCED: lag order; SINGLE: by time, then
 * template). */
mfgpu_status mfgpu_mf_detect(mfgpu_mf *mf, const mfgpu_detect_params *params, int *n_detections);
/* Copies up to max detections of the last mfgpu_mf_detect. */
mfgpu_status mfgpu_mf_get_detections(mfgpu_mf *mf, int max, mfgpu_detection *out, int *n);
/* Replay apply as a CUDA graph (extension, no reference counterpart):
 * with enable != 0, the second apply with the same input buffer and
 * peak-gathering setup captures the stream work (events, normalisation,
 * correlators) into a graph, and later applies with that setup launch it;
 * staged uploads alternate between two captured graphs.  Results are those
 * of the direct launches.  Call it outside any stream capture. */
mfgpu_status mfgpu_mf_set_graph(mfgpu_mf *mf, int enable);
/* Number of applies launched as graphs so far. */
mfgpu_status mfgpu_mf_get_graph_launches(const mfgpu_mf *mf, long long *count);
/* Relative amplitudes of detected windows against one template:
 * RelativeMagnitude<T>::computeAmplitudeScalingFactor
 * (src/singleChannel/relativeMagnitude.cpp:35-130, :334-372) for a batch of
 * n_windows host windows of L samples (row stride ld, precision
 * MFGPU_FLOAT32 | MFGPU_FLOAT64): gr = GIBBONS_RINGDAL_2006 = |<b, y>| /
 * <b, b>, sr = SCHAFF_RICHARDS_2014 = sqrt(<y, y> / <b, b>) of the demeaned
 * template b (FP64) and window y, in double; valid[w] = 0 for a constant
 * window (the reference throws there).  Extension: the reference takes one
 * window per call. */
mfgpu_status mfgpu_relative_amplitudes(int precision, int L, const double *templ, int n_windows, const void *windows,
                                       long ld, double *gr, double *sr, int *valid);
/* Block until the object's streams are idle (work and staged uploads);
 * reports device-side errors.  Result getters and find_peaks wait for the
 * work only: a staged upload in flight feeds the next apply. */
mfgpu_status mfgpu_mf_synchronize(mfgpu_mf *mf);
/* Device time (ms) of the last apply's correlation kernel and of the whole
 * apply (correlation + dead-trace checks), measured with CUDA events on
 * the object's stream. */
mfgpu_status mfgpu_mf_get_last_timings(mfgpu_mf *mf, float *xcorr_ms, float *apply_ms);
/* Number of kernel launches issued by the object since it was created. */
mfgpu_status mfgpu_mf_get_launch_count(const mfgpu_mf *mf, long long *count);
/* No reference counterpart.  FP32 objects: the number of 32-lag runs (per
 * channel row) that the last apply recomputed by direct correlation because
 * the chosen correlator's rounding-error bound exceeded 2e-5 of the run's
 * quietest window (windows or FFT blocks that straddle amplitude changes of
 * several decades); 0 for FP64 objects.  Waits for the apply. */
mfgpu_status mfgpu_mf_get_fixup_runs(mfgpu_mf *mf, long long *runs);
/* No reference counterpart; for tests of the bounded device waits.  The
 * next apply's FFT correlator expects its segment copy without issuing it
 * (no copy is in flight) and gives up after a short bounded wait: that apply
 * fails with MFGPU_ETIMEOUT at the next synchronising call, which also clears
 * the device status word, and later applies run normally.  The apply is not
 * captured into a CUDA graph.  MFGPU_EINVAL for the tensor-core correlator. */
mfgpu_status mfgpu_mf_test_wait_timeout(mfgpu_mf *mf);
/* No reference counterpart; for measuring a correlator's raw rounding
 * error.  skip = 1: later applies of an FP32 object still flag the runs
 * whose error bound exceeds the tolerance (mfgpu_mf_get_fixup_runs counts
 * them) but do not recompute them, so the coefficients carry the chosen
 * correlator's own error; skip = 0 restores the fix-up.  Waits for the
 * object's work and drops its captured CUDA graphs. */
mfgpu_status mfgpu_mf_test_skip_fixup(mfgpu_mf *mf, int skip);
/* The object's CUDA stream (a cudaStream_t), on which every launch and
 * copy of the object is issued; for event timing by the caller. */
mfgpu_status mfgpu_mf_get_stream(const mfgpu_mf *mf, void **stream);

/* Batched peak finding on the device over every template's coefficients
 * (PeakFinder<T>::apply, src/peakFinder.cpp:329-446, applied per template
 * as SingleChannel::Detector does, src/singleChannel/detector.cpp:466-489).
 * trace_length: lags searched per template; 0 = getFilteredSignalLength().
 * Results stay on the device; read them with mfgpu_mf_get_peaks. */
mfgpu_status mfgpu_mf_find_peaks(mfgpu_mf *mf, double threshold, int min_distance, int trace_length);
/* Extension (no reference counterpart): from the next apply on, the
 * correlator also gathers the peak candidates above `threshold` of the
 * default trace length, and a find_peaks with the same
 * threshold and the default trace length uses them instead of scanning the
 * stored coefficients again.  The peaks are identical either way.  A
 * negative threshold turns the gathering off (the default). */
mfgpu_status mfgpu_mf_set_peak_threshold(mfgpu_mf *mf, double threshold);
/* Requested gathering threshold (negative: off) and whether the last apply
 * gathered candidates (active = 1). */
mfgpu_status mfgpu_mf_get_peak_threshold(const mfgpu_mf *mf, double *threshold, int *active);
/* Peaks of template it (ascending lag indices). */
mfgpu_status mfgpu_mf_get_peaks(mfgpu_mf *mf, int it, int maxn, int *dst, int *nout);
/* Total peaks over all templates, and all of them at once: counts[nt] and
 * indices[sum counts] (template-major, ascending within a template).
 * indices == NULL with max_total == 0 only fills counts and *total. */
mfgpu_status mfgpu_mf_get_all_peaks(mfgpu_mf *mf, int nt, int *counts, int max_total, int *indices,
                                    int *total);

/* ------------------------------------------------------------------------ */
/* Peak finder: MFLib::PeakFinder<T> (include/private/peakFinder.hpp:12-138). */
typedef struct mfgpu_peaks mfgpu_peaks;
mfgpu_status mfgpu_peaks_create(int precision, mfgpu_peaks **pf);
mfgpu_status mfgpu_peaks_destroy(mfgpu_peaks *pf);
/* PeakFinder<T>::setThreshold (must be in [0,1]), src/peakFinder.cpp:226-235 */
mfgpu_status mfgpu_peaks_set_threshold(mfgpu_peaks *pf, double threshold);
mfgpu_status mfgpu_peaks_get_threshold(const mfgpu_peaks *pf, double *threshold);
/* PeakFinder<T>::setMinimumPeakDistance, src/peakFinder.cpp:251-256 */
mfgpu_status mfgpu_peaks_set_minimum_peak_distance(mfgpu_peaks *pf, int min_distance);
mfgpu_status mfgpu_peaks_get_minimum_peak_distance(const mfgpu_peaks *pf, int *min_distance);
/* PeakFinder<T>::setSignal (host samples, n >= 1), src/peakFinder.cpp:260-283 */
mfgpu_status mfgpu_peaks_set_signal(mfgpu_peaks *pf, int n, const void *x);
/* PeakFinder<T>::apply, src/peakFinder.cpp:329-446 */
mfgpu_status mfgpu_peaks_apply(mfgpu_peaks *pf);
/* PeakFinder<T>::getNumberOfPeaks, src/peakFinder.cpp:287-290 */
mfgpu_status mfgpu_peaks_get_number_of_peaks(const mfgpu_peaks *pf, int *n);
/* PeakFinder<T>::getPeakIndices, src/peakFinder.cpp:294-311 */
mfgpu_status mfgpu_peaks_get_peak_indices(const mfgpu_peaks *pf, int maxn, int *dst);
/* PeakFinder<T>::clear */
mfgpu_status mfgpu_peaks_clear(mfgpu_peaks *pf);

/* ------------------------------------------------------------------------ */
/* DBSCAN: MFLib::DBSCAN (include/private/dbscan.hpp:10-132). */
typedef struct mfgpu_dbscan mfgpu_dbscan;
mfgpu_status mfgpu_dbscan_create(mfgpu_dbscan **db);
mfgpu_status mfgpu_dbscan_destroy(mfgpu_dbscan *db);
/* DBSCAN::initialize(epsilon >= 0, minObservations >= 1), src/dbscan.cpp:95-112 */
mfgpu_status mfgpu_dbscan_initialize(mfgpu_dbscan *db, double epsilon, int min_observations);
/* DBSCAN::setData, src/dbscan.cpp:115-138: row-major [n_obs x n_features] */
mfgpu_status mfgpu_dbscan_set_data(mfgpu_dbscan *db, int n_obs, int n_features, const double *X);
/* DBSCAN::setWeightedData, src/dbscan.cpp:141-184: weights > 0 or NULL */
mfgpu_status mfgpu_dbscan_set_weighted_data(mfgpu_dbscan *db, int n_obs, int n_features, const double *X,
                                            const double *weights);
/* DBSCAN::cluster, src/dbscan.cpp:187-214 */
mfgpu_status mfgpu_dbscan_cluster(mfgpu_dbscan *db);
/* DBSCAN::getNumberOfClusters, src/dbscan.cpp:229-232 */
mfgpu_status mfgpu_dbscan_get_number_of_clusters(const mfgpu_dbscan *db, int *n);
/* DBSCAN::getLabels, src/dbscan.cpp:235-239 (-1 = noise) */
mfgpu_status mfgpu_dbscan_get_labels(const mfgpu_dbscan *db, int maxn, int *labels);
/* Extension: number of kernel launches issued by the object so far. */
mfgpu_status mfgpu_dbscan_get_launch_count(const mfgpu_dbscan *db, long long *count);
mfgpu_status mfgpu_dbscan_is_initialized(const mfgpu_dbscan *db, int *flag);
mfgpu_status mfgpu_dbscan_have_data(const mfgpu_dbscan *db, int *flag);
mfgpu_status mfgpu_dbscan_have_labels(const mfgpu_dbscan *db, int *flag);
mfgpu_status mfgpu_dbscan_clear(mfgpu_dbscan *db);

/* Segmented DBSCAN (extension): n_segments independent problems in one
 * launch sequence, as SingleChannel::Associator::associate runs one DBSCAN
 * per template id (src/singleChannel/associator.cpp:192-264).  Observations
 * of segment s are rows seg_offsets[s]..seg_offsets[s+1]-1; labels are
 * numbered per segment; n_clusters[s] receives each segment's count.
 * weights may be NULL. */
mfgpu_status mfgpu_dbscan_segmented(mfgpu_dbscan *db, int n_segments, const int *seg_offsets, int n_features,
                                    const double *X, const double *weights, int *labels, int *n_clusters);

/* Segmented DBSCAN without any device allocation.  No counterpart in the
 * reference: it serves callers that cannot call cudaMalloc -- a host
 * framework that has reserved all device memory for its own pools, or a
 * real-time pipeline that must not allocate or free (and so synchronise the
 * device) after start-up.  Same semantics as mfgpu_dbscan_segmented, but
 * every pointer is DEVICE memory supplied by the caller (X [n_obs x
 * n_features] FP64 row-major, weights or NULL, seg_offsets [n_segments+1]
 * with seg_offsets[0] = 0 and seg_offsets[n_segments] = n_obs, labels
 * [n_obs], n_clusters [n_segments]) and the work is enqueued on `stream`
 * (a cudaStream_t, NULL = default stream); the caller synchronises.
 * Working memory is a fixed file-scope device array sized for at most
 * MFGPU_DBSCAN_NOALLOC_MAX_OBS observations and
 * MFGPU_DBSCAN_NOALLOC_MAX_SEGMENTS segments (about 2.4 MB, held on every
 * device that loads the library until the process exits; with one feature
 * the segments are sorted there on the device, so each point visits its
 * neighbours only); larger requests
 * fail with MFGPU_EINVAL.  Every call looks up the array's device address
 * in the current context (no allocation); the first call in a context also
 * loads the module that places the array, so make that first call before
 * any stream capture.  All calls share the array: calls that overlap on the
 * GPU race, so the caller must serialise them.
 * Unchecked on the device (the call does not wait for the GPU): weights
 * must be > 0 as the reference requires (src/dbscan.cpp:152-158), and
 * malformed seg_offsets (first not 0, decreasing, last not n_obs) are
 * clamped into a valid partition of [0, n_obs) instead of rejected.
 * n_obs = 0 writes zero clusters for every segment. */
#define MFGPU_DBSCAN_NOALLOC_MAX_OBS 65536
#define MFGPU_DBSCAN_NOALLOC_MAX_SEGMENTS 4096
mfgpu_status mfgpu_dbscan_segmented_noalloc(int n_segments, const int *seg_offsets, int n_obs, int n_features,
                                            const double *X, const double *weights, double epsilon,
                                            int min_observations, int *labels, int *n_clusters, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* MFGPU_H */
