/*
 * ref_driver.cpp -- C entry points over the reference's own C++ classes,
 * compiled together with the unchanged reference sources into
 * oracle/_ref/libmflib_ref.so.  TEST INFRASTRUCTURE ONLY: the tests use it
 * to pin the oracle restatement (oracle/mf_oracle.c) against the reference
 * itself and to generate the golden fixtures under tests/golden/.
 *
 * Calls: MFLib::computeOptimalFFTAndBlockLength
 *        (include/mflib/matchedFilterParameters.hpp:208),
 *        MFLib::MatchedFilterParameters::getFFTLength / getBlockLength,
 *        MFLib::MatchedFilter<T> (include/mflib/matchedFilter.hpp:28-178),
 *        MFLib::PeakFinder<T> (include/private/peakFinder.hpp:12-138),
 *        MFLib::SingleChannel::{MatchedFilter, Detector}<T>
 *        (include/mflib/singleChannel/matchedFilter.hpp, detector.hpp).
 */
#include <cstdio>
#include <cstring>
#include <exception>
#include <vector>
#include "mflib/waveformTemplate.hpp"
#include "mflib/matchedFilterParameters.hpp"
#include "mflib/matchedFilter.hpp"
#include "mflib/enums.hpp"
#include "private/peakFinder.hpp"
#include "mflib/networkStationPhase.hpp"
#include "mflib/singleChannel/matchedFilterParameters.hpp"
#include "mflib/singleChannel/matchedFilter.hpp"
#include "mflib/singleChannel/detector.hpp"
#include "mflib/singleChannel/detectorParameters.hpp"
#include "mflib/singleChannel/detectionTimeInterpolationParameters.hpp"
#include "mflib/singleChannel/detection.hpp"
#include "mflib/singleChannel/relativeMagnitude.hpp"

using namespace MFLib;

#define REF_API extern "C" __attribute__((visibility("default")))

REF_API int ref_fft_sizes(int nb, int nx, int *nfft, int *L)
{
    try
    {
        auto r = computeOptimalFFTAndBlockLength(nb, nx);
        *nfft = r.first;
        *L = r.second;
        return 0;
    }
    catch (const std::exception &) { return -1; }
}

/* MatchedFilterParameters::getFFTLength / getBlockLength for one template
 * of nb samples and a signal of nx samples: the window-length rule the
 * parameters object applies (computeWindowLength), not the public
 * function's stricter precondition. */
REF_API int ref_window_length(int nb, int nx, int *nfft, int *L)
{
    try
    {
        std::vector<double> b(nb, 0.0);
        for (int i = 0; i < nb; ++i) b[i] = (double) (i % 7) - 3.0;
        WaveformTemplate wt;
        wt.setSamplingRate(1.0);
        wt.setSignal(nb, b.data());
        MatchedFilterParameters p;
        p.addTemplate(wt);
        p.setSignalSize(nx);
        *nfft = p.getFFTLength();
        *L = p.getBlockLength();
        return 0;
    }
    catch (const std::exception &) { return -1; }
}

/* Runs MatchedFilter<T>; rows of `out` (stride ldo) receive lags
 * 0..n-L_t from getMatchedFilterSignalPointer.  If `stack` is non-null
 * the templates carry onset/travel times and shiftAndStack() is returned
 * in stack (length *nstack). */
template<class T>
static int run_mf(int multi, int nt, const int *lens, const double *const *templates,
                  int n, const T *const *signals, T *out, long ldo,
                  double fs, const double *onsets, const double *travel,
                  const double *weights, int stackAbs, T *stack, int *nstack)
{
    try
    {
        MatchedFilterParameters parms;
        parms.setDetectionMode(multi ? MatchedFilterDetectionMode::MULTI_CHANNEL
                                     : MatchedFilterDetectionMode::SINGLE_CHANNEL);
        parms.setStackAbsoluteValues(stackAbs != 0);
        for (int t = 0; t < nt; ++t)
        {
            WaveformTemplate wt;
            wt.setSignal(lens[t], templates[t]);
            wt.setSamplingRate(fs);
            if (onsets) { wt.setPhaseOnsetTime(onsets[t]); }
            if (travel) { wt.setTravelTime(travel[t]); }
            if (weights) { wt.setShiftAndStackWeight(weights[t]); }
            parms.addTemplate(wt);
        }
        parms.setSignalSize(n);
        // MatchedFilter<float>::clear() frees mSingleSegmentSpectra twice
        // (src/matchedFilter.cpp:372 and :374), which corrupts the heap when
        // a SINGLE_CHANNEL float object is destroyed.  That one object is
        // intentionally leaked here so the reference can still be exercised.
        const bool leak = sizeof(T) == sizeof(float) && !multi;
        MatchedFilter<T> *owned = new MatchedFilter<T>();
        struct Holder
        {
            MatchedFilter<T> *p;
            bool leak;
            ~Holder() { if (!leak) delete p; }
        } holder{owned, leak};
        MatchedFilter<T> &mf = *owned;
        mf.initialize(parms);
        int nsig = multi ? nt : 1;
        for (int s = 0; s < nsig; ++s) { mf.setSignal(s, n, signals[s]); }
        mf.apply();
        for (int t = 0; t < nt; ++t)
        {
            const T *p = mf.getMatchedFilterSignalPointer(t);
            int nv = n - lens[t] + 1;
            for (int k = 0; k < nv; ++k) { out[(size_t) t*ldo + k] = p[k]; }
            for (long k = nv; k < ldo; ++k) { out[(size_t) t*ldo + k] = 0; }
        }
        if (stack)
        {
            auto s = mf.shiftAndStack();
            for (size_t k = 0; k < s.size(); ++k) { stack[k] = s[k]; }
            *nstack = static_cast<int> (s.size());
        }
        return 0;
    }
    catch (const std::exception &e)
    {
        fprintf(stderr, "ref_driver: %s", e.what());
        return -1;
    }
}

REF_API int ref_mf_d(int multi, int nt, const int *lens, const double *const *templates,
                     int n, const double *const *signals, double *out, long ldo)
{
    return run_mf<double>(multi, nt, lens, templates, n, signals, out, ldo, 1.0,
                          nullptr, nullptr, nullptr, 1, nullptr, nullptr);
}

REF_API int ref_mf_f(int multi, int nt, const int *lens, const double *const *templates,
                     int n, const float *const *signals, float *out, long ldo)
{
    return run_mf<float>(multi, nt, lens, templates, n, signals, out, ldo, 1.0,
                         nullptr, nullptr, nullptr, 1, nullptr, nullptr);
}

REF_API int ref_mf_stack_d(int nt, const int *lens, const double *const *templates,
                           int n, const double *const *signals, double *out, long ldo,
                           double fs, const double *onsets, const double *travel,
                           const double *weights, int stackAbs, double *stack, int *nstack)
{
    return run_mf<double>(1, nt, lens, templates, n, signals, out, ldo, fs,
                          onsets, travel, weights, stackAbs, stack, nstack);
}

REF_API int ref_peaks_d(int n, const double *x, double thr, int minDist, int *peaks)
{
    try
    {
        PeakFinder<double> pf;
        pf.setThreshold(thr);
        pf.setMinimumPeakDistance(minDist);
        pf.setSignal(n, x);
        pf.apply();
        int np = pf.getNumberOfPeaks();
        if (np > 0)
        {
            int *ptr = peaks;
            pf.getPeakIndices(np, &ptr);
        }
        return np;
    }
    catch (const std::exception &) { return -1; }
}

REF_API int ref_peaks_f(int n, const float *x, float thr, int minDist, int *peaks)
{
    try
    {
        PeakFinder<float> pf;
        pf.setThreshold(thr);
        pf.setMinimumPeakDistance(minDist);
        pf.setSignal(n, x);
        pf.apply();
        int np = pf.getNumberOfPeaks();
        if (np > 0)
        {
            int *ptr = peaks;
            pf.getPeakIndices(np, &ptr);
        }
        return np;
    }
    catch (const std::exception &) { return -1; }
}

/* SingleChannel::MatchedFilter<T> on one signal, then SingleChannel::
 * Detector<T>::detect; templates carry COMPRESSION polarity and no
 * identifier (so a detection's identifier is the template index).  Up to
 * maxdet detections are returned; the result is the number found or -1.
 * The float matched filter object is not destroyed: the reference's float
 * clear() frees one buffer twice. */
template<class T>
static int run_detect(int nt, const int *lens, const double *const *templates, int n, const T *signal,
                      double fs, double thr, int minDist, int absMax, int single, int interp, int alpha,
                      int npts, int amplitudes, int maxdet, int *o_tmpl, double *o_xc, double *o_time,
                      double *o_itime, int *o_pol, int *o_have, double *o_gr, double *o_sr)
{
    try
    {
        SingleChannel::MatchedFilterParameters parms;
        for (int t = 0; t < nt; ++t)
        {
            WaveformTemplate wt;
            wt.setSignal(lens[t], templates[t]);
            wt.setSamplingRate(fs);
            wt.setPolarity(Polarity::COMPRESSION);
            parms.addTemplate(wt);
        }
        parms.setSignalSize(n);
        auto *mf = new SingleChannel::MatchedFilter<T>();
        mf->initialize(parms);
        mf->setSignal(n, signal);
        mf->apply();
        SingleChannel::DetectorParameters dp;
        dp.setDetectionThreshold(thr);
        dp.setMinimumDetectionSpacing(minDist);
        dp.setMaximaPolicy(absMax ? MaximumMatchedFilterPolicy::ABSOLUTE_MAXIMUM
                                  : MaximumMatchedFilterPolicy::MAXIMUM);
        dp.setMatchedFilteredSignalDetectorPolicy(single ? MatchedFilteredSignalDetectorPolicy::SINGLE
                                                         : MatchedFilteredSignalDetectorPolicy::REDUCED);
        SingleChannel::DetectionTimeInterpolationParameters ip;
        if (interp == 0) { ip.enableLanczos(); }
        else if (interp == 1) { ip.enableQuadratic(); }
        else { ip.disable(); }
        ip.setLanczosAlpha(alpha);
        ip.setLanczosNumberOfInterpolationPoints(npts);
        dp.setDetectionTimeInterpolationParameters(ip);
        if (amplitudes) { dp.enableSaveAmplitudeScalingFactor(); }
        else { dp.disableSaveAmplitudeScalingFactor(); }
        SingleChannel::Detector<T> det;
        det.initialize(dp);
        det.detect(*mf);
        const int nd = det.getNumberOfDetections();
        for (int i = 0; i < nd && i < maxdet; ++i)
        {
            auto d = det.getDetection(i);
            o_tmpl[i] = (int) d.getTemplateIdentifier().second;
            o_xc[i] = d.getCorrelationCoefficient();
            o_time[i] = d.getDetectionTime();
            o_itime[i] = d.getInterpolatedDetectionTime();
            o_pol[i] = (int) d.getPolarity();
            const bool h = d.haveAmplitudeScalingFactor(RelativeMagnitudeType::GIBBONS_RINGDAL_2006);
            o_have[i] = h ? 1 : 0;
            o_gr[i] = h ? (double) d.getAmplitudeScalingFactor(RelativeMagnitudeType::GIBBONS_RINGDAL_2006) : 0.0;
            o_sr[i] = h ? (double) d.getAmplitudeScalingFactor(RelativeMagnitudeType::SCHAFF_RICHARDS_2014) : 0.0;
        }
        if (sizeof(T) == 8) { delete mf; }
        return nd;
    }
    catch (const std::exception &e)
    {
        fprintf(stderr, "ref_detect: %s\n", e.what());
        return -1;
    }
}

REF_API int ref_detect_d(int nt, const int *lens, const double *const *templates, int n, const double *signal,
                         double fs, double thr, int minDist, int absMax, int single, int interp, int alpha,
                         int npts, int amplitudes, int maxdet, int *o_tmpl, double *o_xc, double *o_time,
                         double *o_itime, int *o_pol, int *o_have, double *o_gr, double *o_sr)
{
    return run_detect<double>(nt, lens, templates, n, signal, fs, thr, minDist, absMax, single, interp, alpha, npts,
                              amplitudes, maxdet, o_tmpl, o_xc, o_time, o_itime, o_pol, o_have, o_gr, o_sr);
}

REF_API int ref_detect_f(int nt, const int *lens, const double *const *templates, int n, const float *signal,
                         double fs, double thr, int minDist, int absMax, int single, int interp, int alpha,
                         int npts, int amplitudes, int maxdet, int *o_tmpl, double *o_xc, double *o_time,
                         double *o_itime, int *o_pol, int *o_have, double *o_gr, double *o_sr)
{
    return run_detect<float>(nt, lens, templates, n, signal, fs, thr, minDist, absMax, single, interp, alpha, npts,
                             amplitudes, maxdet, o_tmpl, o_xc, o_time, o_itime, o_pol, o_have, o_gr, o_sr);
}

/* RelativeMagnitude<double> of one window y against template b (both L
 * samples): the two amplitude scaling factors; -1 if the reference throws. */
REF_API int ref_relmag_d(int L, const double *b, const double *y, double *gr, double *sr)
{
    try
    {
        WaveformTemplate wt;
        wt.setSignal(L, b);
        wt.setSamplingRate(100.0);
        SingleChannel::RelativeMagnitude<double> rm;
        rm.initialize(wt);
        rm.setDetectedSignal(L, y);
        *gr = rm.computeAmplitudeScalingFactor(RelativeMagnitudeType::GIBBONS_RINGDAL_2006);
        *sr = rm.computeAmplitudeScalingFactor(RelativeMagnitudeType::SCHAFF_RICHARDS_2014);
        return 0;
    }
    catch (const std::exception &) { return -1; }
}
