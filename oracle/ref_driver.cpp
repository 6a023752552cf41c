/*
 * ref_driver.cpp -- C entry points over the reference's own C++ classes,
 * compiled together with the unchanged reference sources into
 * oracle/_ref/libmflib_ref.so.  TEST INFRASTRUCTURE ONLY: the tests use it
 * to pin the oracle restatement (oracle/mf_oracle.c) against the reference
 * itself and to generate the golden fixtures under tests/golden/.
 *
 * Calls: MFLib::computeOptimalFFTAndBlockLength
 *        (include/mflib/matchedFilterParameters.hpp:208),
 *        MFLib::MatchedFilter<T> (include/mflib/matchedFilter.hpp:28-178),
 *        MFLib::PeakFinder<T> (include/private/peakFinder.hpp:12-138).
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
