/*
 * mfgpu.hpp -- mflib's C++ classes (namespace MFLib) over the C ABI of
 * libmfgpu (mfgpu.h), header-only: link with -lmfgpu.
 *
 * Same class and method names, argument meaning and exception types as the
 * reference headers, so code written against mflib compiles unchanged:
 *   MFLib::MatchedFilterParameters       include/mflib/matchedFilterParameters.hpp
 *   MFLib::MatchedFilter<T>              include/mflib/matchedFilter.hpp
 *   MFLib::SingleChannel::MatchedFilterParameters / MatchedFilter<T>
 *                                        include/mflib/singleChannel/matchedFilter*.hpp
 *   MFLib::WaveformTemplate              include/mflib/waveformTemplate.hpp
 *   MFLib::NetworkStationPhase           include/mflib/networkStationPhase.hpp
 *   MFLib::PeakFinder<T>                 include/private/peakFinder.hpp
 *   MFLib::DBSCAN                        include/private/dbscan.hpp
 *   enums                                include/mflib/enums.hpp
 * MFGPU_EINVAL becomes std::invalid_argument, every other failure
 * std::runtime_error.  Pointers returned by get*Pointer() point into host
 * copies owned by the object, valid until the next apply, setSignal,
 * initialize or clear (the reference's contract for its own buffers).
 */
#ifndef MFGPU_HPP
#define MFGPU_HPP

#include <algorithm>
#include <cctype>
#include <cmath>
#include <complex>
#include <cstdint>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "mfgpu.h"

namespace MFLib
{

/* include/mflib/enums.hpp */
enum class MatchedFilterImplementation { DIRECT, OVERLAP_ADD, AUTO };
enum class MatchedFilterDetectionMode { SINGLE_CHANNEL, MULTI_CHANNEL };
enum class Polarity : int { UNKNOWN = 0, COMPRESSION = 1, DILATATION = -1 };
enum class RelativeMagnitudeType { GIBBONS_RINGDAL_2006 = 0, SCHAFF_RICHARDS_2014 };
enum class MaximumMatchedFilterPolicy { MAXIMUM = 0, ABSOLUTE_MAXIMUM };
enum class MatchedFilteredSignalDetectorPolicy { REDUCED = 0, SINGLE };
enum class DetectionTimeInterpolationType { LANCZOS = 0, QUADRATIC, NONE };

namespace detail
{
inline void check(mfgpu_status s)
{
    if (s == MFGPU_OK) return;
    const std::string msg = mfgpu_last_error();
    if (s == MFGPU_EINVAL) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}
template <class T> struct precision;
template <> struct precision<float> { static constexpr int value = MFGPU_FLOAT32; };
template <> struct precision<double> { static constexpr int value = MFGPU_FLOAT64; };
// blanks removed, upper case (src/networkStationPhase.cpp:88-187)
inline std::string canonical(std::string s)
{
    s.erase(std::remove(s.begin(), s.end(), ' '), s.end());
    for (char &c : s) c = (char) std::toupper((unsigned char) c);
    return s;
}
}  // namespace detail

/* ------------------------------------------------------------------------ */
/* MFLib::NetworkStationPhase (src/networkStationPhase.cpp) */
class NetworkStationPhase
{
  public:
    void clear() noexcept { mNet.clear(); mSta.clear(); mCha.clear(); mLoc.clear(); mPha.clear(); }
    void setNetwork(const std::string &v) noexcept { mNet = detail::canonical(v); }
    std::string getNetwork() const noexcept { return mNet; }
    void setStation(const std::string &v) noexcept { mSta = detail::canonical(v); }
    std::string getStation() const noexcept { return mSta; }
    void setChannel(const std::string &v) noexcept { mCha = detail::canonical(v); }
    std::string getChannel() const noexcept { return mCha; }
    void setLocationCode(const std::string &v) noexcept { mLoc = detail::canonical(v); }
    std::string getLocationCode() const noexcept { return mLoc; }
    void setPhase(const std::string &v) noexcept { mPha = detail::canonical(v); }
    std::string getPhase() const noexcept { return mPha; }
    /* equal objects hash equally (the reference hashes the joined fields) */
    size_t getHash() const noexcept
    {
        return std::hash<std::string>()(mNet + "." + mSta + "." + mCha + "." + mLoc + "." + mPha);
    }

  private:
    std::string mNet, mSta, mCha, mLoc, mPha;
};
inline bool operator==(const NetworkStationPhase &a, const NetworkStationPhase &b)
{
    return a.getNetwork() == b.getNetwork() && a.getStation() == b.getStation() && a.getChannel() == b.getChannel() &&
           a.getLocationCode() == b.getLocationCode() && a.getPhase() == b.getPhase();
}
inline bool operator!=(const NetworkStationPhase &a, const NetworkStationPhase &b) { return !(a == b); }

/* ------------------------------------------------------------------------ */
/* MFLib::WaveformTemplate (src/waveformTemplate.cpp:60-410) */
class WaveformTemplate
{
  public:
    void clear() noexcept { *this = WaveformTemplate(); }

    void setSignal(int npts, const double x[]) { setSignalT(npts, x); }
    void setSignal(int npts, const float x[]) { setSignalT(npts, x); }
    void getSignal(int maxx, double *x[]) const { getSignalT(maxx, x); }
    void getSignal(int maxx, float *x[]) const { getSignalT(maxx, x); }
    int getSignalLength() const
    {
        if (!haveSignal()) throw std::runtime_error("Signal not set");
        return (int) mX.size();
    }
    bool haveSignal() const noexcept { return !mX.empty(); }

    /* setting the sampling rate clears the onset time (:150-162) */
    void setSamplingRate(double fs)
    {
        if (fs <= 0) throw std::invalid_argument("Sampling rate = " + std::to_string(fs) + " must be positive");
        mOnset = -1;
        mFs = fs;
    }
    double getSamplingRate() const
    {
        if (!haveSamplingRate()) throw std::runtime_error("Sampling rate not set");
        return mFs;
    }
    bool haveSamplingRate() const noexcept { return mFs > 0; }

    void setShiftAndStackWeight(double w)
    {
        if (w < 0 || w > 1) throw std::invalid_argument("weight = " + std::to_string(w) + " must be in range [0,1]");
        mWeight = w;
    }
    double getShiftAndStackWeight() const noexcept { return mWeight; }

    /* bound (npts - 1) * fs as in the reference (:297) */
    void setPhaseOnsetTime(double t)
    {
        if (t < 0) throw std::invalid_argument("onsetTime = " + std::to_string(t) + " must be positive");
        const double tmax = (getSignalLength() - 1) * getSamplingRate();
        if (t > tmax)
            throw std::invalid_argument("onsetTime = " + std::to_string(t) + " cannot exceed maxOnsetTime = " +
                                        std::to_string(tmax));
        mOnset = t;
    }
    double getPhaseOnsetTime() const
    {
        if (!havePhaseOnsetTime()) throw std::runtime_error("Onset time not set");
        return mOnset;
    }
    bool havePhaseOnsetTime() const noexcept { return mOnset >= 0; }

    void setTravelTime(double t)
    {
        if (t < 0) throw std::runtime_error("Travel time cannot be negative");
        mTravel = t;
    }
    double getTravelTime() const
    {
        if (!haveTravelTime()) throw std::runtime_error("Travel time not yet set");
        return mTravel;
    }
    bool haveTravelTime() const noexcept { return mTravel >= 0; }

    void setIdentifier(const std::pair<NetworkStationPhase, uint64_t> &id) noexcept
    {
        mId = id;
        mHaveId = true;
    }
    std::pair<NetworkStationPhase, uint64_t> getIdentifier() const
    {
        if (!mHaveId) throw std::runtime_error("Waveform identifier not set");
        return mId;
    }
    bool haveIdentifier() const noexcept { return mHaveId; }

    void setMagnitude(double m) noexcept { mMag = m; mHaveMag = true; }
    double getMagnitude() const
    {
        if (!mHaveMag) throw std::runtime_error("Magnitude not set");
        return mMag;
    }
    bool haveMagnitude() const noexcept { return mHaveMag; }

    void setPolarity(Polarity p) noexcept { mPolarity = p; }
    Polarity getPolarity() const noexcept { return mPolarity; }

    /* FP64 samples without a copy (used by the matched filter) */
    const std::vector<double> &samples() const noexcept { return mX; }

  private:
    template <class U> void setSignalT(int npts, const U *x)
    {
        if (npts < 1) throw std::invalid_argument("npts must be positive");
        if (!x) throw std::invalid_argument("x is NULL");
        mOnset = -1;
        mX.assign(x, x + npts);
    }
    template <class U> void getSignalT(int maxx, U **x) const
    {
        const int n = getSignalLength();
        if (maxx < n) throw std::invalid_argument("maxx = " + std::to_string(maxx) + " must be at least " +
                                                  std::to_string(n));
        if (!x || !*x) throw std::invalid_argument("x is NULL");
        for (int i = 0; i < n; ++i) (*x)[i] = (U) mX[i];
    }
    std::vector<double> mX;
    double mFs = 0, mWeight = 1, mOnset = -1, mTravel = -1, mMag = 0;
    bool mHaveMag = false, mHaveId = false;
    std::pair<NetworkStationPhase, uint64_t> mId{};
    Polarity mPolarity = Polarity::UNKNOWN;
};

/* ------------------------------------------------------------------------ */
/* MFLib::computeOptimalFFTAndBlockLength (src/matchedFilterParameters.cpp:371-385) */
inline std::pair<int, int> computeOptimalFFTAndBlockLength(int nb, int nx)
{
    int n = 0, l = 0;
    detail::check(mfgpu_fft_sizes(nb, nx, &n, &l));
    return {n, l};
}

/* MFLib::MatchedFilterParameters (src/matchedFilterParameters.cpp:108-369) */
class MatchedFilterParameters
{
  public:
    void clear() noexcept
    {
        const MatchedFilterDetectionMode mode = mMode;
        *this = MatchedFilterParameters();
        mMode = mode;
    }
    /* needs a signal; sampling rates agree to 1e-4 (:199-219) */
    void addTemplate(const WaveformTemplate &wt)
    {
        if (!wt.haveSignal()) throw std::invalid_argument("Waveform not yet set on template");
        const double fs = wt.haveSamplingRate() ? wt.getSamplingRate() : 0.0;
        if (mTemplates.empty()) mFs = fs;
        if (std::abs(fs - mFs) > 1.e-4)
            throw std::invalid_argument("Template sampling rate = " + std::to_string(fs) + " must equal " +
                                        std::to_string(mFs));
        mTemplates.push_back(wt);
        mFFT = mBlock = 0;
    }
    void clearTemplates() noexcept
    {
        mTemplates.clear();
        mFFT = mBlock = 0;
    }
    WaveformTemplate getTemplate(int it) const
    {
        if (it < 0 || it >= getNumberOfTemplates())
            throw std::invalid_argument("template index = " + std::to_string(it) + " must be in range [0," +
                                        std::to_string(getNumberOfTemplates() - 1) + "]");
        return mTemplates[it];
    }
    int getNumberOfTemplates() const noexcept { return (int) mTemplates.size(); }
    int getMaxTemplateLength() const
    {
        if (mTemplates.empty()) throw std::runtime_error("No templates set");
        int m = 0;
        for (const auto &t : mTemplates) m = std::max(m, t.getSignalLength());
        return m;
    }
    void setSignalSize(int nx)
    {
        if (nx < 1) throw std::invalid_argument("Signal size must be positive");
        mNx = nx;
        mFFT = mBlock = 0;
    }
    int getSignalSize() const
    {
        if (mNx < 1) throw std::runtime_error("Signal size not set");
        return mNx;
    }
    /* stored only: initialize picks its own sizes, like the reference (:250-265) */
    void setFFTLength(int fftLength)
    {
        const int nb = getMaxTemplateLength();
        if (fftLength < nb)
            throw std::invalid_argument("fftLength = " + std::to_string(fftLength) + " must be at least " +
                                        std::to_string(nb));
        mFFT = fftLength;
        mBlock = fftLength - nb + 1;
    }
    int getFFTLength() const { return sizes().first; }
    int getBlockLength() const { return sizes().second; }
    void setDetectionMode(const MatchedFilterDetectionMode mode) noexcept { mMode = mode; }
    MatchedFilterDetectionMode getDetectionMode() const noexcept { return mMode; }
    void setMatchedFilterImplementation(const MatchedFilterImplementation impl) noexcept { mImpl = impl; }
    MatchedFilterImplementation getMatchedFilterImplementation() const noexcept { return mImpl; }
    void setStackAbsoluteValues(bool labs) noexcept { mStackAbs = labs; }
    bool getStackAbsoluteValues() const noexcept { return mStackAbs; }
    bool isValid() const noexcept { return !mTemplates.empty() && mNx >= 1; }

  private:
    std::pair<int, int> sizes() const
    {
        if (mTemplates.empty()) throw std::runtime_error("Templates must be set prior to calling this");
        if (mFFT > 0) return {mFFT, mBlock};
        /* the window-length rule of getFFTLength (src/matchedFilterParameters.cpp:268-300) */
        int n = 0, l = 0;
        detail::check(mfgpu_window_length(getMaxTemplateLength(), getSignalSize(), &n, &l));
        return {n, l};
    }
    std::vector<WaveformTemplate> mTemplates;
    double mFs = 0;
    int mNx = 0, mFFT = 0, mBlock = 0;
    MatchedFilterDetectionMode mMode = MatchedFilterDetectionMode::MULTI_CHANNEL;
    MatchedFilterImplementation mImpl = MatchedFilterImplementation::DIRECT;
    bool mStackAbs = true;
};

/* ------------------------------------------------------------------------ */
/* Extension, no reference counterpart: the stations' latest samples kept on
   the device (mfgpu_ring_*).  append() sends only new samples; a
   MatchedFilter<T> sets a request window from the ring on the device
   (setWindowFromRing). */
template <class T = double> class SignalRing
{
  public:
    SignalRing(int nChannels, long capacity)
    {
        detail::check(mfgpu_ring_create(detail::precision<T>::value, nChannels, capacity, &mH));
    }
    ~SignalRing() { mfgpu_ring_destroy(mH); }
    SignalRing(const SignalRing &) = delete;
    SignalRing &operator=(const SignalRing &) = delete;
    /* n new samples of every channel, rows of stride ld */
    void append(int n, const T *x, long ld) { detail::check(mfgpu_ring_append(mH, n, x, ld)); }
    /* samples appended per channel so far */
    long long getHead() const
    {
        long long h = 0;
        detail::check(mfgpu_ring_get_head(mH, &h));
        return h;
    }
    mfgpu_ring *handle() const noexcept { return mH; }

  private:
    mfgpu_ring *mH = nullptr;
};

/* ------------------------------------------------------------------------ */
/* MFLib::MatchedFilter<T> (include/mflib/matchedFilter.hpp:28-178) */
template <class T = double> class MatchedFilter
{
  public:
    MatchedFilter() { detail::check(mfgpu_mf_create(detail::precision<T>::value, &mH)); }
    ~MatchedFilter() { mfgpu_mf_destroy(mH); }
    MatchedFilter(const MatchedFilter &) = delete;
    MatchedFilter &operator=(const MatchedFilter &) = delete;

    void clear() noexcept
    {
        mfgpu_mf_clear(mH);
        mParams = MatchedFilterParameters();
        invalidate();
    }
    /* src/matchedFilter.cpp:507-821 */
    void initialize(const MatchedFilterParameters &parameters)
    {
        if (!parameters.isValid()) throw std::invalid_argument("Parameters are invalid");
        const int nt = parameters.getNumberOfTemplates();
        std::vector<WaveformTemplate> tps;
        std::vector<int> lens(nt);
        std::vector<const double *> ptrs(nt);
        for (int t = 0; t < nt; ++t) tps.push_back(parameters.getTemplate(t));
        for (int t = 0; t < nt; ++t)
        {
            lens[t] = tps[t].getSignalLength();
            ptrs[t] = tps[t].samples().data();
        }
        mfgpu_mf_params p{};
        p.detection_mode = parameters.getDetectionMode() == MatchedFilterDetectionMode::SINGLE_CHANNEL
                               ? MFGPU_SINGLE_CHANNEL
                               : MFGPU_MULTI_CHANNEL;
        p.n_templates = nt;
        p.template_lengths = lens.data();
        p.templates = ptrs.data();
        p.signal_size = parameters.getSignalSize();
        // shift-and-stack inputs when every template has an onset and a
        // travel time (src/matchedFilter.cpp:577-592)
        std::vector<int> shifts;
        std::vector<double> weights;
        bool stack = true;
        for (const auto &t : tps) stack = stack && t.havePhaseOnsetTime() && t.haveTravelTime();
        if (stack)
        {
            for (const auto &t : tps)
            {
                shifts.push_back((int) ((t.getTravelTime() - t.getPhaseOnsetTime()) * t.getSamplingRate() + 0.5));
                weights.push_back(t.getShiftAndStackWeight());
            }
            p.stack_shifts = shifts.data();
            p.stack_weights = weights.data();
        }
        p.stack_absolute_values = parameters.getStackAbsoluteValues() ? 1 : 0;
        detail::check(mfgpu_mf_initialize(mH, &p));
        mParams = parameters;
        invalidate();
    }
    WaveformTemplate getWaveformTemplate(int it) const { return mParams.getTemplate(it); }
    void setSignal(int it, int nSamples, const T signal[])
    {
        detail::check(mfgpu_mf_set_signal(mH, it, nSamples, signal));
        invalidate();
    }
    const T *getSignalPointer(int it) const
    {
        const int n = getSignalLength();
        if (it < 0 || it >= getNumberOfTemplates()) throw std::invalid_argument("it out of range");
        mSignals.resize(getNumberOfTemplates());
        auto &v = mSignals[it];
        v.resize(n);
        detail::check(mfgpu_mf_get_signal(mH, it, n, v.data()));
        return v.data();
    }
    void zeroSignal(int it)
    {
        detail::check(mfgpu_mf_zero_signal(mH, it));
        invalidate();
    }
    int getNumberOfTemplates() const { return query(mfgpu_mf_get_number_of_templates); }
    int getSignalLength() const { return query(mfgpu_mf_get_signal_length); }
    int getFilteredSignalLength() const { return query(mfgpu_mf_get_filtered_signal_length); }
    void apply()
    {
        invalidate();
        detail::check(mfgpu_mf_apply(mH));
    }
    std::vector<T> shiftAndStack()
    {
        std::vector<T> out(std::max(1, getFilteredSignalLength()));
        int nout = 0;
        detail::check(mfgpu_mf_shift_and_stack(mH, (int) out.size(), out.data(), &nout));
        out.resize(nout);
        return out;
    }
    std::vector<T> getMatchedFilteredSignal(int it) const
    {
        const T *p = getMatchedFilterSignalPointer(it);
        return std::vector<T>(p, p + getFilteredSignalLength());
    }
    /* host copy filled on first use after each apply */
    const T *getMatchedFilterSignalPointer(int it) const
    {
        const int nt = getNumberOfTemplates();
        if (!haveMatchedFilteredSignals()) throw std::runtime_error("Matched filtered signals not yet computed");
        if (it < 0 || it >= nt)
            throw std::invalid_argument("it = " + std::to_string(it) + " must be in the range [0," +
                                        std::to_string(nt - 1) + "]");
        mRho.resize(nt);
        auto &v = mRho[it];
        if (v.empty())
        {
            v.resize(std::max(1, getFilteredSignalLength()));
            int nout = 0;
            detail::check(mfgpu_mf_get_matched_filtered_signal(mH, it, (int) v.size(), v.data(), &nout));
            v.resize(std::max(1, nout));
        }
        return v.data();
    }
    bool haveMatchedFilteredSignals() const noexcept
    {
        int f = 0;
        return mfgpu_mf_have_matched_filtered_signals(mH, &f) == MFGPU_OK && f != 0;
    }
    bool isInitialized() const noexcept
    {
        int f = 0;
        return mfgpu_mf_is_initialized(mH, &f) == MFGPU_OK && f != 0;
    }
    /* debug view: rfft of the reversed, demeaned, unit-norm template at the
       FFT length initialize() picks for the padded signal of n + nb - 1
       samples (src/matchedFilter.cpp:522-530, :1412-1431) */
    std::vector<std::complex<T>> getSpectraOfTemplate(int it) const
    {
        const int nb = mParams.getMaxTemplateLength();
        const int nfft = computeOptimalFFTAndBlockLength(nb, getSignalLength() + nb - 1).first;
        std::vector<T> buf(2 * (size_t) (nfft / 2 + 1));
        int nout = 0;
        detail::check(mfgpu_mf_get_spectra_of_template(mH, it, (int) buf.size(), buf.data(), &nout));
        std::vector<std::complex<T>> out((size_t) nout / 2);
        for (size_t k = 0; k < out.size(); ++k) out[k] = std::complex<T>(buf[2 * k], buf[2 * k + 1]);
        return out;
    }

    /* Extension: samples [end - n, end) of the ring's channels become the
       source rows (mfgpu_mf_set_window_ring; channel c of the object reads
       row c % channels.size(), zero tail past n) */
    void setWindowFromRing(const SignalRing<T> &ring, const std::vector<int> &channels, long long end, int n)
    {
        invalidate();
        detail::check(mfgpu_mf_set_window_ring(mH, ring.handle(), (int) channels.size(), channels.data(), end, n));
    }

    /* the C-ABI handle, for the extensions in mfgpu.h */
    mfgpu_mf *handle() const noexcept { return mH; }

  protected:
    void invalidate() const
    {
        mRho.clear();
        mSignals.clear();
    }
    int query(mfgpu_status (*fn)(const mfgpu_mf *, int *)) const
    {
        int v = 0;
        detail::check(fn(mH, &v));
        return v;
    }
    mfgpu_mf *mH = nullptr;
    MatchedFilterParameters mParams;
    mutable std::vector<std::vector<T>> mRho, mSignals;
};

/* ------------------------------------------------------------------------ */
namespace SingleChannel
{
/* MFLib::SingleChannel::MatchedFilterParameters
   (src/singleChannel/matchedFilterParameters.cpp): the general parameters
   in SINGLE_CHANNEL mode */
class MatchedFilterParameters
{
  public:
    MatchedFilterParameters() { mP.setDetectionMode(MatchedFilterDetectionMode::SINGLE_CHANNEL); }
    void clear() noexcept
    {
        mP.clear();
        mP.setDetectionMode(MatchedFilterDetectionMode::SINGLE_CHANNEL);
    }
    void addTemplate(const MFLib::WaveformTemplate &wt) { mP.addTemplate(wt); }
    void clearTemplates() noexcept { mP.clearTemplates(); }
    WaveformTemplate getTemplate(int it) const { return mP.getTemplate(it); }
    int getNumberOfTemplates() const noexcept { return mP.getNumberOfTemplates(); }
    int getMaxTemplateLength() const { return mP.getMaxTemplateLength(); }
    void setSignalSize(int nx) { mP.setSignalSize(nx); }
    int getSignalSize() const { return mP.getSignalSize(); }
    void setFFTLength(int n) { mP.setFFTLength(n); }
    int getFFTLength() const { return mP.getFFTLength(); }
    int getBlockLength() const { return mP.getBlockLength(); }
    MFLib::MatchedFilterDetectionMode getDetectionMode() const noexcept { return mP.getDetectionMode(); }
    void setMatchedFilterImplementation(const MatchedFilterImplementation impl) noexcept
    {
        mP.setMatchedFilterImplementation(impl);
    }
    MatchedFilterImplementation getMatchedFilterImplementation() const noexcept
    {
        return mP.getMatchedFilterImplementation();
    }
    bool isValid() const noexcept { return mP.isValid(); }
    MFLib::MatchedFilterParameters getParameters() const { return mP; }

  private:
    MFLib::MatchedFilterParameters mP;
};

/* MFLib::SingleChannel::MatchedFilter<T> (src/singleChannel/matchedFilter.cpp:14-141) */
template <class T = double> class MatchedFilter
{
  public:
    void clear() noexcept { mF.clear(); }
    void initialize(const MFLib::SingleChannel::MatchedFilterParameters &parameters)
    {
        if (!parameters.isValid()) throw std::invalid_argument("Parameters are invalid");
        mF.initialize(parameters.getParameters());
    }
    MFLib::WaveformTemplate getWaveformTemplate(int it) const { return mF.getWaveformTemplate(it); }
    void setSignal(int nSamples, const T signal[]) { mF.setSignal(0, nSamples, signal); }
    const T *getSignalPointer() const { return mF.getSignalPointer(0); }
    void zeroSignal() { mF.zeroSignal(0); }
    int getNumberOfTemplates() const { return mF.getNumberOfTemplates(); }
    int getSignalLength() const { return mF.getSignalLength(); }
    int getFilteredSignalLength() const { return mF.getFilteredSignalLength(); }
    void apply() { mF.apply(); }
    std::vector<T> getMatchedFilteredSignal(int it) const { return mF.getMatchedFilteredSignal(it); }
    const T *getMatchedFilterSignalPointer(int it) const { return mF.getMatchedFilterSignalPointer(it); }
    bool haveMatchedFilteredSignals() const noexcept { return mF.haveMatchedFilteredSignals(); }
    bool isInitialized() const noexcept { return mF.isInitialized(); }
    mfgpu_mf *handle() const noexcept { return mF.handle(); }

  private:
    MFLib::MatchedFilter<T> mF;
};

/* MFLib::SingleChannel::DetectionTimeInterpolationParameters
   (src/singleChannel/detectionTimeInterpolationParameters.cpp) */
class DetectionTimeInterpolationParameters
{
  public:
    void clear() noexcept { *this = DetectionTimeInterpolationParameters(); }
    void enableLanczos() noexcept { mType = DetectionTimeInterpolationType::LANCZOS; }
    void enableQuadratic() noexcept { mType = DetectionTimeInterpolationType::QUADRATIC; }
    void disable() noexcept { mType = DetectionTimeInterpolationType::NONE; }
    DetectionTimeInterpolationType getType() const noexcept { return mType; }
    void setLanczosAlpha(int alpha)
    {
        if (alpha < 1) throw std::invalid_argument("alpha must be positive");
        mAlpha = alpha;
    }
    int getLanczosAlpha() const noexcept { return mAlpha; }
    void setLanczosNumberOfInterpolationPoints(int npts)
    {
        if (npts < 1) throw std::invalid_argument("Number of interpolation points must be positive");
        mPoints = npts;
    }
    int getLanczosNumberOfInterpolationPoints() const noexcept { return mPoints; }

  private:
    int mAlpha = 51, mPoints = 100;
    DetectionTimeInterpolationType mType = DetectionTimeInterpolationType::QUADRATIC;
};

/* MFLib::SingleChannel::DetectorParameters (src/singleChannel/detectorParameters.cpp:9-26) */
class DetectorParameters
{
  public:
    void clear() noexcept { *this = DetectorParameters(); }
    void setDetectionThreshold(double tol)
    {
        if (tol <= 0 || tol > 1) throw std::invalid_argument("Threshold must be in range (0,1]");
        mThreshold = tol;
    }
    double getDetectionThreshold() const noexcept { return mThreshold; }
    void setMinimumDetectionSpacing(int n) noexcept { mMinSpacing = n; }
    int getMinimumDetectionSpacing() const noexcept { return mMinSpacing; }
    void setMatchedFilteredSignalDetectorPolicy(MatchedFilteredSignalDetectorPolicy p) noexcept { mPolicy = p; }
    MatchedFilteredSignalDetectorPolicy getMatchedFilteredSignalDetectorPolicy() const noexcept { return mPolicy; }
    void setMaximaPolicy(MaximumMatchedFilterPolicy p) noexcept { mMax = p; }
    MaximumMatchedFilterPolicy getMaximaPolicy() const noexcept { return mMax; }
    void enableSaveDetectedWaveform() noexcept { mWave = true; }
    void disableSaveDetectedWaveform() noexcept { mWave = false; }
    bool wantDetectedWaveform() const noexcept { return mWave; }
    void enableSaveAmplitudeScalingFactor() noexcept { mAmp = true; }
    void disableSaveAmplitudeScalingFactor() noexcept { mAmp = false; }
    bool wantAmplitudeScalingFactor() const noexcept { return mAmp; }
    void setDetectionTimeInterpolationParameters(const DetectionTimeInterpolationParameters &p) noexcept
    {
        mInterp = p;
    }
    const DetectionTimeInterpolationParameters &getDetectionTimeInterpolationParameters() const noexcept
    {
        return mInterp;
    }

  private:
    double mThreshold = 0.7;
    int mMinSpacing = 0;
    MaximumMatchedFilterPolicy mMax = MaximumMatchedFilterPolicy::MAXIMUM;
    MatchedFilteredSignalDetectorPolicy mPolicy = MatchedFilteredSignalDetectorPolicy::SINGLE;
    bool mWave = false, mAmp = true;
    DetectionTimeInterpolationParameters mInterp;
};

/* MFLib::SingleChannel::Detection<T> (src/singleChannel/detection.cpp): the
   value fields the detector fills, each with get / set / have */
template <class T = double> class Detection
{
  public:
    void clear() noexcept { *this = Detection(); }
    void setTemplateIdentifier(const std::pair<NetworkStationPhase, uint64_t> &id) { mId = id; mHaveId = true; }
    std::pair<NetworkStationPhase, uint64_t> getTemplateIdentifier() const
    {
        if (!mHaveId) throw std::runtime_error("Template identifier not set");
        return mId;
    }
    bool haveTemplateIdentifier() const noexcept { return mHaveId; }
    void setCorrelationCoefficient(double v)
    {
        if (v < -1 || v > 1) throw std::invalid_argument("Correlation coefficient must be in range [-1,1]");
        mXc = v;
        mHaveXc = true;
    }
    double getCorrelationCoefficient() const { return get(mXc, mHaveXc, "Correlation coefficient"); }
    bool haveCorrelationCoefficient() const noexcept { return mHaveXc; }
    void setDetectedSignal(int n, const T x[]) { mSignal.assign(x, x + n); }
    const T *getDetectedSignalPointer() const
    {
        if (mSignal.empty()) throw std::runtime_error("Detected signal not set");
        return mSignal.data();
    }
    int getDetectedSignalLength() const { return (int) mSignal.size(); }
    bool haveDetectedSignal() const noexcept { return !mSignal.empty(); }
    /* copies the detected signal into *x, which holds n >= its length */
    void getDetectedSignal(int n, T *x[]) const
    {
        const T *src = getDetectedSignalPointer();
        if (n < (int) mSignal.size())
            throw std::invalid_argument("Signal length = " + std::to_string(n) + " must be at least = " +
                                        std::to_string(mSignal.size()));
        if (!x || !*x) throw std::invalid_argument("x is NULL");
        std::copy(src, src + mSignal.size(), *x);
    }
    void setDetectionTime(double t) { mT = t; mHaveT = true; }
    double getDetectionTime() const { return get(mT, mHaveT, "Detection time"); }
    bool haveDetectionTime() const noexcept { return mHaveT; }
    void setInterpolatedDetectionTime(double t) { mTi = t; mHaveTi = true; }
    double getInterpolatedDetectionTime() const { return get(mTi, mHaveTi, "Interpolated detection time"); }
    bool haveInterpolatedDetectionTime() const noexcept { return mHaveTi; }
    void setTravelTime(double t) { mTt = t; mHaveTt = true; }
    double getTravelTime() const { return get(mTt, mHaveTt, "Travel time"); }
    bool haveTravelTime() const noexcept { return mHaveTt; }
    void setPhaseOnsetTime(double t) { mPo = t; mHavePo = true; }
    double getPhaseOnsetTime() const { return get(mPo, mHavePo, "Phase onset time"); }
    bool havePhaseOnsetTime() const noexcept { return mHavePo; }
    void setInterpolatedPhaseOnsetTime(double t) { mPoi = t; mHavePoi = true; }
    double getInterpolatedPhaseOnsetTime() const { return get(mPoi, mHavePoi, "Interpolated phase onset time"); }
    bool haveInterpolatedPhaseOnsetTime() const noexcept { return mHavePoi; }
    void setAmplitudeScalingFactor(T value, RelativeMagnitudeType type)
    {
        mAmp[(int) type] = value;
        mHaveAmp[(int) type] = true;
    }
    T getAmplitudeScalingFactor(RelativeMagnitudeType type) const
    {
        if (!mHaveAmp[(int) type]) throw std::runtime_error("Amplitude scaling factor not set");
        return mAmp[(int) type];
    }
    bool haveAmplitudeScalingFactor(RelativeMagnitudeType type) const noexcept { return mHaveAmp[(int) type]; }
    T getMagnitudePerturbation(RelativeMagnitudeType type) const
    {
        const T a = getAmplitudeScalingFactor(type);
        if (a <= 0) throw std::invalid_argument("Scaling factor must be positive");
        return std::log10(a);
    }
    bool haveMagnitudePerturbation(RelativeMagnitudeType type) const noexcept { return haveAmplitudeScalingFactor(type); }
    void setPolarity(Polarity p) noexcept { mPol = p; }
    Polarity getPolarity() const noexcept { return mPol; }

  private:
    static double get(double v, bool have, const char *what)
    {
        if (!have) throw std::runtime_error(std::string(what) + " not set");
        return v;
    }
    std::pair<NetworkStationPhase, uint64_t> mId;
    double mXc = 0, mT = 0, mTi = 0, mTt = 0, mPo = 0, mPoi = 0;
    bool mHaveId = false, mHaveXc = false, mHaveT = false, mHaveTi = false, mHaveTt = false, mHavePo = false,
         mHavePoi = false;
    T mAmp[2] = {0, 0};
    bool mHaveAmp[2] = {false, false};
    std::vector<T> mSignal;
    Polarity mPol = Polarity::UNKNOWN;
};

/* MFLib::SingleChannel::Detector<T> (src/singleChannel/detector.cpp:385-691):
   the data-parallel work in one mfgpu_mf_detect call, the Detection objects
   filled from the templates' metadata */
template <class T = double> class Detector
{
  public:
    void clear() noexcept
    {
        mInit = false;
        mDets.clear();
    }
    void initialize(const DetectorParameters &parameters)
    {
        clear();
        mP = parameters;
        mInit = true;
    }
    bool isInitialized() const noexcept { return mInit; }
    /* the traces detect() reduces: checks them and records their length
       (detect runs the reduction and the detections in one device call) */
    void setMatchedFilteredSignals(const MFLib::SingleChannel::MatchedFilter<T> &mf)
    {
        if (!mInit) throw std::runtime_error("Detector class not initialized");
        if (!mf.haveMatchedFilteredSignals()) throw std::invalid_argument("Matched filtered signals not computed");
        mLength = (int) mf.getMatchedFilteredSignal(0).size();
    }
    int getMatchedFilteredSignalLength() const noexcept { return mLength; }
    void detect(const MFLib::SingleChannel::MatchedFilter<T> &mf)
    {
        mDets.clear();
        if (!mInit) throw std::invalid_argument("Detector class not initialized");
        if (!mf.haveMatchedFilteredSignals()) throw std::invalid_argument("Matched filtered signals not computed");
        const int nt = mf.getNumberOfTemplates();
        std::vector<WaveformTemplate> tps;
        for (int t = 0; t < nt; ++t) tps.push_back(mf.getWaveformTemplate(t));
        const DetectionTimeInterpolationParameters &ip = mP.getDetectionTimeInterpolationParameters();
        mfgpu_detect_params dp{};
        dp.threshold = std::min(1.0, std::max(0.0, mP.getDetectionThreshold()));
        dp.min_distance = mP.getMinimumDetectionSpacing();
        dp.absolute_maximum = mP.getMaximaPolicy() == MaximumMatchedFilterPolicy::ABSOLUTE_MAXIMUM;
        dp.single = mP.getMatchedFilteredSignalDetectorPolicy() == MatchedFilteredSignalDetectorPolicy::SINGLE;
        dp.interpolation = (int) ip.getType();
        dp.lanczos_alpha = ip.getLanczosAlpha();
        dp.lanczos_points = ip.getLanczosNumberOfInterpolationPoints();
        dp.sampling_rate = tps.at(0).getSamplingRate();
        dp.amplitudes = mP.wantAmplitudeScalingFactor();
        int n = 0;
        detail::check(mfgpu_mf_detect(mf.handle(), &dp, &n));
        std::vector<mfgpu_detection> raw(std::max(1, n));
        detail::check(mfgpu_mf_get_detections(mf.handle(), n, raw.data(), &n));
        const T *signal = mP.wantDetectedWaveform() ? mf.getSignalPointer() : nullptr;
        const int ns = mf.getSignalLength();
        mLength = ns - mf.getWaveformTemplate(0).getSignalLength() + 1;
        for (int i = 0; i < n; ++i)
        {
            const mfgpu_detection &r = raw[i];
            const WaveformTemplate &wt = tps[r.template_index];
            Detection<T> d;
            if (wt.haveIdentifier()) d.setTemplateIdentifier(wt.getIdentifier());
            else d.setTemplateIdentifier({NetworkStationPhase(), (uint64_t) r.template_index});
            d.setCorrelationCoefficient(r.correlation);
            d.setDetectionTime(r.detection_time);
            d.setInterpolatedDetectionTime(r.interpolated_time);
            if (wt.havePhaseOnsetTime())
            {
                d.setPhaseOnsetTime(r.detection_time + wt.getPhaseOnsetTime());
                d.setInterpolatedPhaseOnsetTime(r.interpolated_time + wt.getPhaseOnsetTime());
            }
            d.setPolarity((Polarity) (r.sign * (int) wt.getPolarity()));
            if (wt.haveTravelTime()) d.setTravelTime(wt.getTravelTime());
            if (r.have_amplitude)
            {
                d.setAmplitudeScalingFactor((T) r.gibbons_ringdal, RelativeMagnitudeType::GIBBONS_RINGDAL_2006);
                d.setAmplitudeScalingFactor((T) r.schaff_richards, RelativeMagnitudeType::SCHAFF_RICHARDS_2014);
            }
            if (signal)
                d.setDetectedSignal(std::min(wt.getSignalLength(), ns - r.sample), signal + r.sample);
            mDets.push_back(std::move(d));
        }
    }
    int getNumberOfDetections() const noexcept { return (int) mDets.size(); }
    Detection<T> getDetection(int id) const
    {
        if (id < 0 || id >= (int) mDets.size()) throw std::invalid_argument("detection index out of range");
        return mDets[id];
    }

  private:
    DetectorParameters mP;
    std::vector<Detection<T>> mDets;
    bool mInit = false;
    int mLength = 0;
};

/* MFLib::SingleChannel::convertAmplitudeScalingFactorToMagnitudePerturbation
   (src/singleChannel/relativeMagnitude.cpp:399-420) */
inline double convertAmplitudeScalingFactorToMagnitudePerturbation(double alpha)
{
    if (alpha <= 0) throw std::invalid_argument("Scaling factor = " + std::to_string(alpha) + " must be positive");
    return std::log10(alpha);
}
inline float convertAmplitudeScalingFactorToMagnitudePerturbation(float alpha)
{
    if (alpha <= 0) throw std::invalid_argument("Scaling factor = " + std::to_string(alpha) + " must be positive");
    return std::log10(alpha);
}

/* MFLib::SingleChannel::RelativeMagnitude<T>
   (src/singleChannel/relativeMagnitude.cpp:260-396): the two amplitude
   scaling factors of a detected window against the template, from
   mfgpu_relative_amplitudes (which also takes many windows per call) */
template <class T = double> class RelativeMagnitude
{
  public:
    void clear() noexcept
    {
        mB.clear();
        mHave = false;
    }
    void initialize(const WaveformTemplate &wt)
    {
        clear();
        if (!wt.haveSignal()) throw std::invalid_argument("Template signal length = 0 must be positive");
        const int L = wt.getSignalLength();
        std::vector<double> b((size_t) L);
        double *pb = b.data();
        wt.getSignal(L, &pb);
        bool constant = true;
        for (int i = 1; i < L && constant; ++i) constant = b[i] == b[0];
        if (constant) throw std::invalid_argument("Template signal cannot be constant");
        mB = std::move(b);
    }
    bool isInitialized() const noexcept { return !mB.empty(); }
    int getDetectedSignalLength() const
    {
        if (!isInitialized()) throw std::runtime_error("Class not initialized");
        return (int) mB.size();
    }
    void setDetectedSignal(int n, const T y[])
    {
        mHave = false;
        if (!isInitialized()) throw std::runtime_error("Class not initialized");
        if (n != (int) mB.size())
            throw std::invalid_argument("Signal length = " + std::to_string(n) + " must = " + std::to_string(mB.size()));
        if (!y) throw std::invalid_argument("Signal is NULL");
        int valid = 0;
        detail::check(mfgpu_relative_amplitudes(detail::precision<T>::value, n, mB.data(), 1, y, n, &mAlpha[0],
                                                &mAlpha[1], &valid));
        if (!valid) throw std::invalid_argument("Detected signal cannot be constant");
        mHave = true;
    }
    bool haveDetectedSignal() const noexcept { return mHave; }
    T computeAmplitudeScalingFactor(RelativeMagnitudeType type) const
    {
        if (!isInitialized()) throw std::runtime_error("Class is not initialized");
        if (!mHave) throw std::runtime_error("Detected waveform not set");
        return (T) mAlpha[type == RelativeMagnitudeType::GIBBONS_RINGDAL_2006 ? 0 : 1];
    }
    T computeMagnitudePerturbation(RelativeMagnitudeType type) const
    {
        return convertAmplitudeScalingFactorToMagnitudePerturbation(computeAmplitudeScalingFactor(type));
    }

  private:
    std::vector<double> mB;
    double mAlpha[2] = {0, 0};
    bool mHave = false;
};

/* MFLib::SingleChannel::AssociatorParameters
   (src/singleChannel/associatorParameters.cpp, defaults :10-18) */
class AssociatorParameters
{
  public:
    void clear() noexcept { *this = AssociatorParameters(); }
    void setOriginTimeTolerance(double tol)
    {
        if (tol < 0) throw std::invalid_argument("tolerance = " + std::to_string(tol) + " must be positive");
        mTol = tol;
    }
    double getOriginTimeTolerance() const noexcept { return mTol; }
    void setMinimumNumberOfPicksInEvent(int n)
    {
        if (n < 1) throw std::invalid_argument("minPicks = " + std::to_string(n) + " must be positive");
        mMinPicks = n;
    }
    int getMinimumNumberOfPicksInEvent() const noexcept { return mMinPicks; }
    void enableCorrelationCoefficientWeighting() noexcept { mWeight = true; }
    void disableCorrelationCoefficientWeighting() noexcept { mWeight = false; }
    bool useCorrelationCoefficientWeighting() const noexcept { return mWeight; }

  private:
    double mTol = 2.0;
    int mMinPicks = 5;
    bool mWeight = false;
};

/* MFLib::SingleChannel::Associator<T> (src/singleChannel/associator.cpp):
   detections grouped by their template identifier's id, each group sorted
   by phase onset time, the origin times (onset - travel time) of every
   group clustered by DBSCAN with eps = the origin-time tolerance and
   minPts = the minimum number of picks (weighted by the coefficients when
   asked), all groups in one mfgpu_dbscan_segmented call; each cluster is an
   event, events ordered by id, then cluster.  The sorts are stable (the
   reference's std::sort leaves equal keys in unspecified order), and
   getDetectionsInEvent checks the event index against the number of events. */
template <class T = double> class Associator
{
  public:
    Associator() = default;
    ~Associator()
    {
        if (mDb) mfgpu_dbscan_destroy(mDb);
    }
    Associator(const Associator &) = delete;
    Associator &operator=(const Associator &) = delete;
    void clear() noexcept
    {
        mInit = false;
        mDets.clear();
        mEvents.clear();
    }
    void initialize(const AssociatorParameters &parameters)
    {
        clear();
        mP = parameters;
        mInit = true;
    }
    bool isInitialized() const noexcept { return mInit; }
    void addDetection(const Detection<T> &det)
    {
        mEvents.clear();
        if (!mInit) throw std::runtime_error("Class not initialized");
        if (!det.haveTravelTime()) throw std::invalid_argument("Travel time must be set");
        if (!det.haveTemplateIdentifier()) throw std::invalid_argument("Template identifier must be set");
        if (mP.useCorrelationCoefficientWeighting() && !det.haveCorrelationCoefficient())
            throw std::invalid_argument("XC coefficient must be set");
        mDets.push_back(det);
    }
    int getNumberOfDetections() const noexcept { return (int) mDets.size(); }
    void clearDetections() noexcept
    {
        mDets.clear();
        mEvents.clear();
    }
    void associate()
    {
        mEvents.clear();
        if (!mInit) throw std::runtime_error("Class is not intialized");
        if (mDets.empty()) return;
        const size_t n = mDets.size();
        std::vector<uint64_t> id(n);
        std::vector<double> onset(n), travel(n);
        for (size_t i = 0; i < n; ++i)
        {
            id[i] = mDets[i].getTemplateIdentifier().second;
            onset[i] = mDets[i].getPhaseOnsetTime();
            travel[i] = mDets[i].getTravelTime();
        }
        std::vector<size_t> order(n);
        for (size_t i = 0; i < n; ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
            return id[a] < id[b] || (id[a] == id[b] && onset[a] < onset[b]);
        });
        std::vector<Detection<T>> sorted;
        sorted.reserve(n);
        std::vector<double> X(n), w;
        std::vector<int> offs{0};
        std::vector<uint64_t> ids;
        for (size_t r = 0; r < n; ++r)
        {
            const size_t i = order[r];
            if (r == 0 || id[i] != ids.back())
            {
                if (r > 0) offs.push_back((int) r);
                ids.push_back(id[i]);
            }
            X[r] = onset[i] - travel[i];
            sorted.push_back(mDets[i]);
        }
        offs.push_back((int) n);
        if (mP.useCorrelationCoefficientWeighting())
        {
            w.resize(n);
            for (size_t r = 0; r < n; ++r)
            {
                w[r] = sorted[r].getCorrelationCoefficient();
                if (!(w[r] > 0)) throw std::invalid_argument("All weights must be positive");
            }
        }
        mDets = std::move(sorted);
        if (!mDb) detail::check(mfgpu_dbscan_create(&mDb));
        detail::check(mfgpu_dbscan_initialize(mDb, mP.getOriginTimeTolerance(), mP.getMinimumNumberOfPicksInEvent()));
        const int nseg = (int) ids.size();
        std::vector<int> labels(n), ncl((size_t) nseg);
        detail::check(mfgpu_dbscan_segmented(mDb, nseg, offs.data(), 1, X.data(), w.empty() ? nullptr : w.data(),
                                             labels.data(), ncl.data()));
        for (int s = 0; s < nseg; ++s)
            for (int c = 0; c < ncl[s]; ++c)
            {
                std::vector<int> members;
                for (int i = offs[s]; i < offs[s + 1]; ++i)
                    if (labels[i] == c) members.push_back(i);
                mEvents.push_back(std::move(members));
            }
    }
    int getNumberOfEvents() const noexcept { return (int) mEvents.size(); }
    std::vector<Detection<T>> getDetectionsInEvent(int iev) const
    {
        if (mEvents.empty()) throw std::runtime_error("No detections have been associated");
        if (iev < 0 || iev >= (int) mEvents.size())
            throw std::invalid_argument("iev = " + std::to_string(iev) + " must be in range [0," +
                                        std::to_string(mEvents.size() - 1) + "]");
        std::vector<Detection<T>> out;
        for (int i : mEvents[iev]) out.push_back(mDets[i]);
        return out;
    }

  private:
    AssociatorParameters mP;
    std::vector<Detection<T>> mDets;
    std::vector<std::vector<int>> mEvents;
    mfgpu_dbscan *mDb = nullptr;
    bool mInit = false;
};
}  // namespace SingleChannel

/* ------------------------------------------------------------------------ */
/* MFLib::PeakFinder<T> (include/private/peakFinder.hpp:12-138) */
template <class T = double> class PeakFinder
{
  public:
    PeakFinder() { detail::check(mfgpu_peaks_create(detail::precision<T>::value, &mH)); }
    ~PeakFinder() { mfgpu_peaks_destroy(mH); }
    PeakFinder(const PeakFinder &) = delete;
    PeakFinder &operator=(const PeakFinder &) = delete;
    void clear() noexcept
    {
        mfgpu_peaks_clear(mH);
        mPeaks.clear();
    }
    void setMinimumPeakDistance(int minDistance) noexcept { mfgpu_peaks_set_minimum_peak_distance(mH, minDistance); }
    int getMinimumPeakDistance() const noexcept
    {
        int d = 0;
        mfgpu_peaks_get_minimum_peak_distance(mH, &d);
        return d;
    }
    /* throws outside [0, 1] (src/peakFinder.cpp:229-233) */
    void setThreshold(T threshold) { detail::check(mfgpu_peaks_set_threshold(mH, (double) threshold)); }
    T getThreshold() const noexcept
    {
        double v = 0;
        mfgpu_peaks_get_threshold(mH, &v);
        return (T) v;
    }
    void setSignal(const int n, const T x[])
    {
        detail::check(mfgpu_peaks_set_signal(mH, n, x));
        mPeaks.clear();
    }
    void apply()
    {
        detail::check(mfgpu_peaks_apply(mH));
        int n = 0;
        detail::check(mfgpu_peaks_get_number_of_peaks(mH, &n));
        mPeaks.assign(n, 0);
        if (n > 0) detail::check(mfgpu_peaks_get_peak_indices(mH, n, mPeaks.data()));
    }
    int getNumberOfPeaks() const noexcept { return (int) mPeaks.size(); }
    void getPeakIndices(int maxSpace, int *peakIndices[]) const
    {
        const int n = getNumberOfPeaks();
        if (maxSpace < n) throw std::invalid_argument("maxSpace = " + std::to_string(maxSpace) + " must be at least " +
                                                      std::to_string(n));
        if (n > 0 && (!peakIndices || !*peakIndices)) throw std::invalid_argument("peakIndices is NULL");
        std::copy(mPeaks.begin(), mPeaks.end(), n > 0 ? *peakIndices : nullptr);
    }
    /* nullptr when there are no peaks (include/private/peakFinder.hpp) */
    const int *getPeakIndicesPointer() const { return mPeaks.empty() ? nullptr : mPeaks.data(); }

  private:
    mfgpu_peaks *mH = nullptr;
    std::vector<int> mPeaks;
};

/* ------------------------------------------------------------------------ */
/* MFLib::DBSCAN (include/private/dbscan.hpp:10-132, DAAL semantics) */
class DBSCAN
{
  public:
    DBSCAN() { detail::check(mfgpu_dbscan_create(&mH)); }
    ~DBSCAN() { mfgpu_dbscan_destroy(mH); }
    DBSCAN(const DBSCAN &) = delete;
    DBSCAN &operator=(const DBSCAN &) = delete;
    void clear() noexcept { mfgpu_dbscan_clear(mH); }
    void initialize(double epsilon, int minSamples) { detail::check(mfgpu_dbscan_initialize(mH, epsilon, minSamples)); }
    bool isInitialized() const noexcept { return flag(mfgpu_dbscan_is_initialized); }
    void setData(int nObservations, int nFeatures, const double X[])
    {
        detail::check(mfgpu_dbscan_set_data(mH, nObservations, nFeatures, X));
        mNobs = nObservations;
    }
    void setWeightedData(int nObservations, int nFeatures, const double X[], const double weights[])
    {
        detail::check(mfgpu_dbscan_set_weighted_data(mH, nObservations, nFeatures, X, weights));
        mNobs = nObservations;
    }
    bool haveData() const noexcept { return flag(mfgpu_dbscan_have_data); }
    void cluster() { detail::check(mfgpu_dbscan_cluster(mH)); }
    int getNumberOfClusters() const noexcept
    {
        int n = 0;
        mfgpu_dbscan_get_number_of_clusters(mH, &n);
        return n;
    }
    std::vector<int> getLabels() const
    {
        std::vector<int> out(std::max(1, mNobs));
        detail::check(mfgpu_dbscan_get_labels(mH, (int) out.size(), out.data()));
        out.resize(mNobs);
        return out;
    }
    bool haveLabels() const noexcept { return flag(mfgpu_dbscan_have_labels); }

  private:
    bool flag(mfgpu_status (*fn)(const mfgpu_dbscan *, int *)) const noexcept
    {
        int f = 0;
        return fn(mH, &f) == MFGPU_OK && f != 0;
    }
    mfgpu_dbscan *mH = nullptr;
    int mNobs = 0;
};

}  // namespace MFLib

#endif
