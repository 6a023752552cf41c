// C++ API mirror (include/mfgpu.hpp) on the device, checked the way the
// reference's own C++ tests check mflib: known-answer matched filters against
// a two-pass Pearson correlation (testing/matchedFilter.cpp,
// testing/singleChannel.cpp, testing/utilities.hpp), the peak finder's exact
// index lists (testing/peakFinder.cpp), the DBSCAN golden labels
// (testing/dbscan.cpp) and the FFT-sizing values
// (testing/matchedFilterParameters.cpp).  Prints one line per check and
// "ALL PASSED"; exits non-zero on the first failure.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "mfgpu.hpp"

namespace {

int g_checks = 0;

void require(bool ok, const std::string &what)
{
    ++g_checks;
    if (!ok)
    {
        std::printf("FAIL: %s\n", what.c_str());
        std::exit(1);
    }
    std::printf("ok   %s\n", what.c_str());
}

template <class F> bool throws_invalid(F f)
{
    try { f(); } catch (const std::invalid_argument &) { return true; } catch (...) { return false; }
    return false;
}
template <class F> bool throws_runtime(F f)
{
    try { f(); } catch (const std::invalid_argument &) { return false; } catch (const std::runtime_error &) { return true; }
    catch (...) { return false; }
    return false;
}

// two-pass Pearson correlation of template b against every window of x, in
// long double (the reference tests' naive check)
std::vector<double> pearson(const std::vector<double> &b, const std::vector<double> &x)
{
    const size_t L = b.size(), n = x.size() - L + 1;
    long double mb = 0;
    for (double v : b) mb += v;
    mb /= L;
    long double sb = 0;
    for (double v : b) sb += (v - mb) * (v - mb);
    std::vector<double> out(n);
    for (size_t k = 0; k < n; ++k)
    {
        long double mx = 0;
        for (size_t j = 0; j < L; ++j) mx += x[k + j];
        mx /= L;
        long double sxy = 0, sx = 0;
        for (size_t j = 0; j < L; ++j)
        {
            const long double d = x[k + j] - mx;
            sxy += d * (b[j] - mb);
            sx += d * d;
        }
        out[k] = (sx > 0 && sb > 0) ? (double) (sxy / std::sqrt(sx * sb)) : 0.0;
    }
    return out;
}

template <class T> double max_err(const std::vector<T> &a, const std::vector<double> &b)
{
    double m = 0;
    for (size_t i = 0; i < a.size() && i < b.size(); ++i) m = std::max(m, std::abs((double) a[i] - b[i]));
    return a.size() == b.size() ? m : 1e30;
}

MFLib::WaveformTemplate make_template(const std::vector<double> &s, double fs)
{
    MFLib::WaveformTemplate wt;
    wt.setSignal((int) s.size(), s.data());
    wt.setSamplingRate(fs);
    return wt;
}

// damped sine/cosine signals and 2 s templates (testing/matchedFilter.cpp:63-90)
void damped(std::vector<double> &x, std::vector<double> &x2, std::vector<double> &b, std::vector<double> &b2)
{
    const int n = 1000;
    const double tmax = 8, dt = tmax / (n - 1), f0 = 4 / tmax, pi = 3.14159265358979323846;
    x.resize(n);
    x2.resize(n);
    for (int i = 0; i < n; ++i)
    {
        const double t = i * dt;
        x[i] = 2 * std::exp(-0.1 * t) * std::sin(2 * pi * f0 * t);
        x2[i] = 2 * std::exp(-0.15 * t) * std::cos(2 * pi * f0 * t);
    }
    const int nb = (int) (2.0 / dt + 0.5) + 1;
    b.resize(nb);
    b2.resize(nb);
    for (int i = 0; i < nb; ++i)
    {
        b[i] = std::sin(2 * pi * f0 * i * dt);
        b2[i] = std::cos(2 * pi * f0 * i * dt);
    }
}

void test_fft_sizes()
{
    const int cases[4][4] = {{4500, 75000, 32768, 28269}, {4500, 8640000, 65536, 61037}, {101, 1024, 512, 412},
                             {99, 1024, 512, 414}};
    for (const auto &c : cases)
    {
        auto r = MFLib::computeOptimalFFTAndBlockLength(c[0], c[1]);
        require(r.first == c[2] && r.second == c[3], "computeOptimalFFTAndBlockLength(" + std::to_string(c[0]) + ", " +
                                                         std::to_string(c[1]) + ")");
    }
    require(throws_invalid([] { MFLib::computeOptimalFFTAndBlockLength(0, 10); }), "fft sizes reject nb < 1");
}

void test_multichannel_double()
{
    std::vector<double> x, x2, b, b2;
    damped(x, x2, b, b2);
    MFLib::MatchedFilterParameters p;
    for (auto *t : {&b, &b2, &b, &b2}) p.addTemplate(make_template(*t, 1.0));
    p.setSignalSize((int) x.size());
    MFLib::MatchedFilter<double> mf;
    require(throws_runtime([&] { mf.apply(); }), "apply before initialize throws runtime_error");
    mf.initialize(p);
    require(mf.isInitialized() && mf.getNumberOfTemplates() == 4, "initialize");
    require(mf.getFilteredSignalLength() == (int) (x.size() - b.size() + 1), "getFilteredSignalLength");
    const std::vector<double> *sig[4] = {&x, &x2, &x, &x2};
    for (int i = 0; i < 4; ++i) mf.setSignal(i, (int) sig[i]->size(), sig[i]->data());
    require(throws_invalid([&] { mf.setSignal(0, 10, x.data()); }), "setSignal with a wrong length throws");
    require(!mf.haveMatchedFilteredSignals(), "no results before apply");
    require(throws_runtime([&] { mf.getMatchedFilteredSignal(0); }), "results before apply throw runtime_error");
    mf.apply();
    require(mf.haveMatchedFilteredSignals(), "results after apply");
    const std::vector<double> *tp[4] = {&b, &b2, &b, &b2};
    for (int i = 0; i < 4; ++i)
    {
        const double e = max_err(mf.getMatchedFilteredSignal(i), pearson(*tp[i], *sig[i]));
        require(e < 1e-13, "FP64 template " + std::to_string(i) + " vs two-pass Pearson (" + std::to_string(e) + ")");
    }
    const double *ptr = mf.getMatchedFilterSignalPointer(1);
    require(ptr && std::abs(ptr[5] - mf.getMatchedFilteredSignal(1)[5]) == 0, "getMatchedFilterSignalPointer");
    const double *sp = mf.getSignalPointer(2);
    require(sp && sp[17] == x[17], "getSignalPointer");
    require(throws_invalid([&] { mf.getMatchedFilteredSignal(7); }), "template index out of range throws");
    auto spec = mf.getSpectraOfTemplate(0);
    const int nfft = MFLib::computeOptimalFFTAndBlockLength((int) b.size(), (int) (x.size() + b.size() - 1)).first;
    require((int) spec.size() == nfft / 2 + 1, "getSpectraOfTemplate length");
}

void test_multichannel_float()
{
    std::vector<double> x, x2, b, b2;
    damped(x, x2, b, b2);
    MFLib::MatchedFilterParameters p;
    p.addTemplate(make_template(b, 1.0));
    p.addTemplate(make_template(b2, 1.0));
    p.setSignalSize((int) x.size());
    MFLib::MatchedFilter<float> mf;
    mf.initialize(p);
    std::vector<float> xf(x.begin(), x.end()), x2f(x2.begin(), x2.end());
    mf.setSignal(0, (int) xf.size(), xf.data());
    mf.setSignal(1, (int) x2f.size(), x2f.data());
    mf.apply();
    std::vector<double> bd(b.size()), b2d(b2.size()), xd(xf.begin(), xf.end()), x2d(x2f.begin(), x2f.end());
    for (size_t i = 0; i < b.size(); ++i) { bd[i] = (float) b[i]; b2d[i] = (float) b2[i]; }
    const double e0 = max_err(mf.getMatchedFilteredSignal(0), pearson(bd, xd));
    const double e1 = max_err(mf.getMatchedFilteredSignal(1), pearson(b2d, x2d));
    require(e0 < 2e-6 && e1 < 2e-6, "FP32 vs two-pass Pearson (" + std::to_string(std::max(e0, e1)) + ")");
}

// extension: a window read from the device ring equals the same samples set
// from the host
void test_signal_ring()
{
    std::vector<double> x, x2, b, b2;
    damped(x, x2, b, b2);
    const int n = 400;
    MFLib::MatchedFilterParameters p;
    p.addTemplate(make_template(b, 1.0));
    p.addTemplate(make_template(b2, 1.0));
    p.setSignalSize(n);
    MFLib::MatchedFilter<double> mf;
    mf.initialize(p);
    const long cap = 700;
    MFLib::SignalRing<double> ring(2, cap);
    const int total = (int) x.size();
    std::vector<double> rows(2 * (size_t) total);
    for (int i = 0; i < total; ++i) { rows[i] = x[i]; rows[total + i] = x2[i]; }
    for (int a = 0; a < total; a += 130)
    {
        const int k = std::min(130, total - a);
        std::vector<double> chunk(2 * (size_t) k);
        for (int i = 0; i < k; ++i) { chunk[i] = rows[a + i]; chunk[k + i] = rows[total + a + i]; }
        ring.append(k, chunk.data(), k);
    }
    require(ring.getHead() == total, "ring head counts every appended sample");
    const long long end = total - 37;
    mf.setWindowFromRing(ring, {1, 0}, end, n);
    mf.apply();
    const std::vector<double> r0 = mf.getMatchedFilteredSignal(0), r1 = mf.getMatchedFilteredSignal(1);
    mf.setSignal(0, n, rows.data() + total + (end - n));
    mf.setSignal(1, n, rows.data() + (end - n));
    mf.apply();
    require(r0 == mf.getMatchedFilteredSignal(0) && r1 == mf.getMatchedFilteredSignal(1),
            "ring window equals the same samples set from the host");
    require(throws_invalid([&] { mf.setWindowFromRing(ring, {0}, end - cap, n); }),
            "a window no longer in the ring is refused");
}

void test_single_channel()
{
    // testing/singleChannel.cpp:104-160: one signal, three templates cut from it
    std::mt19937_64 g(7);
    std::uniform_real_distribution<double> u(2, 3);
    std::vector<double> wave(4000);
    for (double &v : wave) v = u(g);
    const int cuts[3][2] = {{25, 155}, {1124, 1264}, {3601, 3726}};
    MFLib::SingleChannel::MatchedFilterParameters p;
    std::vector<std::vector<double>> tps;
    for (const auto &c : cuts)
    {
        tps.emplace_back(wave.begin() + c[0], wave.begin() + c[1]);
        p.addTemplate(make_template(tps.back(), 100.0));
    }
    p.setSignalSize((int) wave.size());
    require(p.getDetectionMode() == MFLib::MatchedFilterDetectionMode::SINGLE_CHANNEL, "single-channel mode");
    MFLib::SingleChannel::MatchedFilter<double> mf;
    mf.initialize(p);
    mf.setSignal((int) wave.size(), wave.data());
    mf.apply();
    for (int i = 0; i < 3; ++i)
    {
        std::vector<double> r = mf.getMatchedFilteredSignal(i);
        std::vector<double> ref = pearson(tps[i], wave);
        ref.resize(r.size());
        const double e = max_err(r, ref);
        require(e < 1e-12, "single-channel template " + std::to_string(i) + " (" + std::to_string(e) + ")");
        // the template's own position correlates perfectly
        require(std::abs(r[cuts[i][0]] - 1.0) < 1e-12, "single-channel self match " + std::to_string(i));
    }
}

void test_shift_and_stack()
{
    // three templates with onsets and travel times; the stack is the
    // weighted sum of |rho_t| shifted by round((travel - onset) * fs)
    std::mt19937_64 g(11);
    std::normal_distribution<double> nd;
    const double fs = 100;
    const int n = 6000, L = 200;
    std::vector<double> sig(n);
    for (double &v : sig) v = nd(g);
    MFLib::MatchedFilterParameters p;
    const double travel[3] = {1.0, 2.5, 4.0}, onset[3] = {0.5, 0.25, 1.0}, w[3] = {0.5, 0.3, 0.2};
    std::vector<std::vector<double>> tps;
    for (int t = 0; t < 3; ++t)
    {
        tps.emplace_back(sig.begin() + 1000 * (t + 1), sig.begin() + 1000 * (t + 1) + L);
        MFLib::WaveformTemplate wt = make_template(tps.back(), fs);
        wt.setPhaseOnsetTime(onset[t]);
        wt.setTravelTime(travel[t]);
        wt.setShiftAndStackWeight(w[t]);
        p.addTemplate(wt);
    }
    p.setSignalSize(n);
    MFLib::MatchedFilter<double> mf;
    mf.initialize(p);
    for (int t = 0; t < 3; ++t) mf.setSignal(t, n, sig.data());
    mf.apply();
    std::vector<double> stack = mf.shiftAndStack();
    std::vector<std::vector<double>> rho(3);
    int smax = 0;
    int sh[3];
    for (int t = 0; t < 3; ++t)
    {
        rho[t] = mf.getMatchedFilteredSignal(t);
        sh[t] = (int) ((travel[t] - onset[t]) * fs + 0.5);
        smax = std::max(smax, sh[t]);
    }
    const int m = (int) rho[0].size() - smax;
    double e = (int) stack.size() == m ? 0.0 : 1e30;
    for (int k = 0; k < m && e < 1; ++k)
    {
        double s = 0;
        for (int t = 0; t < 3; ++t) s += w[t] * std::abs(rho[t][k + sh[t]]);
        e = std::max(e, std::abs(s - stack[k]));
    }
    require(e < 1e-12, "shiftAndStack (" + std::to_string(e) + ")");
}

// testing/peakFinder.cpp:145-170
std::vector<double> gaussian_sine()
{
    const double tdur = 4, dt = 0.01, sigma = 1.2, freq = 12, pi = 3.14159265358979323846;
    const double t0 = -tdur / 2, t1 = tdur / 2;
    const int npts = (int) ((t1 - t0) / dt + 0.5) + 1;
    std::vector<double> y(npts);
    double mx = 0;
    for (int i = 0; i < npts; ++i)
    {
        const double t = t0 + i * dt, a = (t / sigma) * (t / sigma);
        y[i] = std::exp(-a * a) * std::cos(2 * pi * (t - t0) / tdur * freq);
        mx = std::max(mx, std::abs(y[i]));
    }
    for (double &v : y) v /= mx;
    y.front() = 0;
    y.back() = 0;
    return y;
}

void test_peak_finder()
{
    // testing/peakFinder.cpp:16-143
    const int n = 4000;
    std::vector<double> tp = gaussian_sine(), sig(n, 0.0);
    const int ih = (int) tp.size() / 2;
    for (int i = 0; i < (int) tp.size() - ih; ++i) sig[i] = tp[ih + i];
    for (double frac : {0.25, 0.5, 0.75})
    {
        const int i1 = (int) (n * frac) - ih;
        for (size_t i = 0; i < tp.size(); ++i) sig[i1 + i] = tp[i];
    }
    for (int i = 0; i < ih; ++i) sig[n - ih + i] = tp[1 + i];
    MFLib::PeakFinder<double> pf;
    require(throws_invalid([&] { pf.setThreshold(1.5); }), "PeakFinder threshold outside [0,1] throws");
    std::vector<double> flat(n, 0.4);
    pf.setThreshold(0.8);
    pf.setMinimumPeakDistance(52);
    pf.setSignal(n, flat.data());
    pf.apply();
    require(pf.getNumberOfPeaks() == 0 && pf.getPeakIndicesPointer() == nullptr, "no peaks below threshold");
    const std::vector<int> p13 = {0, 67, 933, 1000, 1067, 1933, 2000, 2067, 2933, 3000, 3067, 3932, 3999};
    const std::vector<int> p21 = {0,    33,   67,   933,  967,  1000, 1033, 1067, 1933, 1967, 2000,
                                  2033, 2067, 2933, 2967, 3000, 3033, 3067, 3932, 3966, 3999};
    pf.setMinimumPeakDistance((int) (0.5 / 0.01 + 1) + 1);
    pf.setSignal(n, sig.data());
    pf.apply();
    std::vector<int> got(pf.getNumberOfPeaks());
    int *gp = got.data();
    if (!got.empty()) pf.getPeakIndices((int) got.size(), &gp);
    require(got == p13, "PeakFinder 13 peaks with separation 52");
    pf.setMinimumPeakDistance(0);
    pf.apply();
    got.assign(pf.getNumberOfPeaks(), 0);
    gp = got.data();
    if (!got.empty()) pf.getPeakIndices((int) got.size(), &gp);
    require(got == p21, "PeakFinder 21 peaks without separation");
}

void test_dbscan()
{
    // testing/dbscan.cpp:8-60
    const double X[12] = {1, 2, 2, 2, 2, 2, 8, 7, 8, 8, 25, 80};
    MFLib::DBSCAN db;
    require(!db.isInitialized(), "DBSCAN not initialised");
    db.initialize(3, 2);
    db.setData(6, 2, X);
    db.cluster();
    require(db.haveLabels() && db.getNumberOfClusters() == 2, "DBSCAN 2 clusters");
    require(db.getLabels() == std::vector<int>({0, 0, 0, 1, 1, -1}), "DBSCAN labels with one noise point");
    db.setData(5, 2, X);
    db.cluster();
    require(db.getLabels() == std::vector<int>({0, 0, 0, 1, 1}), "DBSCAN labels without noise");
}

void test_value_types()
{
    MFLib::NetworkStationPhase a, b;
    a.setNetwork("uu ");
    a.setStation("fo r");
    b.setNetwork("UU");
    b.setStation("FOR");
    require(a == b && a.getHash() == b.getHash() && a.getStation() == "FOR", "NetworkStationPhase canonical form");
    MFLib::WaveformTemplate wt;
    require(throws_runtime([&] { wt.getSignalLength(); }), "WaveformTemplate without a signal throws");
    require(throws_invalid([&] { wt.setSamplingRate(-1); }), "negative sampling rate throws");
    require(throws_runtime([&] { wt.setTravelTime(-1); }), "negative travel time throws runtime_error");
    MFLib::MatchedFilterParameters p;
    require(!p.isValid(), "empty parameters invalid");
    require(throws_invalid([&] { p.addTemplate(wt); }), "template without a signal rejected");
}

// The detector on a signal holding exact copies of two templates at known
// samples: REDUCED and SINGLE policies find each copy with coefficient 1 at
// its sample, the quadratic refinement of a self match stays within a sample,
// the polarity follows the template's, the amplitude of a copy scaled by 3 is
// 3 (Gibbons-Ringdal and Schaff-Richards).
void test_detector()
{
    const int n = 6000, L = 150;
    std::vector<double> x(n), t0(L), t1(L);
    unsigned s = 7;
    auto rnd = [&] {
        s = s * 1664525u + 1013904223u;
        return ((s >> 8) & 0xFFFF) / 65536.0 - 0.5;
    };
    for (double &v : x) v = 0.1 * rnd();
    for (int i = 0; i < L; ++i)
    {
        t0[i] = std::sin(0.21 * i) * std::exp(-0.01 * i) + 0.05 * rnd();
        t1[i] = std::cos(0.37 * i) * std::exp(-0.02 * i) + 0.05 * rnd();
    }
    const int at0 = 1000, at1 = 3500;
    for (int i = 0; i < L; ++i)
    {
        x[at0 + i] = 3.0 * t0[i];
        x[at1 + i] = -2.0 * t1[i];
    }
    MFLib::SingleChannel::MatchedFilterParameters p;
    for (const auto *t : {&t0, &t1})
    {
        MFLib::WaveformTemplate wt;
        wt.setSignal(L, t->data());
        wt.setSamplingRate(100.0);
        wt.setPolarity(MFLib::Polarity::COMPRESSION);
        wt.setPhaseOnsetTime(0.0);
        p.addTemplate(wt);
    }
    p.setSignalSize(n);
    MFLib::SingleChannel::MatchedFilter<double> mf;
    mf.initialize(p);
    mf.setSignal(n, x.data());
    mf.apply();
    for (auto policy : {MFLib::MatchedFilteredSignalDetectorPolicy::REDUCED,
                        MFLib::MatchedFilteredSignalDetectorPolicy::SINGLE})
    {
        MFLib::SingleChannel::DetectorParameters dp;
        dp.setDetectionThreshold(0.95);
        dp.setMinimumDetectionSpacing(100);
        dp.setMaximaPolicy(MFLib::MaximumMatchedFilterPolicy::ABSOLUTE_MAXIMUM);
        dp.setMatchedFilteredSignalDetectorPolicy(policy);
        MFLib::SingleChannel::Detector<double> det;
        det.initialize(dp);
        det.detect(mf);
        require(det.getNumberOfDetections() == 2, "detector: two detections");
        auto a = det.getDetection(0), b = det.getDetection(1);
        require(std::abs(a.getDetectionTime() - at0 / 100.0) < 1e-12 && a.getTemplateIdentifier().second == 0,
                "detector: first copy at its sample, template 0");
        require(std::abs(b.getDetectionTime() - at1 / 100.0) < 1e-12 && b.getTemplateIdentifier().second == 1,
                "detector: second copy at its sample, template 1");
        require(std::abs(a.getCorrelationCoefficient() - 1.0) < 1e-9 &&
                    std::abs(b.getCorrelationCoefficient() + 1.0) < 1e-9,
                "detector: coefficients +1 and -1");
        require(std::abs(a.getInterpolatedDetectionTime() - a.getDetectionTime()) <= 0.01,
                "detector: refinement within a sample");
        require(a.getPolarity() == MFLib::Polarity::COMPRESSION && b.getPolarity() == MFLib::Polarity::DILATATION,
                "detector: polarity from the coefficient's sign");
        require(std::abs(a.getAmplitudeScalingFactor(MFLib::RelativeMagnitudeType::GIBBONS_RINGDAL_2006) - 3.0) < 1e-9 &&
                    std::abs(a.getAmplitudeScalingFactor(MFLib::RelativeMagnitudeType::SCHAFF_RICHARDS_2014) - 3.0) < 1e-9,
                "detector: amplitude scaling factors of a copy scaled by 3");
        require(std::abs(a.getPhaseOnsetTime() - a.getDetectionTime()) < 1e-12, "detector: phase onset time");
        require(det.getMatchedFilteredSignalLength() == n - L + 1, "detector: matched-filtered signal length");
        require(a.haveMagnitudePerturbation(MFLib::RelativeMagnitudeType::GIBBONS_RINGDAL_2006) &&
                    std::abs(a.getMagnitudePerturbation(MFLib::RelativeMagnitudeType::GIBBONS_RINGDAL_2006) -
                             std::log10(3.0)) < 1e-9,
                "detector: magnitude perturbation log10(3)");
    }
    // the relative magnitude of a scaled, offset copy of template 0
    MFLib::WaveformTemplate wt;
    wt.setSignal(L, t0.data());
    MFLib::SingleChannel::RelativeMagnitude<double> rm;
    require(throws_runtime([&] { rm.getDetectedSignalLength(); }), "relative magnitude: not initialised");
    rm.initialize(wt);
    std::vector<double> y(L);
    for (int i = 0; i < L; ++i) y[i] = 2.5 * t0[i] + 7.0;
    rm.setDetectedSignal(L, y.data());
    const double gr = rm.computeAmplitudeScalingFactor(MFLib::RelativeMagnitudeType::GIBBONS_RINGDAL_2006);
    const double sr = rm.computeAmplitudeScalingFactor(MFLib::RelativeMagnitudeType::SCHAFF_RICHARDS_2014);
    require(std::abs(gr - 2.5) < 1e-12 && std::abs(sr - 2.5) < 1e-12, "relative magnitude: both factors 2.5");
    require(std::abs(rm.computeMagnitudePerturbation(MFLib::RelativeMagnitudeType::SCHAFF_RICHARDS_2014) -
                     std::log10(2.5)) < 1e-12,
            "relative magnitude: perturbation log10(2.5)");
    std::vector<double> flat(L, 4.0);
    require(throws_invalid([&] { rm.setDetectedSignal(L, flat.data()); }), "relative magnitude: constant window rejected");
    require(throws_invalid([&] { rm.setDetectedSignal(L - 1, y.data()); }), "relative magnitude: wrong length rejected");
    require(throws_invalid([&] { MFLib::SingleChannel::convertAmplitudeScalingFactorToMagnitudePerturbation(0.0); }),
            "non-positive scaling factor rejected");
}

// Associator: detections grouped by their template id, origin times (onset -
// travel time) clustered within the tolerance, isolated picks left out.
void test_associator()
{
    using D = MFLib::SingleChannel::Detection<double>;
    auto make = [](uint64_t id, double onset, double travel, double xc) {
        D d;
        d.setTemplateIdentifier({MFLib::NetworkStationPhase(), id});
        d.setPhaseOnsetTime(onset);
        d.setTravelTime(travel);
        d.setCorrelationCoefficient(xc);
        return d;
    };
    MFLib::SingleChannel::AssociatorParameters ap;
    ap.setOriginTimeTolerance(1.0);
    ap.setMinimumNumberOfPicksInEvent(2);
    MFLib::SingleChannel::Associator<double> as;
    require(throws_runtime([&] { as.addDetection(make(1, 0, 0, 0.5)); }), "associator: not initialised");
    as.initialize(ap);
    // id 2: origins 100.0, 100.4, 160 (noise); id 1: origins 20.1, 20.5, 20.9, 75 (noise)
    as.addDetection(make(2, 103.0, 3.0, 0.8));
    as.addDetection(make(1, 24.1, 4.0, 0.9));
    as.addDetection(make(2, 102.4, 2.0, 0.7));
    as.addDetection(make(1, 75.0, 0.0, 0.6));
    as.addDetection(make(1, 21.5, 1.0, 0.8));
    as.addDetection(make(2, 160.0, 0.0, 0.9));
    as.addDetection(make(1, 22.9, 2.0, 0.5));
    D bad;
    bad.setTemplateIdentifier({MFLib::NetworkStationPhase(), 3});
    require(throws_invalid([&] { as.addDetection(bad); }), "associator: travel time required");
    as.associate();
    require(as.getNumberOfDetections() == 7 && as.getNumberOfEvents() == 2, "associator: two events");
    const auto e0 = as.getDetectionsInEvent(0), e1 = as.getDetectionsInEvent(1);
    require(e0.size() == 3 && e0[0].getTemplateIdentifier().second == 1 &&
                std::abs(e0[0].getPhaseOnsetTime() - e0[0].getTravelTime() - 20.5) < 1e-12,
            "associator: first event is id 1's three picks, by onset time");
    require(e1.size() == 2 && e1[0].getTemplateIdentifier().second == 2, "associator: second event is id 2's pair");
    require(throws_invalid([&] { as.getDetectionsInEvent(2); }), "associator: event index checked");
    ap.enableCorrelationCoefficientWeighting();
    ap.setMinimumNumberOfPicksInEvent(3);
    MFLib::SingleChannel::Associator<double> aw;
    aw.initialize(ap);
    // id 5: four picks of weight 0.9 (sum 3.6 >= 3) form an event; id 6:
    // two of 0.95 (1.9) do not
    for (const D &d : {make(5, 10.0, 0, 0.9), make(5, 10.3, 0, 0.9), make(5, 10.6, 0, 0.9), make(5, 10.2, 0, 0.9),
                       make(6, 40.0, 0, 0.95), make(6, 40.5, 0, 0.95)})
        aw.addDetection(d);
    aw.associate();
    require(aw.getNumberOfEvents() == 1 && aw.getDetectionsInEvent(0).size() == 4,
            "associator: weighted picks need a weight sum of 3");
}

}  // namespace

int main()
{
    std::setvbuf(stdout, nullptr, _IONBF, 0);
    int ndev = 0;
    if (mfgpu_device_count(&ndev) != MFGPU_OK || ndev < 1)
    {
        std::printf("no CUDA device\n");
        return 2;
    }
    try
    {
        test_fft_sizes();
        test_value_types();
        test_multichannel_double();
        test_multichannel_float();
        test_signal_ring();
        test_single_channel();
        test_shift_and_stack();
        test_peak_finder();
        test_dbscan();
        test_detector();
        test_associator();
    }
    catch (const std::exception &e)
    {
        std::printf("FAIL: unexpected exception after %d checks: %s\n", g_checks, e.what());
        return 1;
    }
    std::printf("ALL PASSED (%d checks)\n", g_checks);
    return 0;
}
