// The host-side classes of include/mfgpu.hpp (no GPU, no library calls),
// checked the way the reference's own C++ tests check them:
//   NetworkStationPhase            testing/networkStationPhase.cpp:10-45
//   WaveformTemplate               testing/waveformTemplate.cpp:10-90
//   SingleChannel::Detection       testing/detection.cpp:15-135
//   DetectionTimeInterpolationParameters, DetectorParameters
//                                  testing/detector.cpp:29-98
//   SingleChannel::AssociatorParameters
//                                  testing/associator.cpp:18-34
// Prints one line per check and "ALL PASSED"; exits non-zero on the first
// failure.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "mfgpu.hpp"

using namespace MFLib;

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

void networkStationPhase()
{
    NetworkStationPhase a;
    a.setNetwork(" uU ");
    a.setStation(" DuG  ");
    a.setChannel("HHz");
    a.setLocationCode(" 01 ");
    a.setPhase(" s");
    require(a.getNetwork() == "UU" && a.getStation() == "DUG" && a.getChannel() == "HHZ" &&
                a.getLocationCode() == "01" && a.getPhase() == "S",
            "NetworkStationPhase: blanks removed, upper case");
    NetworkStationPhase b(a);
    require(a == b && a.getHash() == b.getHash(), "NetworkStationPhase: copies compare equal");
    b.setPhase("P");
    require(!(a == b), "NetworkStationPhase: a changed phase compares unequal");
    a.clear();
    b.clear();
    require(a == b && a.getNetwork().empty(), "NetworkStationPhase: cleared objects compare equal");
}

void waveformTemplate()
{
    WaveformTemplate t;
    NetworkStationPhase nsp;
    nsp.setNetwork("UU");
    nsp.setStation("BSUT");
    nsp.setChannel("EHZ");
    nsp.setLocationCode("01");
    nsp.setPhase("P");
    const std::pair<NetworkStationPhase, uint64_t> id(nsp, 942);
    t.setSamplingRate(10);
    t.setTravelTime(3);
    t.setMagnitude(4);
    t.setIdentifier(id);
    t.setPolarity(Polarity::COMPRESSION);
    require(t.getSamplingRate() == 10 && t.getTravelTime() == 3 && t.getMagnitude() == 4 &&
                t.getIdentifier() == id && t.getPolarity() == Polarity::COMPRESSION,
            "WaveformTemplate: scalar fields");
    require(t.getShiftAndStackWeight() == 1, "WaveformTemplate: default weight 1");
    t.setShiftAndStackWeight(0.5);
    require(t.getShiftAndStackWeight() == 0.5 && throws_invalid([&] { t.setShiftAndStackWeight(1.5); }),
            "WaveformTemplate: weight in [0, 1]");
    require(!t.haveSignal() && throws_invalid([&] { t.setSamplingRate(0); }), "WaveformTemplate: no signal yet; fs > 0");
    double x8[10];
    for (int i = 0; i < 10; ++i) x8[i] = i + 1;
    t.setSignal(10, x8);
    t.setPhaseOnsetTime(0.2);
    require(t.haveSignal() && t.getSignalLength() == 10 && std::abs(t.getPhaseOnsetTime() - 0.2) < 1e-14,
            "WaveformTemplate: signal and onset time");
    double back[10] = {0};
    double *bp = back;
    t.getSignal(10, &bp);
    bool ok = true;
    for (int i = 0; i < 10; ++i) ok = ok && back[i] == i + 1;
    require(ok, "WaveformTemplate: FP64 samples returned");
    float x4[10];
    for (int i = 0; i < 10; ++i) x4[i] = (float) -(i + 1);
    t.setSignal(10, x4);
    require(!t.havePhaseOnsetTime(), "WaveformTemplate: a new signal clears the onset time");
    t.setPhaseOnsetTime(0.2);
    float b4[10] = {0};
    float *b4p = b4;
    t.getSignal(10, &b4p);
    ok = true;
    for (int i = 0; i < 10; ++i) ok = ok && b4[i] == (float) -(i + 1);
    require(ok && throws_invalid([&] { t.getSignal(9, &b4p); }), "WaveformTemplate: FP32 samples; short buffer refused");
    const WaveformTemplate c(t);
    require(c.getShiftAndStackWeight() == 0.5 && c.getSamplingRate() == 10 && c.getTravelTime() == 3 &&
                c.getPhaseOnsetTime() == t.getPhaseOnsetTime() && c.getSignalLength() == 10 && c.getMagnitude() == 4 &&
                c.getIdentifier() == id && c.getPolarity() == Polarity::COMPRESSION,
            "WaveformTemplate: copy");
}

void detection()
{
    using SingleChannel::Detection;
    Detection<double> d;
    auto empty = [](const Detection<double> &e) {
        return !e.haveCorrelationCoefficient() && !e.haveTemplateIdentifier() && !e.haveDetectedSignal() &&
               !e.haveDetectionTime() && !e.haveInterpolatedDetectionTime() && !e.havePhaseOnsetTime() &&
               !e.haveInterpolatedPhaseOnsetTime() && !e.haveTravelTime() &&
               !e.haveAmplitudeScalingFactor(RelativeMagnitudeType::GIBBONS_RINGDAL_2006) &&
               !e.haveAmplitudeScalingFactor(RelativeMagnitudeType::SCHAFF_RICHARDS_2014) &&
               e.getPolarity() == Polarity::UNKNOWN;
    };
    require(empty(d), "Detection: nothing set at construction");
    NetworkStationPhase nsp;
    nsp.setNetwork("PB");
    nsp.setStation("B206");
    nsp.setPhase("S");
    std::vector<double> sig(10);
    for (int i = 0; i < 10; ++i) sig[i] = i + 1;
    d.setCorrelationCoefficient(0.8);
    d.setTemplateIdentifier({nsp, 20});
    d.setDetectedSignal(10, sig.data());
    d.setDetectionTime(1);
    d.setInterpolatedDetectionTime(2);
    d.setPhaseOnsetTime(3);
    d.setTravelTime(2);
    d.setInterpolatedPhaseOnsetTime(4);
    d.setAmplitudeScalingFactor(10, RelativeMagnitudeType::GIBBONS_RINGDAL_2006);
    d.setAmplitudeScalingFactor(100, RelativeMagnitudeType::SCHAFF_RICHARDS_2014);
    d.setPolarity(Polarity::DILATATION);
    const double mGR = SingleChannel::convertAmplitudeScalingFactorToMagnitudePerturbation(10.0);
    const double mSR = SingleChannel::convertAmplitudeScalingFactorToMagnitudePerturbation(100.0);
    require(std::abs(mGR - 1.0) < 1e-14 && std::abs(mSR - 2.0) < 1e-14,
            "convertAmplitudeScalingFactorToMagnitudePerturbation: log10");
    auto full = [&](const Detection<double> &e) {
        std::vector<double> back(10);
        double *bp = back.data();
        e.getDetectedSignal(10, &bp);
        return e.getCorrelationCoefficient() == 0.8 && e.getTemplateIdentifier().first == nsp &&
               e.getTemplateIdentifier().second == 20 && e.getDetectedSignalLength() == 10 && back == sig &&
               e.getDetectionTime() == 1 && e.getInterpolatedDetectionTime() == 2 && e.getPhaseOnsetTime() == 3 &&
               e.getTravelTime() == 2 && e.getInterpolatedPhaseOnsetTime() == 4 &&
               e.getAmplitudeScalingFactor(RelativeMagnitudeType::GIBBONS_RINGDAL_2006) == 10 &&
               e.getAmplitudeScalingFactor(RelativeMagnitudeType::SCHAFF_RICHARDS_2014) == 100 &&
               std::abs(e.getMagnitudePerturbation(RelativeMagnitudeType::GIBBONS_RINGDAL_2006) - mGR) < 1e-14 &&
               std::abs(e.getMagnitudePerturbation(RelativeMagnitudeType::SCHAFF_RICHARDS_2014) - mSR) < 1e-14 &&
               e.getPolarity() == Polarity::DILATATION;
    };
    require(full(d), "Detection: every field set and read back");
    const Detection<double> c(d);
    require(full(c), "Detection: copy");
    require(throws_invalid([&] { d.setCorrelationCoefficient(1.5); }), "Detection: coefficient outside [-1, 1] refused");
    d.clear();
    require(empty(d) && full(c), "Detection: clear empties only the cleared object");
}

void detectorParameters()
{
    SingleChannel::DetectionTimeInterpolationParameters ip;
    require(ip.getType() == DetectionTimeInterpolationType::QUADRATIC, "interpolation: quadratic by default");
    ip.enableLanczos();
    ip.setLanczosAlpha(21);
    ip.setLanczosNumberOfInterpolationPoints(50);
    const SingleChannel::DetectionTimeInterpolationParameters ipc(ip);
    require(ipc.getType() == DetectionTimeInterpolationType::LANCZOS && ipc.getLanczosAlpha() == 21 &&
                ipc.getLanczosNumberOfInterpolationPoints() == 50,
            "interpolation: Lanczos settings and copy");
    SingleChannel::DetectorParameters p;
    SingleChannel::DetectionTimeInterpolationParameters none;
    none.disable();
    p.setMinimumDetectionSpacing(50);
    p.setDetectionThreshold(0.8);
    p.setMaximaPolicy(MaximumMatchedFilterPolicy::ABSOLUTE_MAXIMUM);
    p.setDetectionTimeInterpolationParameters(none);
    p.setMatchedFilteredSignalDetectorPolicy(MatchedFilteredSignalDetectorPolicy::SINGLE);
    p.disableSaveDetectedWaveform();
    const bool noWave = !p.wantDetectedWaveform();
    p.enableSaveDetectedWaveform();
    p.disableSaveAmplitudeScalingFactor();
    const bool noAmp = !p.wantAmplitudeScalingFactor();
    p.enableSaveAmplitudeScalingFactor();
    require(noWave && noAmp, "detector parameters: waveform and amplitude switches");
    auto same = [](const SingleChannel::DetectorParameters &q) {
        return q.getMinimumDetectionSpacing() == 50 && std::abs(q.getDetectionThreshold() - 0.8) < 1e-14 &&
               q.getMaximaPolicy() == MaximumMatchedFilterPolicy::ABSOLUTE_MAXIMUM && q.wantDetectedWaveform() &&
               q.wantAmplitudeScalingFactor() &&
               q.getMatchedFilteredSignalDetectorPolicy() == MatchedFilteredSignalDetectorPolicy::SINGLE &&
               q.getDetectionTimeInterpolationParameters().getType() == DetectionTimeInterpolationType::NONE;
    };
    require(same(p), "detector parameters: every setting");
    const SingleChannel::DetectorParameters pc(p);
    require(same(pc), "detector parameters: copy");
    require(throws_invalid([&] { p.setDetectionThreshold(0); }) && throws_invalid([&] { p.setDetectionThreshold(1.1); }),
            "detector parameters: threshold in (0, 1]");
}

void associatorParameters()
{
    SingleChannel::AssociatorParameters p;
    require(!p.useCorrelationCoefficientWeighting(), "associator parameters: unweighted by default");
    p.setOriginTimeTolerance(4);
    p.setMinimumNumberOfPicksInEvent(8);
    p.enableCorrelationCoefficientWeighting();
    const SingleChannel::AssociatorParameters c(p);
    require(std::abs(c.getOriginTimeTolerance() - 4) < 1e-14 && c.getMinimumNumberOfPicksInEvent() == 8 &&
                c.useCorrelationCoefficientWeighting(),
            "associator parameters: settings and copy");
    require(throws_invalid([&] { p.setOriginTimeTolerance(-1); }) &&
                throws_invalid([&] { p.setMinimumNumberOfPicksInEvent(0); }),
            "associator parameters: negative tolerance and no picks refused");
}

}  // namespace

int main()
{
    networkStationPhase();
    waveformTemplate();
    detection();
    detectorParameters();
    associatorParameters();
    std::printf("%d checks\nALL PASSED\n", g_checks);
    return 0;
}
