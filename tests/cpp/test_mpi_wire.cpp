// MFLib::MPI of include/mfgpu_mpi.hpp over the in-process MPI stand-in
// (tests/cpp/fake_mpi/mpi.h): records round-trip every field of a
// detection, Send / Recv (a named source and MPI_ANY_SOURCE), Broadcast from
// a non-zero root over a template that had other fields, Gather to either
// rank, and an MPI failure surfacing as std::runtime_error.  With a
// directory argument it also writes the wire bytes of one fixed detection
// and one fixed template there, for comparison with the Python module's
// bytes.  Prints one line per check and "ALL PASSED"; exits non-zero on the
// first failure.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "mfgpu_mpi.hpp"

using namespace MFLib;
using SingleChannel::Detection;

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

NetworkStationPhase nsp(const std::string &net, const std::string &sta, const std::string &pha,
                        const std::string &cha = "", const std::string &loc = "")
{
    NetworkStationPhase n;
    n.setNetwork(net);
    n.setStation(sta);
    n.setPhase(pha);
    n.setChannel(cha);
    n.setLocationCode(loc);
    return n;
}

// the fixed detection whose record bytes the Python module must reproduce
template <class T> Detection<T> fixedDetection()
{
    Detection<T> d;
    d.setTemplateIdentifier({nsp("uu", "ctu", "p"), 12345678901234ull});
    d.setCorrelationCoefficient(0.625);
    d.setDetectionTime(101.25);
    d.setInterpolatedDetectionTime(101.3125);
    d.setTravelTime(7.5);
    d.setAmplitudeScalingFactor((T) 2.5, RelativeMagnitudeType::GIBBONS_RINGDAL_2006);
    d.setPolarity(Polarity::DILATATION);
    const T x[3] = {(T) 0.5, (T) -1.25, (T) 2.0};
    d.setDetectedSignal(3, x);
    return d;
}

WaveformTemplate fixedTemplate()
{
    WaveformTemplate t;
    const double x[4] = {1.0, -2.0, 3.5, 0.25};
    t.setSignal(4, x);
    t.setSamplingRate(100.0);
    t.setShiftAndStackWeight(0.5);
    t.setPhaseOnsetTime(0.0);
    t.setTravelTime(3.0);
    t.setMagnitude(1.5);
    t.setPolarity(Polarity::COMPRESSION);
    t.setIdentifier({nsp("uu", "ctu", "p", "ehz", "01"), 42});
    return t;
}

template <class T> Detection<T> variedDetection(int i)
{
    Detection<T> d;
    if (i % 2 == 0) d.setTemplateIdentifier({nsp("uu", "st" + std::to_string(i), i % 4 ? "p" : "s"), 1000u + i});
    if (i % 3 != 1) d.setCorrelationCoefficient(-0.9 + 0.15 * i);
    if (i % 3 != 2)
    {
        std::vector<T> x(1 + 3 * i);
        for (size_t k = 0; k < x.size(); ++k) x[k] = (T) (0.25 * k - i);
        d.setDetectedSignal((int) x.size(), x.data());
    }
    d.setDetectionTime(10.0 * i + 0.5);
    if (i % 2)
    {
        d.setInterpolatedDetectionTime(10.0 * i + 0.625);
        d.setPhaseOnsetTime(0.0);
        d.setAmplitudeScalingFactor((T) (0.5 + i), RelativeMagnitudeType::GIBBONS_RINGDAL_2006);
    }
    else
    {
        d.setInterpolatedPhaseOnsetTime(10.0 * i + 0.75);
        d.setTravelTime(1.5 * i);
        d.setAmplitudeScalingFactor((T) (0.25 + i), RelativeMagnitudeType::SCHAFF_RICHARDS_2014);
    }
    d.setPolarity(i % 3 == 0 ? Polarity::COMPRESSION : (i % 3 == 1 ? Polarity::DILATATION : Polarity::UNKNOWN));
    return d;
}

template <class T> bool same(const Detection<T> &a, const Detection<T> &b)
{
    auto eq = [](bool ha, bool hb, double va, double vb) { return ha == hb && (!ha || va == vb); };
    if (a.haveTemplateIdentifier() != b.haveTemplateIdentifier()) return false;
    if (a.haveTemplateIdentifier() && a.getTemplateIdentifier() != b.getTemplateIdentifier()) return false;
    if (a.haveDetectedSignal() != b.haveDetectedSignal()) return false;
    if (a.haveDetectedSignal())
    {
        if (a.getDetectedSignalLength() != b.getDetectedSignalLength()) return false;
        for (int k = 0; k < a.getDetectedSignalLength(); ++k)
            if (a.getDetectedSignalPointer()[k] != b.getDetectedSignalPointer()[k]) return false;
    }
    for (auto t : {RelativeMagnitudeType::GIBBONS_RINGDAL_2006, RelativeMagnitudeType::SCHAFF_RICHARDS_2014})
        if (!eq(a.haveAmplitudeScalingFactor(t), b.haveAmplitudeScalingFactor(t),
                a.haveAmplitudeScalingFactor(t) ? a.getAmplitudeScalingFactor(t) : 0,
                b.haveAmplitudeScalingFactor(t) ? b.getAmplitudeScalingFactor(t) : 0))
            return false;
#define SAME_FIELD(H, G) \
    if (!eq(a.H(), b.H(), a.H() ? a.G() : 0, b.H() ? b.G() : 0)) return false;
    SAME_FIELD(haveCorrelationCoefficient, getCorrelationCoefficient)
    SAME_FIELD(haveDetectionTime, getDetectionTime)
    SAME_FIELD(haveInterpolatedDetectionTime, getInterpolatedDetectionTime)
    SAME_FIELD(havePhaseOnsetTime, getPhaseOnsetTime)
    SAME_FIELD(haveInterpolatedPhaseOnsetTime, getInterpolatedPhaseOnsetTime)
    SAME_FIELD(haveTravelTime, getTravelTime)
#undef SAME_FIELD
    return a.getPolarity() == b.getPolarity();
}

bool sameTemplate(const WaveformTemplate &a, const WaveformTemplate &b)
{
    if (a.samples() != b.samples() || a.haveSamplingRate() != b.haveSamplingRate()) return false;
    if (a.haveSamplingRate() && a.getSamplingRate() != b.getSamplingRate()) return false;
    if (a.getShiftAndStackWeight() != b.getShiftAndStackWeight()) return false;
    if (a.havePhaseOnsetTime() != b.havePhaseOnsetTime() ||
        (a.havePhaseOnsetTime() && a.getPhaseOnsetTime() != b.getPhaseOnsetTime()))
        return false;
    if (a.haveTravelTime() != b.haveTravelTime() || (a.haveTravelTime() && a.getTravelTime() != b.getTravelTime()))
        return false;
    if (a.haveMagnitude() != b.haveMagnitude() || (a.haveMagnitude() && a.getMagnitude() != b.getMagnitude()))
        return false;
    if (a.haveIdentifier() != b.haveIdentifier() || (a.haveIdentifier() && a.getIdentifier() != b.getIdentifier()))
        return false;
    return a.getPolarity() == b.getPolarity();
}

template <class T> void roundTrips(const char *name)
{
    for (int i = 0; i < 9; ++i)
    {
        const Detection<T> d = variedDetection<T>(i);
        const MPI::DetectionRecord r = MPI::toRecord(d);
        Detection<T> e = variedDetection<T>(i + 1);  // other fields, cleared by fromRecord
        MPI::fromRecord<T>(r, d.haveDetectedSignal() ? d.getDetectedSignalPointer() : nullptr, &e);
        require(same(d, e), std::string(name) + " record round trip " + std::to_string(i));
    }
    Detection<T> d;
    d.setTemplateIdentifier({nsp(std::string(70, 'n'), "sta", "p", "ehz", "01"), 7});
    Detection<T> e;
    MPI::fromRecord<T>(MPI::toRecord(d), nullptr, &e);
    const auto id = e.getTemplateIdentifier();
    require(id.first.getNetwork() == std::string(64, 'N') && id.first.getStation() == "STA" &&
                id.first.getChannel().empty() && id.first.getLocationCode().empty() && id.second == 7,
            std::string(name) + " names truncated to 64 bytes; channel and location code not in the record");
    MPI::DetectionRecord bad = MPI::toRecord(d);
    bad.polarity = 77;
    MPI::fromRecord<T>(bad, nullptr, &e);
    require(e.getPolarity() == Polarity::UNKNOWN, std::string(name) + " a polarity byte outside -1, 0, 1 reads as unknown");
}

template <class T> void transport(const char *name)
{
    FakeWorld w(2);
    FakeComm c0{&w, 0}, c1{&w, 1};
    const Detection<T> a = variedDetection<T>(0), b = variedDetection<T>(1), nosig = variedDetection<T>(2);
    MPI::Send(a, 0, 5, &c1);
    MPI::Send(b, 0, 6, &c1);
    MPI::Send(nosig, 0, 6, &c1);
    Detection<T> ra, rb, rn;
    MPI_Status st;
    MPI::Recv(&rb, 1, 6, &c0, &st);
    require(same(b, rb) && st.MPI_SOURCE == 1 && st.MPI_TAG == 6, std::string(name) + " Send / Recv by tag");
    MPI::Recv(&ra, MPI_ANY_SOURCE, 5, &c0, &st);
    require(same(a, ra) && st.MPI_SOURCE == 1, std::string(name) + " Recv from MPI_ANY_SOURCE");
    MPI::Recv(&rn, 1, 6, &c0, MPI_STATUS_IGNORE);
    require(same(nosig, rn) && !rn.haveDetectedSignal(), std::string(name) + " detection without a signal");
    require(w.p2p[0].empty(), std::string(name) + " every message consumed");

    // gather to rank 1, then to rank 0 (non-root ranks call first)
    std::vector<Detection<T>> l0 = {variedDetection<T>(3), variedDetection<T>(4), variedDetection<T>(5)};
    std::vector<Detection<T>> l1 = {variedDetection<T>(6), variedDetection<T>(7)};
    require(MPI::Gather(l0, 1, &c0).empty(), std::string(name) + " Gather returns nothing off the root");
    const auto g1 = MPI::Gather(l1, 1, &c1);
    bool ok = g1.size() == 5;
    for (size_t i = 0; ok && i < 5; ++i) ok = same(g1[i], i < 3 ? l0[i] : l1[i - 3]);
    require(ok, std::string(name) + " Gather to rank 1 in rank order");
    MPI::Gather(std::vector<Detection<T>>(), 0, &c1);
    const auto g0 = MPI::Gather(l0, 0, &c0);
    ok = g0.size() == 3;
    for (size_t i = 0; ok && i < 3; ++i) ok = same(g0[i], l0[i]);
    require(ok && w.coll[0].empty() && w.coll[1].empty(), std::string(name) + " Gather with an empty rank");

    w.fail_after = 1;
    bool threw = false;
    try { MPI::Send(a, 0, 5, &c1); } catch (const std::runtime_error &) { threw = true; }
    require(threw, std::string(name) + " an MPI failure throws std::runtime_error");
}

void broadcast()
{
    FakeWorld w(3);
    FakeComm c[3] = {{&w, 0}, {&w, 1}, {&w, 2}};
    WaveformTemplate root = fixedTemplate(), r0, r2;
    const double junk[2] = {9, 9};
    r0.setSignal(2, junk);
    r0.setSamplingRate(40);
    r0.setMagnitude(3);
    MPI::Broadcast(root, 1, &c[1]);
    MPI::Broadcast(r0, 1, &c[0]);
    MPI::Broadcast(r2, 1, &c[2]);
    require(sameTemplate(root, fixedTemplate()), "Broadcast leaves the root's template");
    require(sameTemplate(r0, root) && sameTemplate(r2, root), "Broadcast from rank 1 (onset 0, all five names)");
    WaveformTemplate bare, got;
    MPI::Broadcast(bare, 0, &c[0]);
    MPI::Broadcast(got = fixedTemplate(), 0, &c[1]);
    WaveformTemplate got2;
    MPI::Broadcast(got2, 0, &c[2]);
    require(sameTemplate(got, bare) && sameTemplate(got2, bare) && !got.haveSignal() && !got.haveIdentifier() &&
                !got.haveMagnitude() && got.getShiftAndStackWeight() == 1,
            "Broadcast of an empty template clears the others");
}

void writeBytes(const std::string &path, const void *p, size_t n)
{
    std::ofstream f(path, std::ios::binary);
    f.write((const char *) p, (std::streamsize) n);
}

void dumpFixed(const std::string &dir)
{
    const MPI::DetectionRecord r = MPI::toRecord(fixedDetection<double>());
    writeBytes(dir + "/detection.bin", &r, sizeof(r));
    FakeWorld w(2);
    FakeComm c1{&w, 1};
    WaveformTemplate t = fixedTemplate();
    MPI::Broadcast(t, 1, &c1);
    const char *names[3] = {"/template_header.bin", "/template_strings.bin", "/template_samples.bin"};
    for (int i = 0; i < 3; ++i)
    {
        writeBytes(dir + names[i], w.coll[0].front().bytes.data(), w.coll[0].front().bytes.size());
        w.coll[0].pop_front();
    }
    require(w.coll[0].empty(), "fixed wire bytes written");
}

}  // namespace

int main(int argc, char **argv)
{
    roundTrips<double>("double");
    roundTrips<float>("float");
    transport<double>("double");
    transport<float>("float");
    broadcast();
    if (argc > 1) dumpFixed(argv[1]);
    std::printf("%d checks\nALL PASSED\n", g_checks);
    return 0;
}
