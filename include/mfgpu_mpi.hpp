/*
 * mfgpu_mpi.hpp -- MFLib::MPI (include/mflib/mpi.hpp, src/mpi.cpp) for the
 * classes of mfgpu.hpp: Broadcast of a WaveformTemplate, Send / Recv of a
 * Detection<T>, and Gather, the one collective of the multi-rank path (every
 * rank's detections to one rank).  Header-only; include it where <mpi.h> is
 * available and link with the MPI library.  Every MPI failure throws
 * std::runtime_error (the reference's contract, include/mflib/mpi.hpp:24).
 *
 * Wire records (the same bytes as the Python module mflib_gb300.mpi):
 *   DetectionRecord  the reference's MPIDetection struct (src/mpi.cpp:20-51)
 *                    in its natural C layout, 280 bytes, sent as bytes and
 *                    followed by the detected signal (T) when it has one;
 *   TemplateHeader   a template's scalars with a presence flag for each
 *                    optional field, followed by the identifier's five
 *                    strings and the FP64 samples.
 * Differences from the reference, each deliberate: the record travels whole,
 * so the two have-amplitude flags arrive (src/mpi.cpp:95-96 lists the
 * amplitudes' offsets in their place); byte 278, padding in the reference
 * struct, carries the detection's polarity; a received detection or
 * template is cleared first and then holds exactly the sent fields; a
 * template's onset time of 0 travels (src/mpi.cpp:372 drops it); every rank
 * asks the communicator for its rank (src/mpi.cpp:299 passes the root's
 * rank in the communicator's place).  The channel and location code of a
 * detection's identifier are not in the record; network, station and phase
 * are, truncated to 64 bytes.
 */
#ifndef MFGPU_MPI_HPP
#define MFGPU_MPI_HPP

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include <mpi.h>

#include "mfgpu.hpp"

namespace MFLib
{
namespace MPI
{

struct DetectionRecord
{
    double amplitude1, amplitude2, correlationCoefficient, detectionTime;
    double interpolatedDetectionTime, phaseOnsetTime, interpolatedPhaseOnsetTime, travelTime;
    char network[64], station[64], phase[64];
    uint64_t templateID;
    int32_t signalLength;
    bool haveAmplitude1, haveAmplitude2, haveCorrelationCoefficient, haveDetectedSignal, haveDetectionTime,
        haveInterpolatedDetectionTime, havePhaseOnsetTime, haveInterpolatedPhaseOnsetTime, haveTravelTime,
        haveTemplateID;
    int8_t polarity;
};
static_assert(sizeof(DetectionRecord) == 280, "detection record is 280 bytes");
static_assert(offsetof(DetectionRecord, network) == 64 && offsetof(DetectionRecord, templateID) == 256 &&
                  offsetof(DetectionRecord, signalLength) == 264 && offsetof(DetectionRecord, haveAmplitude1) == 268 &&
                  offsetof(DetectionRecord, haveTemplateID) == 277 && offsetof(DetectionRecord, polarity) == 278,
              "detection record layout");

struct TemplateHeader
{
    double samplingRate, weight, onset, travel, magnitude;
    uint64_t templateID;
    int64_t nSamples;
    int32_t stringBytes[5];
    int32_t polarity;
    bool haveMagnitude, haveIdentifier;
};
static_assert(sizeof(TemplateHeader) == 88 && offsetof(TemplateHeader, stringBytes) == 56 &&
                  offsetof(TemplateHeader, polarity) == 76 && offsetof(TemplateHeader, haveIdentifier) == 81,
              "template header layout");

namespace detail
{
inline void check(int rc, const char *what)
{
    if (rc != MPI_SUCCESS) throw std::runtime_error(std::string(what) + " failed");
}
template <class T> MPI_Datatype type();
template <> inline MPI_Datatype type<float>() { return MPI_FLOAT; }
template <> inline MPI_Datatype type<double>() { return MPI_DOUBLE; }
inline void put64(char *dst, const std::string &s) { std::memcpy(dst, s.data(), std::min<size_t>(64, s.size())); }
inline std::string get64(const char *src) { return std::string(src, strnlen(src, 64)); }
inline int rank(MPI_Comm comm)
{
    int r = 0;
    check(MPI_Comm_rank(comm, &r), "MPI_Comm_rank");
    return r;
}
}  // namespace detail

/* the detection's record: zeroed, then its fields and flags (src/mpi.cpp:119-195) */
template <class T> DetectionRecord toRecord(const SingleChannel::Detection<T> &det)
{
    DetectionRecord r;
    std::memset(&r, 0, sizeof(r));
    if ((r.haveAmplitude1 = det.haveAmplitudeScalingFactor(RelativeMagnitudeType::GIBBONS_RINGDAL_2006)))
        r.amplitude1 = det.getAmplitudeScalingFactor(RelativeMagnitudeType::GIBBONS_RINGDAL_2006);
    if ((r.haveAmplitude2 = det.haveAmplitudeScalingFactor(RelativeMagnitudeType::SCHAFF_RICHARDS_2014)))
        r.amplitude2 = det.getAmplitudeScalingFactor(RelativeMagnitudeType::SCHAFF_RICHARDS_2014);
    if ((r.haveCorrelationCoefficient = det.haveCorrelationCoefficient()))
        r.correlationCoefficient = det.getCorrelationCoefficient();
    if ((r.haveDetectionTime = det.haveDetectionTime())) r.detectionTime = det.getDetectionTime();
    if ((r.haveInterpolatedDetectionTime = det.haveInterpolatedDetectionTime()))
        r.interpolatedDetectionTime = det.getInterpolatedDetectionTime();
    if ((r.havePhaseOnsetTime = det.havePhaseOnsetTime())) r.phaseOnsetTime = det.getPhaseOnsetTime();
    if ((r.haveInterpolatedPhaseOnsetTime = det.haveInterpolatedPhaseOnsetTime()))
        r.interpolatedPhaseOnsetTime = det.getInterpolatedPhaseOnsetTime();
    if ((r.haveTravelTime = det.haveTravelTime())) r.travelTime = det.getTravelTime();
    if ((r.haveDetectedSignal = det.haveDetectedSignal())) r.signalLength = det.getDetectedSignalLength();
    if ((r.haveTemplateID = det.haveTemplateIdentifier()))
    {
        const auto id = det.getTemplateIdentifier();
        r.templateID = id.second;
        detail::put64(r.network, id.first.getNetwork());
        detail::put64(r.station, id.first.getStation());
        detail::put64(r.phase, id.first.getPhase());
    }
    r.polarity = (int8_t) det.getPolarity();
    return r;
}

/* *det cleared and given the record's fields; signal holds signalLength
   samples when the record has a detected signal */
template <class T> void fromRecord(const DetectionRecord &r, const T *signal, SingleChannel::Detection<T> *det)
{
    if (!det) throw std::invalid_argument("detection is NULL");
    if (r.haveDetectedSignal && (r.signalLength < 1 || !signal))
        throw std::invalid_argument("detected signal missing");
    *det = SingleChannel::Detection<T>();
    if (r.haveAmplitude1) det->setAmplitudeScalingFactor((T) r.amplitude1, RelativeMagnitudeType::GIBBONS_RINGDAL_2006);
    if (r.haveAmplitude2) det->setAmplitudeScalingFactor((T) r.amplitude2, RelativeMagnitudeType::SCHAFF_RICHARDS_2014);
    if (r.haveCorrelationCoefficient) det->setCorrelationCoefficient(r.correlationCoefficient);
    if (r.haveDetectionTime) det->setDetectionTime(r.detectionTime);
    if (r.haveInterpolatedDetectionTime) det->setInterpolatedDetectionTime(r.interpolatedDetectionTime);
    if (r.havePhaseOnsetTime) det->setPhaseOnsetTime(r.phaseOnsetTime);
    if (r.haveInterpolatedPhaseOnsetTime) det->setInterpolatedPhaseOnsetTime(r.interpolatedPhaseOnsetTime);
    if (r.haveTravelTime) det->setTravelTime(r.travelTime);
    if (r.haveDetectedSignal) det->setDetectedSignal(r.signalLength, signal);
    if (r.haveTemplateID)
    {
        NetworkStationPhase nsp;
        nsp.setNetwork(detail::get64(r.network));
        nsp.setStation(detail::get64(r.station));
        nsp.setPhase(detail::get64(r.phase));
        det->setTemplateIdentifier({nsp, r.templateID});
    }
    /* a byte other than -1, 0, 1 (a sender's uninitialised padding) reads as unknown */
    det->setPolarity(r.polarity == 1 ? Polarity::COMPRESSION
                                     : (r.polarity == -1 ? Polarity::DILATATION : Polarity::UNKNOWN));
}

/* MPI::Send (src/mpi.cpp:386-414) */
template <class T>
void Send(const SingleChannel::Detection<T> &detection, int dest, int tag, MPI_Comm comm)
{
    const DetectionRecord r = toRecord(detection);
    detail::check(MPI_Send(&r, (int) sizeof(r), MPI_BYTE, dest, tag, comm), "MPI_Send");
    if (r.haveDetectedSignal)
        detail::check(MPI_Send(detection.getDetectedSignalPointer(), r.signalLength, detail::type<T>(), dest, tag, comm),
                      "MPI_Send");
}

/* MPI::Recv (src/mpi.cpp:416-450); source may be MPI_ANY_SOURCE: the signal
   is then taken from the record's sender */
template <class T>
void Recv(SingleChannel::Detection<T> *detection, int source, int tag, MPI_Comm comm, MPI_Status *status)
{
    if (!detection) throw std::invalid_argument("detection is NULL");
    DetectionRecord r;
    MPI_Status st;
    detail::check(MPI_Recv(&r, (int) sizeof(r), MPI_BYTE, source, tag, comm, &st), "MPI_Recv");
    std::vector<T> sig;
    if (r.haveDetectedSignal)
    {
        if (r.signalLength < 1) throw std::runtime_error("bad detected signal length");
        sig.resize(r.signalLength);
        detail::check(MPI_Recv(sig.data(), r.signalLength, detail::type<T>(), st.MPI_SOURCE, st.MPI_TAG, comm,
                               MPI_STATUS_IGNORE),
                      "MPI_Recv");
    }
    fromRecord(r, sig.data(), detection);
    if (status != MPI_STATUS_IGNORE) *status = st;
}

/* MPI::Broadcast (src/mpi.cpp:294-384): on exit every rank's template
   equals the root's */
inline void Broadcast(WaveformTemplate &tplate, int root, MPI_Comm comm)
{
    const bool isRoot = detail::rank(comm) == root;
    TemplateHeader h;
    std::memset(&h, 0, sizeof(h));
    std::string strings;
    std::vector<double> x;
    if (isRoot)
    {
        h.samplingRate = tplate.haveSamplingRate() ? tplate.getSamplingRate() : 0;
        h.weight = tplate.getShiftAndStackWeight();
        h.onset = tplate.havePhaseOnsetTime() ? tplate.getPhaseOnsetTime() : -1;
        h.travel = tplate.haveTravelTime() ? tplate.getTravelTime() : -1;
        if ((h.haveMagnitude = tplate.haveMagnitude())) h.magnitude = tplate.getMagnitude();
        h.polarity = (int32_t) tplate.getPolarity();
        if (tplate.haveSignal()) x = tplate.samples();
        h.nSamples = (int64_t) x.size();
        if ((h.haveIdentifier = tplate.haveIdentifier()))
        {
            const auto id = tplate.getIdentifier();
            h.templateID = id.second;
            const std::string f[5] = {id.first.getNetwork(), id.first.getStation(), id.first.getChannel(),
                                      id.first.getLocationCode(), id.first.getPhase()};
            for (int i = 0; i < 5; ++i)
            {
                h.stringBytes[i] = (int32_t) f[i].size();
                strings += f[i];
            }
        }
    }
    detail::check(MPI_Bcast(&h, (int) sizeof(h), MPI_BYTE, root, comm), "MPI_Bcast");
    int nstr = 0;
    for (int i = 0; i < 5; ++i) nstr += h.stringBytes[i];
    if (nstr > 0)
    {
        strings.resize(nstr);
        detail::check(MPI_Bcast(&strings[0], nstr, MPI_BYTE, root, comm), "MPI_Bcast");
    }
    if (h.nSamples > 0)
    {
        x.resize((size_t) h.nSamples);
        detail::check(MPI_Bcast(x.data(), (int) h.nSamples, MPI_DOUBLE, root, comm), "MPI_Bcast");
    }
    if (isRoot) return;
    WaveformTemplate t;
    if (h.nSamples > 0) t.setSignal((int) h.nSamples, x.data());
    if (h.samplingRate > 0) t.setSamplingRate(h.samplingRate);
    t.setShiftAndStackWeight(h.weight);
    if (h.onset >= 0) t.setPhaseOnsetTime(h.onset);
    if (h.travel >= 0) t.setTravelTime(h.travel);
    if (h.haveMagnitude) t.setMagnitude(h.magnitude);
    t.setPolarity((Polarity) h.polarity);
    if (h.haveIdentifier)
    {
        std::string f[5];
        for (int i = 0, o = 0; i < 5; o += h.stringBytes[i++]) f[i] = strings.substr(o, h.stringBytes[i]);
        NetworkStationPhase nsp;
        nsp.setNetwork(f[0]);
        nsp.setStation(f[1]);
        nsp.setChannel(f[2]);
        nsp.setLocationCode(f[3]);
        nsp.setPhase(f[4]);
        t.setIdentifier({nsp, h.templateID});
    }
    tplate = t;
}

/* Every rank's detections to rank root, in rank order (one gather of the
   counts, then of the records and of the signals); the root's own pass
   through the records too.  Returns the list on root, an empty one
   elsewhere. */
template <class T>
std::vector<SingleChannel::Detection<T>> Gather(const std::vector<SingleChannel::Detection<T>> &detections, int root,
                                                 MPI_Comm comm)
{
    const int me = detail::rank(comm);
    int size = 0;
    detail::check(MPI_Comm_size(comm, &size), "MPI_Comm_size");
    std::vector<DetectionRecord> recs;
    std::vector<T> sig;
    for (const auto &d : detections)
    {
        recs.push_back(toRecord(d));
        if (d.haveDetectedSignal())
            sig.insert(sig.end(), d.getDetectedSignalPointer(), d.getDetectedSignalPointer() + d.getDetectedSignalLength());
    }
    /* MPI counts are int: byte counts of the records and sample counts of the signals must fit */
    if (recs.size() > (size_t) std::numeric_limits<int>::max() / sizeof(DetectionRecord) ||
        sig.size() > (size_t) std::numeric_limits<int>::max())
        throw std::invalid_argument("too many detections or detected samples for one gather");
    const int mine[2] = {(int) recs.size(), (int) sig.size()};
    std::vector<int> counts(me == root ? 2 * size : 0);
    detail::check(MPI_Gather(mine, 2, MPI_INT, counts.data(), 2, MPI_INT, root, comm), "MPI_Gather");
    std::vector<int> nb(size), db(size), ns(size), ds(size);
    int totR = 0, totS = 0;
    if (me == root)
        for (int r = 0; r < size; ++r)
        {
            nb[r] = counts[2 * r] * (int) sizeof(DetectionRecord);
            db[r] = totR * (int) sizeof(DetectionRecord);
            totR += counts[2 * r];
            ns[r] = counts[2 * r + 1];
            ds[r] = totS;
            totS += counts[2 * r + 1];
            if (totR > std::numeric_limits<int>::max() / (int) sizeof(DetectionRecord) || totS < 0)
                throw std::runtime_error("gathered detections exceed one gather's int counts");
        }
    std::vector<DetectionRecord> allR(totR);
    std::vector<T> allS(totS);
    detail::check(MPI_Gatherv(recs.data(), mine[0] * (int) sizeof(DetectionRecord), MPI_BYTE, allR.data(), nb.data(),
                              db.data(), MPI_BYTE, root, comm),
                  "MPI_Gatherv");
    detail::check(MPI_Gatherv(sig.data(), mine[1], detail::type<T>(), allS.data(), ns.data(), ds.data(),
                              detail::type<T>(), root, comm),
                  "MPI_Gatherv");
    std::vector<SingleChannel::Detection<T>> out(totR);
    size_t o = 0;
    for (int i = 0; i < totR; ++i)
    {
        const DetectionRecord &r = allR[i];
        const size_t n = r.haveDetectedSignal ? (size_t) r.signalLength : 0;
        if (o + n > allS.size()) throw std::runtime_error("gathered signals shorter than their records");
        fromRecord<T>(r, n ? allS.data() + o : nullptr, &out[i]);
        o += n;
    }
    return out;
}

}  // namespace MPI
}  // namespace MFLib

#endif
