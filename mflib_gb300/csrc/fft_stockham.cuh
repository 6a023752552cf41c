// fft_stockham.cuh -- shared-memory Stockham FFT with a compile-time radix
// plan, per-pass twiddle tables and pluggable first-pass loads / last-pass
// stores (so pre-processing and epilogues fuse into the transform).
#pragma once
#include <cmath>
#include <type_traits>
#include <vector>
#include "device_common.cuh"

namespace mfgpu {

// Largest radix (log2) of the plan.  Radix 16 everywhere: a radix-8 plan
// keeps all 256 threads busy at P = 2048 but executes more instructions and
// measured slower on GB300.
__host__ __device__ constexpr int fft_max_radix_log(int) { return 4; }

// Radix plan for P = 2^LOG2P complex points: passes of the largest radix,
// then one smaller pass for the remainder.  Pass p has stride Ns_p = product
// of the earlier radices.  Twiddles of pass p >= 1 are stored as
// table[tw_off(p) + (r-1)*Ns_p + k] = exp(-2 pi i r k / (Ns_p R_p)), k < Ns_p,
// 1 <= r < R_p (consecutive k are contiguous: conflict-free shared loads),
// followed by the real-FFT post-processing twiddles exp(-2 pi i k / 2P),
// k = 0..P/2.
template <int LOG2P> struct FftPlan
{
    static constexpr int P = 1 << LOG2P;
    static constexpr int MAXL = fft_max_radix_log(LOG2P);
    static constexpr int step(int rem) { return rem >= MAXL ? MAXL : rem; }
    static constexpr int npass()
    {
        int done = 0, n = 0;
        while (done < LOG2P) { done += step(LOG2P - done); ++n; }
        return n;
    }
    static constexpr int ns_log(int pass)
    {
        int done = 0;
        for (int p = 0; p < pass; ++p) done += step(LOG2P - done);
        return done;
    }
    static constexpr int radix_log(int pass) { return step(LOG2P - ns_log(pass)); }
    static constexpr int tw_off(int pass)
    {
        int off = 0;
        for (int p = 1; p < pass; ++p) off += ((1 << radix_log(p)) - 1) << ns_log(p);
        return off;
    }
    static constexpr int post_off() { return tw_off(npass()); }
    // padded to a multiple of 4 entries (16-byte multiple for TMA copies)
    static constexpr int tw_total() { return (post_off() + P / 2 + 1 + 3) & ~3; }
    // Split layout (pass twiddles only): a pass with NS <= 16 keeps its
    // (R-1) NS entries; a pass with NS > 16 stores, for k = 16 a + b,
    // A[r-1][a] = exp(-2 pi i r a / (R NS / 16)) ((R-1) NS/16 entries) and
    // Bt[r-1][b] = exp(-2 pi i r b / (R NS)) ((R-1) 16 entries); the twiddle
    // is A[r-1][a] Bt[r-1][b].  At P = 4096 that is 720 entries instead of
    // 4080, for a CTA whose shared memory cannot hold the full table.
    static constexpr int tws_size(int pass)
    {
        return ((1 << radix_log(pass)) - 1) * ((1 << ns_log(pass)) <= 16 ? (1 << ns_log(pass))
                                                                            : (1 << ns_log(pass)) / 16 + 16);
    }
    static constexpr int tws_off(int pass)
    {
        int off = 0;
        for (int p = 1; p < pass; ++p) off += tws_size(p);
        return off;
    }
    static constexpr int tws_total() { return (tws_off(npass()) + 1) & ~1; }  // 16-byte multiple
};

// Host-side construction of the same table (double precision, rounded once).
template <int LOG2P, class T> void build_twiddle_table_fixed(std::vector<cx<T>> &out)
{
    using PL = FftPlan<LOG2P>;
    const double two_pi = 6.283185307179586476925286766559;
    out.assign(PL::tw_total(), cx<T>{(T) 0, (T) 0});
    for (int p = 1; p < PL::npass(); ++p)
    {
        const int R = 1 << PL::radix_log(p), NS = 1 << PL::ns_log(p);
        for (int r = 1; r < R; ++r)
            for (int k = 0; k < NS; ++k)
            {
                // exp(-2 pi i r k/(NS R)) with the phase reduced exactly in integers
                const long long m = ((long long) r * k) % ((long long) NS * R);
                const double a = -two_pi * (double) m / (double) (NS * R);
                out[PL::tw_off(p) + (r - 1) * NS + k] = cx<T>{(T) std::cos(a), (T) std::sin(a)};
            }
    }
    for (int k = 0; k <= PL::P / 2; ++k)
    {
        const double a = -two_pi * (double) k / (double) (2 * PL::P);
        out[PL::post_off() + k] = cx<T>{(T) std::cos(a), (T) std::sin(a)};
    }
}

// The split layout of FftPlan::tws_off (double precision, each factor rounded once).
template <int LOG2P, class T> void build_twiddle_split_fixed(std::vector<cx<T>> &out)
{
    using PL = FftPlan<LOG2P>;
    const double two_pi = 6.283185307179586476925286766559;
    out.assign(PL::tws_total(), cx<T>{(T) 0, (T) 0});
    auto ph = [&](long long num, long long den) {
        const double a = -two_pi * (double) (num % den) / (double) den;
        return cx<T>{(T) std::cos(a), (T) std::sin(a)};
    };
    for (int p = 1; p < PL::npass(); ++p)
    {
        const int R = 1 << PL::radix_log(p), NS = 1 << PL::ns_log(p), o = PL::tws_off(p);
        for (int r = 1; r < R; ++r)
        {
            if (NS <= 16)
            {
                for (int k = 0; k < NS; ++k) out[o + (r - 1) * NS + k] = ph((long long) r * k, (long long) NS * R);
            }
            else
            {
                const int NA = NS / 16;
                for (int a = 0; a < NA; ++a) out[o + (r - 1) * NA + a] = ph((long long) r * a, (long long) NA * R);
                for (int b = 0; b < 16; ++b)
                    out[o + (R - 1) * NA + (r - 1) * 16 + b] = ph((long long) r * b, (long long) NS * R);
            }
        }
    }
}

template <class T, int LO = 1, int HI = 13> void build_twiddle_split(int log2p, std::vector<cx<T>> &out)
{
    if (log2p == LO) build_twiddle_split_fixed<LO, T>(out);
    else if constexpr (LO < HI) build_twiddle_split<T, LO + 1, HI>(log2p, out);
}

template <class T, int LO = 1, int HI = 13> void build_twiddle_table(int log2p, std::vector<cx<T>> &out)
{
    if (log2p == LO) build_twiddle_table_fixed<LO, T>(out);
    else if constexpr (LO < HI) build_twiddle_table<T, LO + 1, HI>(log2p, out);
}

// Barrier over the NT threads that run one transform: the whole CTA
// (BAR == 0) or a named hardware barrier shared by a team of NT threads.
template <int BAR, int NT> __device__ __forceinline__ void team_sync()
{
    if constexpr (BAR == 0) __syncthreads();
    else asm volatile("bar.sync %0, %1;" ::"n"(BAR), "n"(NT) : "memory");
}
// BAR < 0: the barrier id is a run-time value (one code path serves every
// team of a CTA, so the instruction cache holds one copy)
template <int BAR, int NT> __device__ __forceinline__ void team_sync(int bar_id)
{
    if constexpr (BAR < 0) asm volatile("bar.sync %0, %1;" ::"r"(bar_id), "n"(NT) : "memory");
    else team_sync<BAR, NT>();
}

template <class T, int LOG2P, int NT, bool INV, bool ST_BUF, int PASS, class LD, class ST, bool LD_ALIAS = false,
          int BAR = 0, bool TWSPLIT = false>
__device__ __forceinline__ void fft_pass_io(cx<T> *s, const cx<T> *tws, int tid, LD &ld, ST &st, int bar_id = 0)
{
    using PL = FftPlan<LOG2P>;
    constexpr int P = PL::P, NP = PL::npass();
    constexpr int R = 1 << PL::radix_log(PASS), NS = 1 << PL::ns_log(PASS);
    constexpr int NB = P / R, BPT = (NB + NT - 1) / NT;
    constexpr bool FIRST = PASS == 0, LAST = PASS == NP - 1;
    cx<T> a[BPT][R];
#pragma unroll
    for (int b = 0; b < BPT; ++b)
    {
        const int q = tid + b * NT;
        if (NB % NT == 0 || q < NB)
        {
#pragma unroll
            for (int r = 0; r < R; ++r)
            {
                if constexpr (FIRST) a[b][r] = ld(q + r * NB);
                else a[b][r] = s[spad(q + r * NB)];
            }
        }
    }
    if constexpr ((!FIRST && (!LAST || ST_BUF)) || (FIRST && LD_ALIAS)) team_sync<BAR, NT>(bar_id);
#pragma unroll
    for (int b = 0; b < BPT; ++b)
    {
        const int q = tid + b * NT;
        if (NB % NT == 0 || q < NB)
        {
            const int k = q & (NS - 1);
            if constexpr (NS > 1 && (!TWSPLIT || NS <= 16))
            {
                const cx<T> *tp = tws + (TWSPLIT ? PL::tws_off(PASS) : PL::tw_off(PASS)) + k;
#pragma unroll
                for (int r = 1; r < R; ++r)
                {
                    cx<T> w = tp[(r - 1) * NS];
                    if (INV) w.y = -w.y;
                    a[b][r] = cmul(a[b][r], w);
                }
            }
            else if constexpr (NS > 1)
            {
                constexpr int NA = NS / 16;
                const cx<T> *ta = tws + PL::tws_off(PASS) + (k >> 4);
                const cx<T> *tb = tws + PL::tws_off(PASS) + (R - 1) * NA + (k & 15);
#pragma unroll
                for (int r = 1; r < R; ++r)
                {
                    cx<T> w = cmul(ta[(r - 1) * NA], tb[(r - 1) * 16]);
                    if (INV) w.y = -w.y;
                    a[b][r] = cmul(a[b][r], w);
                }
            }
            dft<T, R, INV>(a[b]);
            const int base = (q - k) * R + k;
#pragma unroll
            for (int r = 0; r < R; ++r)
            {
                if constexpr (LAST) st(base + r * NS, a[b][r]);
                else s[spad(base + r * NS)] = a[b][r];
            }
        }
    }
    if constexpr (!LAST) team_sync<BAR, NT>(bar_id);
}

// Runs every pass.  The first pass reads its inputs through ld(e) (e in
// [0, P)); the last pass hands each output element e to st(e, value).
// ST_BUF: the last pass stores into s itself (needs the load/store barrier).
// LD_ALIAS: ld reads memory that overlaps s (barrier before the first stores).
// Intermediate results live in the padded buffer s.  The caller must make
// sure s is free on entry; after return (with ST_BUF) the caller
// synchronises before reading s.
template <class T, int LOG2P, int NT, bool INV, bool ST_BUF, class LD, class ST, bool LD_ALIAS = false, int BAR = 0,
          bool TWSPLIT = false, int PASS = 0>
__device__ __forceinline__ void fft_run(cx<T> *s, const cx<T> *tws, int tid, LD &ld, ST &st, int bar_id = 0)
{
    if constexpr (PASS < FftPlan<LOG2P>::npass())
    {
        fft_pass_io<T, LOG2P, NT, INV, ST_BUF, PASS, LD, ST, LD_ALIAS, BAR, TWSPLIT>(s, tws, tid, ld, st, bar_id);
        fft_run<T, LOG2P, NT, INV, ST_BUF, LD, ST, LD_ALIAS, BAR, TWSPLIT, PASS + 1>(s, tws, tid, ld, st, bar_id);
    }
}

}  // namespace mfgpu
