// kernels_tc.cuh -- split-precision tensor-core correlator for FP32 data and
// templates of one length: the Pearson numerators as a Hankel GEMM on the
// 5th-generation tensor cores (tcgen05.mma kind::f16, FP32 accumulators in
// tensor memory), with FP16 hi+lo operand splits (hi*hi + hi*lo + lo*hi)
// that restore about 22 bits of operand precision.  Two MMAs per 16-deep K
// step: A_hi against [B_hi; B_lo] (N = 16 Gp: the hi*hi and hi*lo products
// land in two column halves) and A_lo against B_hi into the first half, so
// the A operand is fetched from shared memory twice per step, not three
// times; the epilogue adds the two halves.
//
// Tile = 128 rows x 8 phases = 1024 consecutive lags of one channel against
// a group of Gp templates.  Row i, phase f is lag k0 + 8i + f:
//   num[8i + f][t] = sum_k x[k0 + 8i + k] * b_t[k - f],   k in [0, Kp)
// so A[i][k] = x[k0 + 8i + k] is a Hankel matrix whose rows start 8 samples
// (16 bytes) apart: its 8x8 core matrices are contiguous 128-byte pieces of
// the signal strip itself (leading-dimension offset 16 B, stride offset
// 128 B), and B holds each template at its 8 phase shifts.  The numerator is
// invariant to a constant added to the window (templates are zero-mean), so
// each strip is offset by the level of its quietest 32-lag run (chosen by
// fix_flag_tc_kernel from the window statistics; the split's error is
// relative to |x - offset|) and scaled by a per-channel power of two before
// the split; templates are scaled by a power of two too.
//
// Persistent, warp-specialised CTA (one per SM):
//   warp 0 lane 0   issues the MMAs (K/16 steps x 2) and the commits;
//   warps 1-3       stage strips: FP32 load, offset, scale, hi/lo split;
//   warps 4-11      epilogue, two warpgroups taking alternate templates:
//                   tcgen05.ld of the accumulator rows (the buffer is
//                   released before the stores), scales, normalisation row
//                   (prefetched a tile ahead), |rho| > 1.1 clamp, 32-byte
//                   stores.
// Strips and accumulators are double-buffered (mbarriers, bounded waits);
// the group's template operands stay resident in shared memory.
//
// BF16 operands (template flag BF, an option): the same kernel with BF16 hi
// and lo (about 16 of the 24 bits kept, against 22 for FP16; BF16's
// exponent range needs no scaling but the powers of two are kept), and the
// instruction descriptor's A and B format fields set to BF16.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include "kernels_mf.cuh"
#include "tc_params.h"

namespace mfgpu {

// hi + lo split of an FP32 value into two 16-bit operands (bit patterns
// stored as __half either way) and the matching kind::f16 A / B format bits
template <bool BF> struct TcSplit;
template <> struct TcSplit<false>
{
    static constexpr uint32_t ab_format = 0u;
    static __device__ __forceinline__ void split(float y, __half &h, __half &l)
    {
        h = __float2half_rn(y);
        l = __float2half_rn(y - __half2float(h));
    }
};
template <> struct TcSplit<true>
{
    static constexpr uint32_t ab_format = (1u << 7) | (1u << 10);
    static __device__ __forceinline__ void split(float y, __half &h, __half &l)
    {
        const __nv_bfloat16 bh = __float2bfloat16_rn(y);
        const __nv_bfloat16 bl = __float2bfloat16_rn(y - __bfloat162float(bh));
        h = __ushort_as_half(__bfloat16_as_ushort(bh));
        l = __ushort_as_half(__bfloat16_as_ushort(bl));
    }
};

// shared-memory matrix descriptor: start address, leading and stride byte
// offsets (16-byte units), descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t) ((addr >> 4) & 0x3FFF) | ((uint64_t) ((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t) ((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t) 1 << 46);
}

__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

// arrives on bar once every tcgen05 operation issued so far has completed
__device__ __forceinline__ void tc_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Template bank in MMA layout: one CTA per (group, slot).  Row 8*slot + f of
// the group's B holds the demeaned unit-norm template (FP64 preparation as
// in the FFT path) shifted right by f, scaled by a power of two, split into
// FP16 (or BF16) hi and lo; element (row n, k) sits in core matrix (n/8, k/8) at
// ((n/8) * Kp/8 + k/8) * 64 + (n%8) * 8 + k%8.
template <bool BF>
__global__ void __launch_bounds__(256) tc_bank_kernel(const double *tmpl, const long *toff, const int *tlen,
                                                      const int *grp_tid, int Gp, int Kp, __half *B, float *bscale)
{
    __shared__ double red[32];
    const int g = blockIdx.x / Gp, slot = blockIdx.x % Gp;
    const int t = grp_tid[g * Gp + slot];
    __half *bh = B + (size_t) g * 16 * Gp * Kp, *bl = bh + (size_t) 8 * Gp * Kp;
    const int KG = Kp / 8;
    auto bsum = [&](double v) {
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        __syncthreads();
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
        __syncthreads();
        double s = 0;
        for (int i = 0; i < 8; ++i) s += red[i];
        return s;
    };
    double mean = 0, inv = 0;
    int L = 0;
    const double *b = nullptr;
    if (t >= 0)
    {
        L = tlen[t];
        b = tmpl + toff[t];
        double s = 0;
        for (int j = threadIdx.x; j < L; j += 256) s += b[j];
        mean = bsum(s) / L;
        double q = 0;
        for (int j = threadIdx.x; j < L; j += 256) q += (b[j] - mean) * (b[j] - mean);
        const double nrm2 = bsum(q);
        inv = nrm2 > 0 ? 1.0 / sqrt(nrm2) : 0.0;
        double mx = 0;
        for (int j = threadIdx.x; j < L; j += 256) mx = fmax(mx, fabs((b[j] - mean) * inv));
        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        __syncthreads();
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
        __syncthreads();
        mx = 0;
        for (int i = 0; i < 8; ++i) mx = fmax(mx, red[i]);
        const float sb = tc_pow2_scale((float) mx, 12);
        inv *= sb;
        if (threadIdx.x == 0) bscale[g * Gp + slot] = 1.f / sb;
    }
    else if (threadIdx.x == 0)
        bscale[g * Gp + slot] = 0.f;
    for (int idx = threadIdx.x; idx < 8 * Kp; idx += 256)
    {
        const int f = idx / Kp, k = idx % Kp;
        const int j = k - f;
        const float v = (t >= 0 && j >= 0 && j < L) ? (float) ((b[j] - mean) * inv) : 0.f;
        __half h, l;
        TcSplit<BF>::split(v, h, l);
        const size_t o = ((size_t) slot * KG + k / 8) * 64 + f * 8 + (k & 7);
        bh[o] = h;
        bl[o] = l;
    }
}

template <bool BF>
__global__ void __launch_bounds__(kTcThreads, 1) tc_xcorr_kernel(TcParams p)
{
    extern __shared__ __align__(128) unsigned char smem_tc[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_tc);  // a_full[2] a_empty[2] acc_full[2] acc_empty[2] b_full
    uint64_t *a_full = bar, *a_empty = bar + 2, *acc_full = bar + 4, *acc_empty = bar + 6, *b_full = bar + 8;
    uint32_t *tmem_holder = reinterpret_cast<uint32_t *>(smem_tc + 96);
    const int Kp = p.Kp, Gp = p.Gp, N = 8 * Gp;
    const int SA = kTcLags + Kp;
    __half *sA = reinterpret_cast<__half *>(smem_tc + TcLayout::off_A());
    __half *sB = reinterpret_cast<__half *>(smem_tc + TcLayout::off_B(Kp));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const long W = (long) p.ngroups * p.tiles;
    const long w0 = W * blockIdx.x / gridDim.x, w1 = W * (blockIdx.x + 1) / gridDim.x;

    if (tid == 0)
    {
        for (int i = 0; i < 9; ++i) mbar_init(&bar[i], (i == 6 || i == 7) ? kTcEpiWarps : 1);
        fence_proxy_async_smem();
    }
    if (warp == 0)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_holder)),
                     "r"(p.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_holder;

    if (warp == 0)
    {
        if (lane == 0)
        {
            // ---- MMA issue.  Instruction descriptors: D f32, A/B f16, both
            //      K-major, N >> 3, M >> 4; N = 16 Gp (hi and lo rows of B)
            //      and N = 8 Gp (hi rows only)
            constexpr uint32_t fmt = (1u << 4) | TcSplit<BF>::ab_format;
            const uint32_t idesc_w = fmt | ((uint32_t) (2 * N >> 3) << 17) | ((uint32_t) (kTcRows >> 4) << 24);
            const uint32_t idesc_n = fmt | ((uint32_t) (N >> 3) << 17) | ((uint32_t) (kTcRows >> 4) << 24);
            const uint32_t bbytes = (uint32_t) TcLayout::b_bytes(Kp, Gp);
            const uint32_t sA0 = smem_u32(sA), sB0 = smem_u32(sB);
            // the lo rows follow the hi rows at the same row-group stride, so
            // one descriptor spans [B_hi; B_lo]
            const uint32_t sbo_b = (uint32_t) (Kp / 8) * 128;
            int cur = -1;
            uint32_t bph = 0;
            bool ok = true;
            long issued = 0;
            for (long w = w0, n = 0; w < w1 && ok; ++w, ++n)
            {
                const int g = (int) (w / p.tiles);
                const int buf = (int) (n & 1);
                if (g != cur)
                {
                    // the tensor core has finished reading the old group's B
                    if (n > 0) ok = mbar_wait_bounded(&acc_full[(n - 1) & 1], (uint32_t) (((n - 1) >> 1) & 1));
                    if (!ok) break;
                    mbar_arrive_expect_tx(b_full, bbytes);
                    tma_load_1d(sB, p.B + (size_t) g * 16 * Gp * Kp, bbytes, b_full);
                    ok = mbar_wait_bounded(b_full, bph);
                    if (!ok)
                    {
                        mbar_wait_bounded(b_full, bph);  // let the copy land before leaving
                        break;
                    }
                    bph ^= 1u;
                    cur = g;
                }
                ok = mbar_wait_bounded(&a_full[buf], (uint32_t) ((n >> 1) & 1));
                if (ok && n >= 2) ok = mbar_wait_bounded(&acc_empty[buf], (uint32_t) (((n - 2) >> 1) & 1));
                if (!ok) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t d = tmem + (uint32_t) (buf * 2 * N);
                const uint32_t ahi = sA0 + (uint32_t) (2 * buf) * SA * 2, alo = ahi + (uint32_t) SA * 2;
                for (int kk = 0; kk < Kp / 16; ++kk)
                {
                    const uint64_t dAh = tc_desc(ahi + kk * 32, 16, 128), dAl = tc_desc(alo + kk * 32, 16, 128);
                    const uint64_t dB = tc_desc(sB0 + kk * 256, 128, sbo_b);
                    tc_mma(d, dAh, dB, idesc_w, kk > 0 ? 1u : 0u);  // [hi*hi | hi*lo]
                    tc_mma(d, dAl, dB, idesc_n, 1u);                 // + lo*hi into the first half
                }
                tc_commit(&a_empty[buf]);
                tc_commit(&acc_full[buf]);
                ++issued;
            }
            if (!ok) atomicExch(p.err, KERR_TMA_TIMEOUT);
            // the last MMAs land before teardown
            if (issued > 0)
                mbar_wait_bounded(&acc_full[(issued - 1) & 1], (uint32_t) (((issued - 1) >> 1) & 1));
        }
    }
    else if (warp < 4)
    {
        // ---- strips: x[k0, k0 + 1024 + Kp) -> (x - off) * s -> FP16 hi, lo
        const int ptid = tid - 32;
        bool ok = true;
        for (long w = w0, n = 0; w < w1; ++w, ++n)
        {
            const int g = (int) (w / p.tiles), j = (int) (w % p.tiles);
            const int buf = (int) (n & 1);
            if (n >= 2 && ok)
            {
                ok = mbar_wait_bounded(&a_empty[buf], (uint32_t) (((n - 2) >> 1) & 1));
                if (!ok) atomicExch(p.err, KERR_TMA_TIMEOUT);
            }
            const int c = p.grp_chan[g];
            const float *xr = p.x + (long) c * p.ldx + (long) j * kTcLags;
            const float s = tc_pow2_scale(p.xrange[c], 13);
            const float off = p.off[(long) c * p.tiles + j];
            __half *ah = sA + (size_t) (2 * buf) * SA, *al = ah + SA;
            constexpr int PR = 4;  // loads in flight per thread
            if (ok)
                for (int e0 = 4 * ptid; e0 < SA; e0 += 4 * kTcProducers * PR)
                {
                    float4 v[PR];
#pragma unroll
                    for (int r = 0; r < PR; ++r)
                    {
                        const int e = e0 + r * 4 * kTcProducers;
                        v[r] = e < SA ? *reinterpret_cast<const float4 *>(xr + e) : make_float4(0.f, 0.f, 0.f, 0.f);
                    }
#pragma unroll
                    for (int r = 0; r < PR; ++r)
                    {
                        const int e = e0 + r * 4 * kTcProducers;
                        if (e >= SA) break;
                        // samples of the channel lie within its range, so |y| < 2^13;
                        // the clamp only touches the zero tail past the samples (or
                        // past a shorter uploaded window), which meets zero template
                        // coefficients at every valid lag: finite there, never inf * 0
                        float y[4] = {(v[r].x - off) * s, (v[r].y - off) * s, (v[r].z - off) * s,
                                      (v[r].w - off) * s};
#pragma unroll
                        for (int q = 0; q < 4; ++q) y[q] = fminf(fmaxf(y[q], -60000.f), 60000.f);
                        __align__(8) __half h[4];
                        __align__(8) __half l[4];
#pragma unroll
                        for (int q = 0; q < 4; ++q) TcSplit<BF>::split(y[q], h[q], l[q]);
                        *reinterpret_cast<uint2 *>(ah + e) = *reinterpret_cast<const uint2 *>(h);
                        *reinterpret_cast<uint2 *>(al + e) = *reinterpret_cast<const uint2 *>(l);
                    }
                }
            fence_proxy_async_smem();  // generic-proxy writes before the tensor core's reads
            asm volatile("bar.sync 1, %0;" ::"n"(kTcProducers) : "memory");
            if (ptid == 0) mbar_arrive(&a_full[buf]);
        }
    }
    else
    {
        // ---- epilogue: row i of the tile = TMEM lane i; warpgroup eg takes
        //      templates eg, eg + 2, ...
        const int q = warp & 3, i = 32 * q + lane, eg = (warp - 4) >> 2;
        constexpr int TB = 2;  // templates per batch of TMEM loads (two halves each)
        float dv[8];
        auto load_den = [&](long w) {
            const int c = p.grp_chan[(int) (w / p.tiles)];
            const long lag0 = (long) (w % p.tiles) * kTcLags + 8 * i;
            const float4 d0 = *reinterpret_cast<const float4 *>(p.den + (long) c * p.ldd + lag0);
            const float4 d1 = *reinterpret_cast<const float4 *>(p.den + (long) c * p.ldd + lag0 + 4);
            dv[0] = d0.x; dv[1] = d0.y; dv[2] = d0.z; dv[3] = d0.w;
            dv[4] = d1.x; dv[5] = d1.y; dv[6] = d1.z; dv[7] = d1.w;
        };
        if (w0 < w1) load_den(w0);
        for (long w = w0, n = 0; w < w1; ++w, ++n)
        {
            const int g = (int) (w / p.tiles), j = (int) (w % p.tiles);
            const int buf = (int) (n & 1);
            if (!mbar_wait_bounded(&acc_full[buf], (uint32_t) ((n >> 1) & 1)))
            {
                atomicExch(p.err, KERR_TMA_TIMEOUT);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int c = p.grp_chan[g];
            const long lag0 = (long) j * kTcLags + 8 * i;
            const float s = tc_pow2_scale(p.xrange[c], 13);
            const bool dead = p.dead[c] != 0;
            float dcur[8];
#pragma unroll
            for (int f = 0; f < 8; ++f) dcur[f] = dv[f];
            const int nmine = (Gp - eg + 1) / 2;  // templates eg, eg + 2, ... below Gp
            bool released = false;
            for (int b0 = 0; b0 < nmine; b0 += TB)
            {
                uint32_t r[TB][8], h[TB][8];
#pragma unroll
                for (int u = 0; u < TB; ++u)
                {
                    if (b0 + u < nmine)  // uniform across the warp
                    {
                        const int t = eg + 2 * (b0 + u);
                        const uint32_t taddr = tmem + ((uint32_t) (32 * q) << 16) + (uint32_t) (buf * 2 * N + 8 * t);
                        asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                                     : "=r"(r[u][0]), "=r"(r[u][1]), "=r"(r[u][2]), "=r"(r[u][3]), "=r"(r[u][4]),
                                       "=r"(r[u][5]), "=r"(r[u][6]), "=r"(r[u][7])
                                     : "r"(taddr));
                        asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                                     : "=r"(h[u][0]), "=r"(h[u][1]), "=r"(h[u][2]), "=r"(h[u][3]), "=r"(h[u][4]),
                                       "=r"(h[u][5]), "=r"(h[u][6]), "=r"(h[u][7])
                                     : "r"(taddr + (uint32_t) N));
                    }
                }
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (b0 + TB >= nmine)
                {
                    // every accumulator value of this tile is in registers:
                    // release the buffer before the stores, prefetch the
                    // next tile's normalisation row
                    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&acc_empty[buf]);
                    released = true;
                    if (w + 1 < w1) load_den(w + 1);
                }
#pragma unroll
                for (int u = 0; u < TB; ++u)
                {
                    if (b0 + u >= nmine) break;
                    const int t = eg + 2 * (b0 + u);
                    const int tt = p.grp_tid[g * Gp + t];
                    if (tt < 0) continue;
                    // a dead channel's tiles store zeros (sc = 0, no flags)
                    const float sc = dead ? 0.f : p.bscale[g * Gp + t] / s;
                    float o[8];
#pragma unroll
                    for (int f = 0; f < 8; ++f)
                        o[f] = clamp_rho((__uint_as_float(r[u][f]) + __uint_as_float(h[u][f])) * sc * dcur[f]);
                    if (p.pk_flags)
                    {
                        // one bit per 64 lags (8 rows); values above the
                        // threshold are rare, so each such row sets its bit
                        // itself, without a warp-wide vote; the lag bound
                        // matters only in the last tile
                        float mx = o[0];
#pragma unroll
                        for (int f = 1; f < 8; ++f) mx = fmaxf(mx, o[f]);
                        if (mx > p.pk_thr)
                        {
                            bool above = false;
#pragma unroll
                            for (int f = 0; f < 8; ++f) above |= lag0 + f < p.nv && o[f] > p.pk_thr;
                            if (above)
                            {
                                const long c = lag0 >> 6;
                                atomicOr(p.pk_flags + (long) tt * p.pk_words + (c >> 5), 1u << (c & 31));
                            }
                        }
                    }
                    float *dst = p.rho + (long) tt * p.ldr + lag0;
                    if (lag0 + 7 < p.nv)
                    {
                        // the row's 8 lags in one 32-byte store (rows of rho
                        // are 256-byte aligned, lag0 a multiple of 8): whole
                        // sectors per store instead of two half-sector halves
                        asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(dst), "f"(o[0]),
                                     "f"(o[1]), "f"(o[2]), "f"(o[3]), "f"(o[4]), "f"(o[5]), "f"(o[6]), "f"(o[7])
                                     : "memory");
                    }
                    else
                    {
#pragma unroll
                        for (int f = 0; f < 8; ++f)
                            if (lag0 + f < p.nv) dst[f] = o[f];
                    }
                }
            }
            if (!released)
            {
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(&acc_empty[buf]);
                if (w + 1 < w1) load_den(w + 1);
            }
        }
    }

    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(p.tmem_cols) : "memory");
}

}  // namespace mfgpu
