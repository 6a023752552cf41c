// device_common.cuh -- device-side building blocks shared by the kernels:
// complex arithmetic, the shared-memory Stockham FFT, double-float
// compensated arithmetic, and the TMA / mbarrier helpers (inline PTX for
// sm_103a).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mfgpu {

// ----------------------------------------------------------------------------
// complex numbers
template <class T> struct alignas(2 * sizeof(T)) cx { T x, y; };

template <class T> __device__ __forceinline__ cx<T> cmk(T a, T b) { cx<T> r; r.x = a; r.y = b; return r; }
template <class T> __device__ __forceinline__ cx<T> operator+(cx<T> a, cx<T> b) { return cmk(a.x + b.x, a.y + b.y); }
template <class T> __device__ __forceinline__ cx<T> operator-(cx<T> a, cx<T> b) { return cmk(a.x - b.x, a.y - b.y); }
template <class T> __device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b)
{
    return cmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <class T> __device__ __forceinline__ cx<T> cconj(cx<T> a) { return cmk(a.x, -a.y); }
template <class T> __device__ __forceinline__ cx<T> cscale(cx<T> a, T s) { return cmk(a.x * s, a.y * s); }
// multiply by -i (forward) or +i (inverse)
template <class T, bool INV> __device__ __forceinline__ cx<T> mul_mi(cx<T> a)
{
    return INV ? cmk(-a.y, a.x) : cmk(a.y, -a.x);
}

// Shared-memory index padding: one spare slot per 16 complex values keeps
// the strided Stockham stores and the contiguous loads free of bank
// conflicts for both 8-byte (float) and 16-byte (double) complex values.
__device__ __forceinline__ int spad(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int spad_size(int n) { return n + (n >> 4) + 1; }

// ----------------------------------------------------------------------------
// In-register DFTs of size 2, 4, 8, 16.  Forward uses exp(-2 pi i/R).
// The constants are cos/sin of multiples of pi/8.
template <class T> struct kconst
{
    static constexpr T c8 = (T) 0.92387953251128675613;  // cos(pi/8)
    static constexpr T s8 = (T) 0.38268343236508977173;  // sin(pi/8)
    static constexpr T r2 = (T) 0.70710678118654752440;  // sqrt(1/2)
};

template <class T, bool INV> __device__ __forceinline__ void dft2(cx<T> &a, cx<T> &b)
{
    cx<T> t = a; a = t + b; b = t - b;
}

template <class T, bool INV> __device__ __forceinline__ void dft4(cx<T> &a0, cx<T> &a1, cx<T> &a2, cx<T> &a3)
{
    cx<T> s0 = a0 + a2, d0 = a0 - a2;
    cx<T> s1 = a1 + a3, d1 = mul_mi<T, INV>(a1 - a3);
    a0 = s0 + s1; a2 = s0 - s1;
    a1 = d0 + d1; a3 = d0 - d1;
}

// multiply by W8^k, W8 = exp(-+2 pi i/8)
template <class T, bool INV, int K> __device__ __forceinline__ cx<T> w8(cx<T> a)
{
    const T r = kconst<T>::r2;
    if (K == 0) return a;
    if (K == 1) return INV ? cmk(r * (a.x - a.y), r * (a.x + a.y)) : cmk(r * (a.x + a.y), r * (a.y - a.x));
    if (K == 2) return mul_mi<T, INV>(a);
    // K == 3: W8^3 = -W8^{-1} ... = exp(-+3 pi i/4)
    return INV ? cmk(-r * (a.x + a.y), r * (a.x - a.y)) : cmk(r * (a.y - a.x), -r * (a.x + a.y));
}

template <class T, bool INV> __device__ __forceinline__ void dft8(cx<T> *a)
{
    // n = j + 2l, k = m + 4p
    dft4<T, INV>(a[0], a[2], a[4], a[6]);
    dft4<T, INV>(a[1], a[3], a[5], a[7]);
    cx<T> c0[4] = {a[0], a[2], a[4], a[6]};
    cx<T> c1[4] = {a[1], w8<T, INV, 1>(a[3]), w8<T, INV, 2>(a[5]), w8<T, INV, 3>(a[7])};
#pragma unroll
    for (int m = 0; m < 4; ++m)
    {
        a[m] = c0[m] + c1[m];
        a[m + 4] = c0[m] - c1[m];
    }
}

// multiply by W16^k for k in 0..9
template <class T, bool INV> __device__ __forceinline__ cx<T> w16(cx<T> a, int k)
{
    const T c1 = kconst<T>::c8, s1 = kconst<T>::s8, r = kconst<T>::r2;
    T c, s;  // exp(-i theta) = c - i s  with theta = 2 pi k / 16
    switch (k)
    {
    case 0: return a;
    case 1: c = c1; s = s1; break;
    case 2: c = r; s = r; break;
    case 3: c = s1; s = c1; break;
    case 4: c = 0; s = 1; break;
    case 6: c = -r; s = r; break;
    case 9: c = -c1; s = -s1; break;
    default: c = 1; s = 0; break;
    }
    if (INV) s = -s;
    // (a.x + i a.y)(c - i s)
    return cmk(a.x * c + a.y * s, a.y * c - a.x * s);
}

template <class T, bool INV> __device__ __forceinline__ void dft16(cx<T> *a)
{
    // n = j + 4l, k = m + 4p:  X[m+4p] = sum_j W4^{jp} W16^{jm} sum_l a[j+4l] W4^{lm}
#pragma unroll
    for (int j = 0; j < 4; ++j) dft4<T, INV>(a[j], a[j + 4], a[j + 8], a[j + 12]);
    // now a[j + 4m] holds c[j][m]
    a[5] = w16<T, INV>(a[5], 1);
    a[9] = w16<T, INV>(a[9], 2);
    a[13] = w16<T, INV>(a[13], 3);
    a[6] = w16<T, INV>(a[6], 2);
    a[10] = w16<T, INV>(a[10], 4);
    a[14] = w16<T, INV>(a[14], 6);
    a[7] = w16<T, INV>(a[7], 3);
    a[11] = w16<T, INV>(a[11], 6);
    a[15] = w16<T, INV>(a[15], 9);
#pragma unroll
    for (int m = 0; m < 4; ++m) dft4<T, INV>(a[4 * m], a[4 * m + 1], a[4 * m + 2], a[4 * m + 3]);
    // a[4m + p] holds X[m + 4p]; transpose the 4x4 index
    cx<T> t[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) t[i] = a[i];
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
        for (int p = 0; p < 4; ++p) a[m + 4 * p] = t[4 * m + p];
}

template <class T, int R, bool INV> __device__ __forceinline__ void dft(cx<T> *a)
{
    if constexpr (R == 2) dft2<T, INV>(a[0], a[1]);
    else if constexpr (R == 4) dft4<T, INV>(a[0], a[1], a[2], a[3]);
    else if constexpr (R == 8) dft8<T, INV>(a);
    else dft16<T, INV>(a);
}

// ----------------------------------------------------------------------------
// Double-float ("two FP32 values") accumulation, Knuth TwoSum / FMA TwoProd.
// Used for the sliding-window sums of x and x^2 in the FP32 path.
struct df { float hi, lo; };
__device__ __forceinline__ df df_make(float a) { df r; r.hi = a; r.lo = 0.f; return r; }
__device__ __forceinline__ df two_sum(float a, float b)
{
    float s = a + b;
    float bb = s - a;
    float e = (a - (s - bb)) + (b - bb);
    df r; r.hi = s; r.lo = e; return r;
}
__device__ __forceinline__ df quick_two_sum(float a, float b)
{
    float s = a + b;
    float e = b - (s - a);
    df r; r.hi = s; r.lo = e; return r;
}
__device__ __forceinline__ df df_add(df a, df b)
{
    df s = two_sum(a.hi, b.hi);
    df t = two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = quick_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_neg(df a) { df r; r.hi = -a.hi; r.lo = -a.lo; return r; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ df df_add_f(df a, float b)
{
    df s = two_sum(a.hi, b);
    s.lo += a.lo;
    return quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df two_prod(float a, float b)
{
    float p = a * b;
    float e = fmaf(a, b, -p);
    df r; r.hi = p; r.lo = e; return r;
}
__device__ __forceinline__ df df_mul_f(df a, float b)
{
    df p = two_prod(a.hi, b);
    p.lo = fmaf(a.lo, b, p.lo);
    return quick_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ df df_sqr(df a)
{
    df p = two_prod(a.hi, a.hi);
    p.lo = fmaf(2.f * a.hi, a.lo, p.lo);
    return quick_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ float df_to_f(df a) { return a.hi + a.lo; }

// Accumulator abstraction: float data accumulates in double-float, double
// data in plain double.
template <class T> struct acc_t;
template <> struct acc_t<float>
{
    using type = df;
    static __device__ __forceinline__ df zero() { return df_make(0.f); }
    static __device__ __forceinline__ df from(float a) { return df_make(a); }
    static __device__ __forceinline__ df add(df a, df b) { return df_add(a, b); }
    static __device__ __forceinline__ df sub(df a, df b) { return df_sub(a, b); }
    static __device__ __forceinline__ df add_val(df a, float v) { return df_add_f(a, v); }
    static __device__ __forceinline__ df add_sq(df a, float v) { return df_add(a, two_prod(v, v)); }
    static __device__ __forceinline__ df shfl_up(df a, int d)
    {
        df r; r.hi = __shfl_up_sync(0xffffffffu, a.hi, d); r.lo = __shfl_up_sync(0xffffffffu, a.lo, d); return r;
    }
};
template <> struct acc_t<double>
{
    using type = double;
    static __device__ __forceinline__ double zero() { return 0.0; }
    static __device__ __forceinline__ double from(double a) { return a; }
    static __device__ __forceinline__ double add(double a, double b) { return a + b; }
    static __device__ __forceinline__ double sub(double a, double b) { return a - b; }
    static __device__ __forceinline__ double add_val(double a, double v) { return a + v; }
    static __device__ __forceinline__ double add_sq(double a, double v) { return fma(v, v, a); }
    static __device__ __forceinline__ double shfl_up(double a, int d) { return __shfl_up_sync(0xffffffffu, a, d); }
};

// ----------------------------------------------------------------------------
// TMA (bulk async copy) and mbarrier helpers.
__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// An mbarrier whose phases have all completed, made ordinary memory again
// (before it is set up anew).
__device__ __forceinline__ void mbar_inval(uint64_t *bar)
{
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// 1-D bulk copy global -> shared; both addresses 16-byte aligned, bytes a
// multiple of 16.
__device__ __forceinline__ void tma_load_1d(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Bounded wait on an mbarrier phase.  Returns false (and the caller records
// an error) if the phase does not complete within the iteration limit.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t limit = (1u << 24))
{
    for (uint32_t it = 0; it < limit; ++it)
    {
        if (mbar_try_wait(bar, parity)) return true;
        if (it > 64) __nanosleep(64);
    }
    return false;
}

// Error codes written by kernels into the context's device status word.
enum : int { KERR_NONE = 0, KERR_TMA_TIMEOUT = 1, KERR_BOUNDS = 2, KERR_OVERFLOW = 3 };

}  // namespace mfgpu
