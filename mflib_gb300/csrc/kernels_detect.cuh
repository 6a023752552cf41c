// kernels_detect.cuh -- the single-channel detector's data-parallel parts
// (MFLib::SingleChannel::Detector<T>::detect, src/singleChannel/detector.cpp)
// on the device:
//   * reduction of the Pearson traces across templates: per lag the maximum
//     (or absolute maximum) and the first template reaching it, clamped to
//     [-1, 1] (reduceAllCorrelations / cleanReducedTemplate, :201-257, :191);
//     or, per template, its own trace transformed the same way
//     (setCorrelations, :259-284);
//   * per detection: the template's clamped coefficient and sign, the
//     detection-time refinement (quadraticRefinement :38-91,
//     lanczosRefinement :114-152) and the relative amplitude sums of
//     RelativeMagnitude (src/singleChannel/relativeMagnitude.cpp:35-130):
//     |<x, y>| / <x, x> and sqrt(<y, y> / <x, x>) of the demeaned template x
//     and the demeaned detected window y, in double.
#pragma once
#include <cfloat>
#include "kernels_util.cuh"

namespace mfgpu {

struct DetectOut
{
    int tmpl;         // template index
    int sample;       // peak lag
    double xc;        // clamped coefficient of that template at the lag
    double shift;     // refinement, seconds
    int sign;         // sign of the coefficient (-1, 0, 1)
    int have_amp;
    double gr, sr;    // amplitude scaling factors (Gibbons-Ringdal, Schaff-Richards)
};

template <class T> __device__ __forceinline__ T det_clamp(T v) { return v > (T) 1 ? (T) 1 : (v < (T) -1 ? (T) -1 : v); }

// det[k] = clamp(max_t f(rho_t[k])), id[k] = first t reaching it (strict >
// in template order, starting from template 0), f = |.| or identity
template <class T>
__global__ void det_reduce_kernel(const T *rho, long ldr, int nt, long len, int use_abs, T *det, int *id)
{
    const long k = (long) blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= len) return;
    T best = rho[k];
    if (use_abs) best = fabs(best);
    int bi = 0;
    for (int t = 1; t < nt; ++t)
    {
        T v = rho[(long) t * ldr + k];
        if (use_abs) v = fabs(v);
        if (v > best)
        {
            best = v;
            bi = t;
        }
    }
    det[k] = det_clamp(best);
    id[k] = bi;
}

// per-template traces for the SINGLE policy: out[t][k] = clamp(f(rho_t[k]))
template <class T>
__global__ void det_single_kernel(const T *rho, long ldr, int nt, long len, int use_abs, T *out)
{
    const long k = (long) blockIdx.x * blockDim.x + threadIdx.x;
    const int t = blockIdx.y;
    if (k >= len || t >= nt) return;
    T v = rho[(long) t * ldr + k];
    if (use_abs) v = fabs(v);
    out[(long) t * ldr + k] = det_clamp(v);
}

struct DetectParams
{
    const int *peak;      // [ndet] lag of each detection
    const int *row;       // [ndet] template (SINGLE) or -1: take id[peak]
    const int *id;        // reduced argmax per lag (REDUCED)
    int ndet;
    long len;             // detection (filtered) length
    int use_abs;
    int interp;           // 0 Lanczos, 1 quadratic, 2 none
    int alpha, nrefine;
    double dt;
    int amplitudes;
    const double *tmpl;   // FP64 templates, template t at toff[t], length tlen[t]
    const long *toff;
    const int *tlen;
    const int *tchan;     // channel of each template
    long n;               // signal samples
    DetectOut *out;
};

// sinc and the Lanczos kernel in the trace's precision, with the
// reference's tolerance (100 machine epsilons) and pi x formed in double
template <class T> __device__ __forceinline__ T det_sinc(T x)
{
    const T tol = (sizeof(T) == 4 ? (T) FLT_EPSILON : (T) DBL_EPSILON) * (T) 100;
    if (fabs(x) > tol)
    {
        const T pix = (T) (3.14159265358979323846 * (double) x);
        return sin(pix) / pix;
    }
    return (T) 1;
}
template <class T> __device__ __forceinline__ T det_lanczos(T x, int a)
{
    if ((int) fabs(x) <= a) return det_sinc<T>(x) * det_sinc<T>(x / (T) a);
    return (T) 0;
}

// quadraticRefinement (src/singleChannel/detector.cpp:46-91), double
__device__ __forceinline__ double det_quadratic(const double *xs, long n, long p, double dt, int use_abs)
{
    if (!(p > 0 && p < n - 1)) return 0.0;
    double y1 = xs[0], y2 = xs[1], y3 = xs[2];
    if (use_abs) { y1 = fabs(y1); y2 = fabs(y2); y3 = fabs(y3); }
    if (y2 < y1 || y2 < y3)
    {
        if (y2 < y1 && y2 < y3) { y1 = -y1; y2 = -y2; y3 = -y3; }
        else return 0.0;
    }
    const double e = 100.0 * DBL_EPSILON;
    y1 = fmin(y2 - e, y1);
    y3 = fmin(y2 - e, y3);
    const double num = __dmul_rn(dt, __dsub_rn(y1, y3));
    const double den = __dmul_rn(2.0, __dadd_rn(__dsub_rn(y1, __dmul_rn(2.0, y2)), y3));
    return __ddiv_rn(num, den);
}

// one warp per detection
template <class T>
__global__ void det_refine_kernel(const T *rho, long ldr, const T *x, long ldx, DetectParams q)
{
    const int w = (int) ((blockIdx.x * (long) blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (w >= q.ndet) return;
    const long p = q.peak[w];
    const int it = q.row[w] >= 0 ? q.row[w] : q.id[p];
    const T *xc = rho + (long) it * ldr;
    const T v = xc[p];
    DetectOut o;
    o.tmpl = it;
    o.sample = (int) p;
    o.xc = (double) det_clamp(v);
    o.sign = v < (T) 0 ? -1 : (v == (T) 0 ? 0 : 1);
    o.shift = 0.0;
    if (q.interp == 1)
    {
        double ys[3] = {0.0, 0.0, 0.0};
        if (p > 0 && p < q.len - 1) { ys[0] = xc[p - 1]; ys[1] = xc[p]; ys[2] = xc[p + 1]; }
        o.shift = (double) (T) det_quadratic(ys, q.len, p, q.dt, q.use_abs);  // returned as T
    }
    else if (q.interp == 0)
    {
        // shifts -0.5 + idx / nrefine, idx = 1 .. nrefine - 1, spread over
        // the lanes; the first of equal maxima wins (strict > in idx order)
        const T dtw = (T) (1.0 / (double) q.nrefine);
        T best = -FLT_MAX;
        if (sizeof(T) == 8) best = (T) -DBL_MAX;
        int bidx = 0;
        for (int idx = 1 + lane; idx < q.nrefine; idx += 32)
        {
            const T shift = (T) (-0.5 + (double) (dtw * (T) idx));
            const T xx = (T) p + shift;
            T y = 0;
            const int fl = (int) floor(xx);
            for (int a = -q.alpha; a <= q.alpha; ++a)
            {
                const int i = fl - a + 1;
                const T xi = xx - (T) i;
                const T xcv = (i >= 0 && i < q.len) ? xc[i] : (T) 0;
                y = y + xcv * det_lanczos<T>(xi, q.alpha);
            }
            if (q.use_abs) y = fabs(y);
            if (bidx == 0 || y > best) { best = y; bidx = idx; }
        }
        for (int off = 16; off > 0; off >>= 1)
        {
            const T ob = __shfl_down_sync(0xffffffffu, best, off);
            const int oi = __shfl_down_sync(0xffffffffu, bidx, off);
            if (oi != 0 && (bidx == 0 || ob > best || (ob == best && oi < bidx))) { best = ob; bidx = oi; }
        }
        bidx = __shfl_sync(0xffffffffu, bidx, 0);
        if (bidx > 0)
        {
            const T shift = (T) (-0.5 + (double) (dtw * (T) bidx));
            o.shift = (double) (T) (q.dt * (double) shift);
        }
    }
    // relative amplitude of the detected window against the template
    o.have_amp = 0;
    o.gr = o.sr = 0.0;
    const int L = q.tlen[it];
    if (q.amplitudes && p + L <= q.n)
    {
        const double *b = q.tmpl + q.toff[it];
        const T *y = x + (long) q.tchan[it] * ldx + p;
        double sb = 0, sy = 0;
        for (int j = lane; j < L; j += 32) { sb += b[j]; sy += (double) y[j]; }
        for (int off = 16; off > 0; off >>= 1)
        {
            sb += __shfl_xor_sync(0xffffffffu, sb, off);
            sy += __shfl_xor_sync(0xffffffffu, sy, off);
        }
        const double mb = sb / L, my = sy / L;
        double bb = 0, yy = 0, by = 0;
        for (int j = lane; j < L; j += 32)
        {
            const double db = b[j] - mb, dy = (double) y[j] - my;
            bb += db * db;
            yy += dy * dy;
            by += db * dy;
        }
        for (int off = 16; off > 0; off >>= 1)
        {
            bb += __shfl_xor_sync(0xffffffffu, bb, off);
            yy += __shfl_xor_sync(0xffffffffu, yy, off);
            by += __shfl_xor_sync(0xffffffffu, by, off);
        }
        if (bb > 0 && yy > 0)
        {
            o.have_amp = 1;
            o.gr = fabs(by) / bb;
            o.sr = sqrt(yy / bb);
        }
    }
    if (lane == 0) q.out[w] = o;
}

// RelativeMagnitude (src/singleChannel/relativeMagnitude.cpp:35-130) for a
// batch of detected windows against one template, one warp per window:
// gr = |<b, y>| / <b, b>, sr = sqrt(<y, y> / <b, b>) of the demeaned
// template b and window y, in double; valid = <y, y> > 0
template <class T>
__global__ void amp_kernel(const double *b, int L, const T *y, long ld, int nw, double *gr, double *sr, int *valid)
{
    const int w = (int) ((blockIdx.x * (long) blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (w >= nw) return;
    const T *yw = y + (long) w * ld;
    double sb = 0, sy = 0;
    for (int j = lane; j < L; j += 32) { sb += b[j]; sy += (double) yw[j]; }
    for (int off = 16; off > 0; off >>= 1)
    {
        sb += __shfl_xor_sync(0xffffffffu, sb, off);
        sy += __shfl_xor_sync(0xffffffffu, sy, off);
    }
    const double mb = sb / L, my = sy / L;
    double bb = 0, yy = 0, by = 0;
    for (int j = lane; j < L; j += 32)
    {
        const double db = b[j] - mb, dy = (double) yw[j] - my;
        bb += db * db;
        yy += dy * dy;
        by += db * dy;
    }
    for (int off = 16; off > 0; off >>= 1)
    {
        bb += __shfl_xor_sync(0xffffffffu, bb, off);
        yy += __shfl_xor_sync(0xffffffffu, yy, off);
        by += __shfl_xor_sync(0xffffffffu, by, off);
    }
    if (lane == 0)
    {
        const bool ok = bb > 0 && yy > 0;
        valid[w] = ok ? 1 : 0;
        gr[w] = ok ? fabs(by) / bb : 0.0;
        sr[w] = ok ? sqrt(yy / bb) : 0.0;
    }
}

}  // namespace mfgpu
