// mf_launch.cuh -- launchers of the matched-filter kernels for one sample
// type; included once by mf_f32.cu and once by mf_f64.cu so the two
// precisions compile in parallel.
#pragma once
#include <algorithm>
#include <type_traits>
#include "launch.h"

namespace mfgpu {

template <class T, int LOG2P> struct XcorrTable
{
    static size_t smem(bool shared_den, int mode, int S) { return XcorrLayout<T, LOG2P>::bytes(shared_den, mode, S); }
    template <bool SD, int MODE, bool PERSIST = false>
    static cudaError_t go(const XcorrParams<T> &p, int nblocks, int ngroups, cudaStream_t s)
    {
        size_t bytes = smem(SD, MODE, p.S);
        auto k = xcorr_kernel<T, LOG2P, SD, MODE, PERSIST>;
        static SmemCap cap;
        cudaError_t e = raise_smem_cap(k, bytes, cap);
        if (e != cudaSuccess) return e;
        const int threads = MODE == 4 ? 2 * kThreads : kThreads;
        if constexpr (PERSIST)
        {
            // as many CTAs as fit on the device at once
            int dev = 0, nsm = 0, occ = 0;
            if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
            if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
            if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, threads, bytes)) != cudaSuccess) return e;
            const long want = (long) std::max(1, occ) * nsm;
            const int grid = (int) std::max<long>(1, std::min<long>(want, (long) p.ntiles));
            k<<<grid, threads, bytes, s>>>(p);
        }
        else
            k<<<dim3(nblocks, ngroups), threads, bytes, s>>>(p);
        return cudaGetLastError();
    }
    // the persistent work-queue form is compiled for the FP32 team
    // organisations (modes 2 and 4) only
    static constexpr bool persist_ok = std::is_same<T, float>::value && LOG2P >= 11;
    // mode 4 (two 256-thread teams, several template lengths): FP32, P >= 2048
    static constexpr bool wide_ok = std::is_same<T, float>::value && LOG2P >= 11;
    // MODE 2 (teams) exists only for a shared template length with its
    // normalisation rows precomputed, MODE 3 only for a shared length
    // normalised inside the CTA
    static cudaError_t launch(bool sd, int mode, const XcorrParams<T> &p, int nblocks, int ngroups, cudaStream_t s)
    {
        if (p.ticket)
        {
            if constexpr (persist_ok)
            {
                if (sd && mode == 2) return go<true, 2, true>(p, nblocks, ngroups, s);
                if (!sd && mode == 4) return go<false, 4, true>(p, nblocks, ngroups, s);
            }
            return cudaErrorInvalidValue;
        }
        if (sd)
        {
            if (mode == 3) return cudaErrorInvalidValue;
            if (mode == 2) return go<true, 2>(p, nblocks, ngroups, s);
            return mode == 1 ? go<true, 1>(p, nblocks, ngroups, s) : go<true, 0>(p, nblocks, ngroups, s);
        }
        if (mode == 2) return cudaErrorInvalidValue;
        if (mode == 3) return go<false, 3>(p, nblocks, ngroups, s);
        if (mode == 4)
        {
            if constexpr (wide_ok) return go<false, 4>(p, nblocks, ngroups, s);
            else return cudaErrorInvalidValue;
        }
        return mode == 1 ? go<false, 1>(p, nblocks, ngroups, s) : go<false, 0>(p, nblocks, ngroups, s);
    }
    static cudaError_t spectra(const SpecParams<T> &p, int nt, cudaStream_t s)
    {
        constexpr int P = 1 << LOG2P;
        size_t bytes = sizeof(cx<T>) * spad_size(P) + 64 * sizeof(double);
        auto k = template_spectra_kernel<T, LOG2P>;
        static SmemCap cap;
        cudaError_t e = raise_smem_cap(k, bytes, cap);
        if (e != cudaSuccess) return e;
        k<<<nt, kThreads, bytes, s>>>(p);
        return cudaGetLastError();
    }
};

template <class T, int LO, int HI> struct XcorrDispatch
{
    static size_t smem(int log2p, bool sd, int mode, int S)
    {
        if (log2p == LO) return XcorrTable<T, LO>::smem(sd, mode, S);
        if constexpr (LO < HI) return XcorrDispatch<T, LO + 1, HI>::smem(log2p, sd, mode, S);
        return 0;
    }
    static cudaError_t launch(int log2p, bool sd, int mode, const XcorrParams<T> &p, int nb, int ng, cudaStream_t s)
    {
        if (log2p == LO) return XcorrTable<T, LO>::launch(sd, mode, p, nb, ng, s);
        if constexpr (LO < HI) return XcorrDispatch<T, LO + 1, HI>::launch(log2p, sd, mode, p, nb, ng, s);
        return cudaErrorInvalidValue;
    }
    static cudaError_t spectra(int log2p, const SpecParams<T> &p, int nt, cudaStream_t s)
    {
        if (log2p == LO) return XcorrTable<T, LO>::spectra(p, nt, s);
        if constexpr (LO < HI) return XcorrDispatch<T, LO + 1, HI>::spectra(log2p, p, nt, s);
        return cudaErrorInvalidValue;
    }
};

using Dispatch = XcorrDispatch<MFGPU_T, fft_limits<MFGPU_T>::lo, fft_limits<MFGPU_T>::hi>;

template <> size_t xcorr_smem_bytes<MFGPU_T>(int log2p, bool shared_den, int mode, int S)
{
    return Dispatch::smem(log2p, shared_den, mode, S);
}

template <>
cudaError_t launch_xcorr<MFGPU_T>(int log2p, bool shared_den, int mode, const XcorrParams<MFGPU_T> &p, int nblocks,
                                  int ngroups, cudaStream_t s)
{
    return Dispatch::launch(log2p, shared_den, mode, p, nblocks, ngroups, s);
}

template <> cudaError_t launch_spectra<MFGPU_T>(int log2p, const SpecParams<MFGPU_T> &p, int nt, cudaStream_t s)
{
    return Dispatch::spectra(log2p, p, nt, s);
}

template <>
cudaError_t launch_den<MFGPU_T>(const MFGPU_T *x, long ldx, int L, MFGPU_T *den, long ldd, MFGPU_T tol, int nblocks,
                                int nch, cudaStream_t s)
{
    const size_t bytes = DenLayout<MFGPU_T>::bytes(L);
    auto k = den_kernel<MFGPU_T>;
    static SmemCap cap;
    cudaError_t e = raise_smem_cap(k, bytes, cap);
    if (e != cudaSuccess) return e;
    k<<<dim3(nblocks, nch), kThreads, bytes, s>>>(x, ldx, L, den, ldd, tol);
    return cudaGetLastError();
}

template <> void twiddle_table<MFGPU_T>(int log2p, std::vector<cx<MFGPU_T>> &out)
{
    build_twiddle_table<MFGPU_T>(log2p, out);
}

template <> void twiddle_split<MFGPU_T>(int log2p, std::vector<cx<MFGPU_T>> &out)
{
    build_twiddle_split<MFGPU_T>(log2p, out);
}

template <>
cudaError_t launch_dead<MFGPU_T>(const MFGPU_T *x, long ldx, int nch, long n, unsigned char *dead, MFGPU_T *pmin,
                                 MFGPU_T *pmax, int nchunks, cudaStream_t s, float *range)
{
    int chunk = (int) ((n + nchunks - 1) / nchunks);
    dim3 grid(nchunks, nch);
    minmax_partial_kernel<MFGPU_T><<<grid, kThreads, 0, s>>>(x, ldx, n, chunk, pmin, pmax, nchunks);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    minmax_final_kernel<MFGPU_T><<<nch, 256, 0, s>>>(pmin, pmax, nchunks, dead, range);
    return cudaGetLastError();
}

// Reference debug spectrum: X[k] = sum_j brev[j] exp(-2 pi i j k / nfft),
// brev = reverse((b - mean)/||b - mean||) (src/matchedFilter.cpp:168-190,
// :595-620), evaluated directly in FP64 with exact integer phase reduction.
template <class T>
__global__ void ref_spectrum_kernel(const double *b, int L, int nfft, T *out)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > nfft / 2) return;
    double mean = 0;
    for (int j = 0; j < L; ++j) mean += b[j];
    mean /= (double) L;
    double nrm = 0;
    for (int j = 0; j < L; ++j) { double d = b[j] - mean; nrm += d * d; }
    double inv = nrm > 0 ? 1.0 / sqrt(nrm) : 0.0;
    double re = 0, im = 0;
    for (int j = 0; j < L; ++j)
    {
        double v = (b[L - 1 - j] - mean) * inv;
        long long m = ((long long) j * k) % nfft;
        double sn, cs;
        sincospi(2.0 * (double) m / (double) nfft, &sn, &cs);
        re += v * cs;
        im -= v * sn;
    }
    out[2 * k] = (T) re;
    out[2 * k + 1] = (T) im;
}

template <>
cudaError_t launch_ref_spectrum<MFGPU_T>(const double *tmpl, int L, int nfft, MFGPU_T *out, cudaStream_t s)
{
    ref_spectrum_kernel<MFGPU_T><<<(nfft / 2 + 1 + 127) / 128, 128, 0, s>>>(tmpl, L, nfft, out);
    return cudaGetLastError();
}

// Shift and stack, src/matchedFilter.cpp:1341-1362: out[k] = sum_t w_t |rho_t[k + shift_t]|
// (or without the absolute value), templates accumulated in index order.
// Lags before 0 contribute nothing.
template <class T>
__global__ void stack_kernel(const T *rho, long ldr, int nt, const int *shifts, const T *weights, int stack_abs,
                             int outlen, T *out)
{
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= outlen) return;
    T acc = 0;
    for (int t = 0; t < nt; ++t)
    {
        long lag = (long) k + shifts[t];
        T v = lag >= 0 ? rho[(long) t * ldr + lag] : (T) 0;
        acc = acc + weights[t] * (stack_abs ? (T) fabs(v) : v);
    }
    out[k] = acc;
}

template <>
cudaError_t launch_stack<MFGPU_T>(const MFGPU_T *rho, long ldr, int nt, const int *shifts, const MFGPU_T *weights,
                                  int stack_abs, int outlen, MFGPU_T *out, cudaStream_t s)
{
    stack_kernel<MFGPU_T><<<(outlen + 255) / 256, 256, 0, s>>>(rho, ldr, nt, shifts, weights, stack_abs, outlen,
                                                              out);
    return cudaGetLastError();
}

}  // namespace mfgpu
