// fixup.cu -- launchers of the accuracy safeguards and the direct correlator (kernels_fix.cuh).
#include "launch.h"
#include "kernels_fix.cuh"

namespace mfgpu {

cudaError_t launch_den_robust(const float *x, long ldx, int L, float *den, long ldd, float tol, float4 *rstat,
                              long ldrs, float2 *cst, long ldc, int nblocks, int nch, cudaStream_t s)
{
    const size_t bytes = DenRobustLayout::bytes(L);
    static SmemCap cap;
    cudaError_t e = raise_smem_cap(den_robust_kernel, bytes, cap);
    if (e != cudaSuccess) return e;
    den_robust_kernel<<<dim3(nblocks, nch), kThreads, bytes, s>>>(x, ldx, L, den, ldd, tol, rstat, ldrs, cst, ldc);
    return cudaGetLastError();
}

cudaError_t launch_fix_flag_fft(const float2 *cst, long ldc, long nchunks, int S, int N, int nblocks, int nch,
                                const float4 *rstat, long ldrs, int nruns, const int *dlags, const unsigned char *dead,
                                unsigned *fbits, int *flist, int *fcount, float coef2, cudaStream_t s)
{
    fix_flag_fft_kernel<<<dim3((nblocks + 7) / 8, nch), 256, 0, s>>>(cst, ldc, nchunks, S, N, nblocks, rstat, ldrs,
                                                                      nruns, dlags, dead, fbits, flist, fcount, coef2);
    return cudaGetLastError();
}

cudaError_t launch_fix_flag_tc(const float *x, long ldx, int L, const float4 *rstat, long ldrs, int nruns,
                               const int *dlags, int tiles, int nch, const unsigned char *dead, const float *xrange,
                               float *off, unsigned *fbits, int *flist, int *fcount, float c1, float c2, float tau,
                               cudaStream_t s)
{
    fix_flag_tc_kernel<<<dim3((tiles + 7) / 8, nch), 256, 0, s>>>(x, ldx, L, rstat, ldrs, nruns, dlags, tiles, dead,
                                                                   xrange, off, fbits, flist, fcount, c1, c2, tau);
    return cudaGetLastError();
}

cudaError_t launch_set_int(int *p, int v, cudaStream_t s)
{
    fix_set_int_kernel<<<1, 1, 0, s>>>(p, v);
    return cudaGetLastError();
}

template <class T> int fixup_warps(int Lmax, int dev_smem)
{
    const size_t w = fix_warp_bytes<T>(Lmax);
    const int k = (int) ((size_t) dev_smem / w);
    return k < 1 ? 0 : (k < kFixWarps ? k : kFixWarps);
}
template int fixup_warps<float>(int, int);
template int fixup_warps<double>(int, int);

template <class T>
cudaError_t launch_fix_prep(const double *tmpl, const long *toff, const int *tlen, const int *btid, const long *boff,
                            const int *bL, int nbatch, T *bco, T *bsum, cudaStream_t s)
{
    fix_prep_kernel<T><<<nbatch * kFixBatch, 256, 0, s>>>(tmpl, toff, tlen, btid, boff, bL, bco, bsum);
    return cudaGetLastError();
}
template cudaError_t launch_fix_prep<float>(const double *, const long *, const int *, const int *, const long *,
                                            const int *, int, float *, float *, cudaStream_t);
template cudaError_t launch_fix_prep<double>(const double *, const long *, const int *, const int *, const long *,
                                             const int *, int, double *, double *, cudaStream_t);

template <class T> cudaError_t launch_fixup(const FixParams<T> &p, int nctas, int warps, cudaStream_t s)
{
    const size_t bytes = (size_t) warps * fix_warp_bytes<T>(p.Lmax);
    static SmemCap cap;
    cudaError_t e = raise_smem_cap(fixup_kernel<T>, bytes, cap);
    if (e != cudaSuccess) return e;
    fixup_kernel<T><<<nctas, 32 * warps, bytes, s>>>(p);
    return cudaGetLastError();
}
template cudaError_t launch_fixup<float>(const FixParams<float> &, int, int, cudaStream_t);
template cudaError_t launch_fixup<double>(const FixParams<double> &, int, int, cudaStream_t);

template <class T>
cudaError_t launch_fix_rescan(const T *rho, long ldr, int nt, int pk_stride, const unsigned char *dirty,
                              const int *row_S, const int *row_nblk, int S0, int nblk0, const int *nvalid, int pk_len,
                              T thr, int *cnt, int *idx, T *val, cudaStream_t s)
{
    const long ns = (long) nt * pk_stride;
    const long warps = (ns + 31) / 32;
    fix_rescan_kernel<T><<<(unsigned) ((warps + 7) / 8), 256, 0, s>>>(rho, ldr, nt, pk_stride, dirty, row_S, row_nblk,
                                                                       S0, nblk0, nvalid, pk_len, thr, cnt, idx, val);
    return cudaGetLastError();
}
template cudaError_t launch_fix_rescan<float>(const float *, long, int, int, const unsigned char *, const int *,
                                              const int *, int, int, const int *, int, float, int *, int *, float *,
                                              cudaStream_t);
template cudaError_t launch_fix_rescan<double>(const double *, long, int, int, const unsigned char *, const int *,
                                               const int *, int, int, const int *, int, double, int *, int *,
                                               double *, cudaStream_t);

}  // namespace mfgpu
