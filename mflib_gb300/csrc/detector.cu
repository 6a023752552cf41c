// detector.cu -- launchers of the single-channel detector kernels
// (kernels_detect.cuh) for both sample types.
#include "launch.h"
#include "kernels_detect.cuh"

namespace mfgpu {

template <class T>
cudaError_t launch_det_reduce(const T *rho, long ldr, int nt, long len, int use_abs, T *det, int *id, cudaStream_t s)
{
    det_reduce_kernel<T><<<(unsigned) ((len + 255) / 256), 256, 0, s>>>(rho, ldr, nt, len, use_abs, det, id);
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_det_single(const T *rho, long ldr, int nt, long len, int use_abs, T *out, cudaStream_t s)
{
    det_single_kernel<T><<<dim3((unsigned) ((len + 255) / 256), (unsigned) nt), 256, 0, s>>>(rho, ldr, nt, len,
                                                                                           use_abs, out);
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_det_refine(const T *rho, long ldr, const T *x, long ldx, const DetectParams &q, cudaStream_t s)
{
    if (q.ndet <= 0) return cudaSuccess;
    const long threads = 32L * q.ndet;
    det_refine_kernel<T><<<(unsigned) ((threads + 255) / 256), 256, 0, s>>>(rho, ldr, x, ldx, q);
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_amp(const double *b, int L, const T *y, long ld, int nw, double *gr, double *sr, int *valid,
                       cudaStream_t s)
{
    if (nw <= 0) return cudaSuccess;
    const long threads = 32L * nw;
    amp_kernel<T><<<(unsigned) ((threads + 255) / 256), 256, 0, s>>>(b, L, y, ld, nw, gr, sr, valid);
    return cudaGetLastError();
}

template cudaError_t launch_amp<float>(const double *, int, const float *, long, int, double *, double *, int *,
                                       cudaStream_t);
template cudaError_t launch_amp<double>(const double *, int, const double *, long, int, double *, double *, int *,
                                        cudaStream_t);
template cudaError_t launch_det_reduce<float>(const float *, long, int, long, int, float *, int *, cudaStream_t);
template cudaError_t launch_det_reduce<double>(const double *, long, int, long, int, double *, int *, cudaStream_t);
template cudaError_t launch_det_single<float>(const float *, long, int, long, int, float *, cudaStream_t);
template cudaError_t launch_det_single<double>(const double *, long, int, long, int, double *, cudaStream_t);
template cudaError_t launch_det_refine<float>(const float *, long, const float *, long, const DetectParams &,
                                              cudaStream_t);
template cudaError_t launch_det_refine<double>(const double *, long, const double *, long, const DetectParams &,
                                               cudaStream_t);

}  // namespace mfgpu
