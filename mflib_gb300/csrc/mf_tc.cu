// mf_tc.cu -- launchers of the tensor-core correlator (kernels_tc.cuh).
#include "launch.h"
#include "kernels_tc.cuh"

namespace mfgpu {

size_t tc_smem_bytes(int Kp, int Gp) { return TcLayout::bytes(Kp, Gp); }

cudaError_t launch_tc_bank(const double *tmpl, const long *toff, const int *tlen, const int *grp_tid, int ngroups,
                           int Gp, int Kp, __half *B, float *bscale, cudaStream_t s)
{
    tc_bank_kernel<<<ngroups * Gp, 256, 0, s>>>(tmpl, toff, tlen, grp_tid, Gp, Kp, B, bscale);
    return cudaGetLastError();
}

cudaError_t launch_tc_xcorr(const TcParams &p, int nctas, cudaStream_t s)
{
    const size_t bytes = TcLayout::bytes(p.Kp, p.Gp);
    static SmemCap cap;
    cudaError_t e = raise_smem_cap(tc_xcorr_kernel, bytes, cap);
    if (e != cudaSuccess) return e;
    tc_xcorr_kernel<<<nctas, kTcThreads, bytes, s>>>(p);
    return cudaGetLastError();
}

}  // namespace mfgpu
