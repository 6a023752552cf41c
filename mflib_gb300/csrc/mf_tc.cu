// mf_tc.cu -- launchers of the tensor-core correlator (kernels_tc.cuh).
#include "launch.h"
#include "kernels_tc.cuh"

namespace mfgpu {

size_t tc_smem_bytes(int Kp, int Gp) { return TcLayout::bytes(Kp, Gp); }

cudaError_t launch_tc_bank(const double *tmpl, const long *toff, const int *tlen, const int *grp_tid, int ngroups,
                           int Gp, int Kp, __half *B, float *bscale, bool bf16, cudaStream_t s)
{
    if (bf16) tc_bank_kernel<true><<<ngroups * Gp, 256, 0, s>>>(tmpl, toff, tlen, grp_tid, Gp, Kp, B, bscale);
    else tc_bank_kernel<false><<<ngroups * Gp, 256, 0, s>>>(tmpl, toff, tlen, grp_tid, Gp, Kp, B, bscale);
    return cudaGetLastError();
}

template <bool BF> static cudaError_t launch_tc_xcorr_t(const TcParams &p, int nctas, cudaStream_t s)
{
    const size_t bytes = TcLayout::bytes(p.Kp, p.Gp);
    static SmemCap cap;
    cudaError_t e = raise_smem_cap(tc_xcorr_kernel<BF>, bytes, cap);
    if (e != cudaSuccess) return e;
    tc_xcorr_kernel<BF><<<nctas, kTcThreads, bytes, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_tc_xcorr(const TcParams &p, int nctas, bool bf16, cudaStream_t s)
{
    return bf16 ? launch_tc_xcorr_t<true>(p, nctas, s) : launch_tc_xcorr_t<false>(p, nctas, s);
}

}  // namespace mfgpu
