// kernels_ring.cuh -- the device ring of recent samples per channel
// (mfgpu_ring): a request window gathered from the ring into a matched-filter
// object's signal rows on the device, so only appended samples cross PCIe.
#pragma once
#include <cuda_runtime.h>

namespace mfgpu {

// rows one gather can fill (the ring channel of each row travels as a
// kernel parameter)
constexpr int kRingMaxRows = 256;

struct RingRows
{
    int src[kRingMaxRows];  // ring channel of destination row r
};

// x[r * ldx + i] = ring[src[r] * cap + (start + i) mod cap] for i in [0, n),
// r = blockIdx.y < rows; grid-stride over the samples, coalesced on both
// sides (one wrap at most per row).
template <class T>
__global__ void ring_gather_kernel(const T *ring, long cap, RingRows rr, long long start, int n, T *x, long ldx)
{
    const int r = blockIdx.y;
    const long p0 = (long) (start % cap);
    const T *src = ring + (long) rr.src[r] * cap;
    T *dst = x + (long) r * ldx;
    for (long i = blockIdx.x * (long) blockDim.x + threadIdx.x; i < n; i += (long) gridDim.x * blockDim.x)
    {
        long p = p0 + i;
        if (p >= cap) p -= cap;
        dst[i] = src[p];
    }
}

}  // namespace mfgpu
