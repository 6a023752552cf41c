// tc_params.h -- parameters and shared-memory layout of the tensor-core
// correlator (kernels_tc.cuh), visible to the host code.
#pragma once
#include <cstddef>
#include <cuda_fp16.h>

namespace mfgpu {

constexpr int kTcRows = 128;              // MMA M: rows of a tile
constexpr int kTcLags = 8 * kTcRows;      // lags per tile (8 phases per row)
constexpr int kTcThreads = 384;           // warp 0 MMA issue, warps 1-3 strips, warps 4-11 epilogue
constexpr int kTcProducers = 96;
constexpr int kTcEpiWarps = 8;            // two warpgroups, each covering the 128 rows

struct TcParams
{
    const float *x;            // channel rows, stride ldx (zero tail up to tiles * 1024 + Kp)
    long ldx;
    const __half *B;           // per group: hi then lo, each 8 Gp rows x Kp in core-matrix layout
    const float *bscale;       // per (group, slot): 1 / template scale
    const int *grp_chan;       // channel of each group
    const int *grp_tid;        // [ngroups * Gp] template id or -1
    const float *xrange;       // per channel: max - min of the samples
    const float *off;          // per (channel, tile): operand offset of the strip, row stride tiles
    const unsigned char *dead; // per channel dead-trace flag
    const float *den;          // per channel normalisation row, stride ldd
    long ldd;
    float *rho;
    long ldr;
    int nv;                    // valid lags per template
    int Kp, Gp, tmem_cols;
    int ngroups, tiles;
    int *err;
    // peak-candidate flags (null: off): bit c of word t * pk_words + c / 32
    // set when a stored lag of [64c, 64c + 64) of template t exceeds pk_thr
    unsigned *pk_flags;
    int pk_words;
    float pk_thr;
};

// barriers and the TMEM address | 2 strip buffers x (hi, lo) | template bank (hi, lo)
struct TcLayout
{
    static constexpr __host__ __device__ size_t up(size_t v) { return (v + 127) & ~size_t(127); }
    static constexpr __host__ __device__ size_t strip(int Kp) { return (size_t) (kTcLags + Kp); }  // halves
    static constexpr __host__ __device__ size_t off_A() { return 128; }
    static constexpr __host__ __device__ size_t off_B(int Kp) { return off_A() + up(8 * strip(Kp)); }
    static constexpr __host__ __device__ size_t b_bytes(int Kp, int Gp) { return (size_t) 32 * Gp * Kp; }
    static constexpr __host__ __device__ size_t bytes(int Kp, int Gp) { return off_B(Kp) + b_bytes(Kp, Gp); }
};

}  // namespace mfgpu
