// fix_params.h -- parameters of the fix-up kernel (kernels_fix.cuh),
// shared by the host code that fills them.
#pragma once

namespace mfgpu {

// templates per fix-up batch
constexpr int kFixBatch = 16;
// The coefficient tolerance the error bounds guard (|drho| against the FP64
// Pearson coefficient), and the bounds' constants: FFT form K 2^-24 sqrt(E_b)
// (a single-precision FFT's error grows as sqrt(log N) times the unit
// roundoff; K = 8 covers N up to 8192 several times over); tensor-core form
// C1 ||x - off|| (FP16 hi+lo keeps 2^-22 of each operand, FP32 accumulation
// over K/16 steps) plus C2 / s for the split's subnormal floor: a low part
// below FP16's normal range is rounded to its 2^-24 spacing, an error of at
// most 2^-25 / s per sample in signal units; summed against a unit-norm
// template, independent roundings give a standard deviation of
// 2^-25 / (s sqrt 3), and C2 = 2^-23 is six of those.
constexpr float kFixTol = 2.0e-5f;
constexpr float kFixFftK = 8.0f;
constexpr float kFixTcC1 = 2.0e-6f;
constexpr float kFixTcC2 = 0x1p-23f;
// BF16 hi+lo leaves each operand with a representation error of at most
// 2^-16 of its value (8-bit significands: 2^-8 for hi, again for lo; FP16:
// 2^-22), and drops lo*lo products of the same order.  Like the FP16
// subnormal term these are independent roundings: against a unit-norm
// template b the three sums over a window have standard deviations of at
// most 2^-16 max|b| ||y - off|| / sqrt(12) (the splits of y and b) and / 3
// (the dropped products), 2^-16 max|b| ||y - off|| / 2 together.  Six of
// those, 3 2^-16 max|b|, are added to the FP16 constant; the host takes
// max|b| over the object's templates (kFixTcC1Bf16Per is its factor).
constexpr float kFixTcC1Bf16Per = 3.f * 0x1p-16f;
constexpr float kFixTcC2Bf16 = 0.f;

// Fix-up batches: the templates of a channel sorted by length, kFixBatch per
// batch; coefficients (demeaned, unit norm, in the sample type) interleaved
// as [i][kFixBatch] and zero past each template's length.  Two uses of the
// same kernel: the FP32 fix-up of listed runs (flist), and the direct
// time-domain correlation of templates too long for any FFT plan (every run
// of batches dir_b0 .. dir_b0 + ndir - 1, both sample types).
template <class T> struct FixParams
{
    const T *x;
    long ldx;
    T *rho;
    long ldr;
    const int *flist;            // listed runs: c * ldf + r (null: direct mode)
    const int *fcount;           // number of listed runs
    long ldf;
    int nruns;                   // runs per channel row
    int nbmax;                   // most batches of one channel (list mode)
    const int *chan_b0;          // first batch of each channel (list mode)
    const int *chan_nb;          // batches of each channel (list mode)
    int dir_b0, ndir;            // direct mode: the batches to correlate
    const int *bch;              // channel of each batch
    const unsigned char *dead;   // per channel dead-trace flag (direct mode writes zeros)
    const int *btid;             // [nbatch][kFixBatch] template ids, -1 empty
    const long *boff;            // first coefficient of each batch in bco
    const int *bL;               // longest template of each batch
    const T *bco;
    const T *bsum;               // per template: sum of its rounded coefficients
    const int *tlen;
    const int *nvalid;
    T tol;
    int Lmax;                    // longest template of the batches (shared-memory rows)
    // tensor-core candidate flags (one bit per 64 lags of each row), or null
    unsigned *pk_flags;
    int pk_words;
    T pk_thr;
    int pk_len;
    // fused FFT candidates: a byte per (template, block) slot to recount, or null
    unsigned char *pk_dirty;
    int pk_stride;
    const int *row_S;            // per template block length (length buckets), or null
    int S0;
};

}  // namespace mfgpu
