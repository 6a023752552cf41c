// fix_params.h -- parameters of the FP32 fix-up kernel (kernels_fix.cuh),
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
// over K/16 steps) plus C2 sqrt(L) / s for the split's subnormal floor (FP16
// subnormal spacing 2^-24, half of it per operand, in units of the strip scale s).
constexpr float kFixTol = 2.0e-5f;
constexpr float kFixFftK = 8.0f;
constexpr float kFixTcC1 = 2.0e-6f;
constexpr float kFixTcC2 = 0x1p-24f;

// Fix-up batches: the templates of a channel sorted by length, kFixBatch per
// batch; coefficients (demeaned, unit norm, FP32) interleaved as
// [i][kFixBatch] and zero past each template's length.
struct FixParams
{
    const float *x;
    long ldx;
    float *rho;
    long ldr;
    const unsigned char *flags;  // per channel and run, row stride ldf
    long ldf;
    int nruns;                   // runs per channel row that may be flagged
    int nspans;                  // (nruns + 31) / 32
    int nbatch;
    const int *bch;              // channel of each batch
    const int *btid;             // [nbatch][kFixBatch] template ids, -1 empty
    const long *boff;            // first coefficient of each batch in bco
    const int *bL;               // longest template of each batch
    const float *bco;
    const float *bsum;           // per template: sum of its FP32 coefficients
    const int *tlen;
    const int *nvalid;
    float tol;
    int Lmax;                    // longest template (shared-memory rows)
    // tensor-core candidate flags (one bit per 64 lags of each row), or null
    unsigned *pk_flags;
    int pk_words;
    float pk_thr;
    int pk_len;
    // fused FFT candidates: a byte per (template, block) slot to recount, or null
    unsigned char *pk_dirty;
    int pk_stride;
    const int *row_S;            // per template block length (length buckets), or null
    int S0;
};

}  // namespace mfgpu
