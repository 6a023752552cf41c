// mf_f32.cu -- FP32 instantiation of the matched-filter kernels and launchers.
#define MFGPU_T float
#include "mf_launch.cuh"
