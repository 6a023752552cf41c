// mf_f64.cu -- FP64 instantiation of the matched-filter kernels and launchers.
#define MFGPU_T double
#include "mf_launch.cuh"
