// k_mixed.cu - mixed-precision solve (FP32 inner CR + V-cycle, FP64 outer
// iterative refinement).  Placeholder translation unit until it is built.
#include "mph_device.cuh"
