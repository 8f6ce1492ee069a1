// Two-pass x-line kernels, FP32 instantiations.
#include "xline2.cuh"
#define XL2_REAL float
#include "xline2_launch.inc"
