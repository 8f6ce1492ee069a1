// Two-pass plane kernels, FP32 instantiations.
#include "plane2.cuh"
#define PL2_REAL float
#include "plane2_launch.inc"
