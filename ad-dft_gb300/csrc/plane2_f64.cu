// Two-pass plane kernels, FP64 instantiations.
#include "plane2.cuh"
#define PL2_REAL double
#include "plane2_launch.inc"
