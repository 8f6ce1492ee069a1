// Two-pass x-line kernels, FP64 instantiations.
#include "xline2.cuh"
#define XL2_REAL double
#include "xline2_launch.inc"
