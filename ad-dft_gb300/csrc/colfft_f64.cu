// Column pipeline of the local H psi, double instantiations.
#include "colfft.cuh"
#define CF_REAL double
#include "colfft_launch.inc"
