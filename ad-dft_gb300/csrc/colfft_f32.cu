// Column pipeline of the local H psi, float instantiations.
#include "colfft.cuh"
#define CF_REAL float
#include "colfft_launch.inc"
