// Fermi-Dirac occupations with the chemical potential found by a fixed number
// of bisection steps, on the device (one CTA).  Reference:
// src/addft/physics/occupation.py:25-49 (80 bisection steps, bracket
// [min eps - 30 sigma - 1, max eps + 30 sigma + 1], f = sigmoid((mu - eps)/sigma)).
#include "common.cuh"

namespace addft {

__device__ __forceinline__ double sigmoid(double x) {
  if (x >= 0.0) return 1.0 / (1.0 + exp(-x));
  const double e = exp(x);
  return e / (1.0 + e);
}

__device__ double block_sum(double v, double *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
  const int nw = (blockDim.x + 31) >> 5;
  for (int w = 0; w < nw; ++w) s += red[w];
  return s;
}

__device__ double block_minmax(double v, double *red, bool is_max) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    const double u = __shfl_down_sync(0xffffffffu, v, o);
    v = is_max ? fmax(v, u) : fmin(v, u);
  }
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = red[0];
  const int nw = (blockDim.x + 31) >> 5;
  for (int w = 1; w < nw; ++w) s = is_max ? fmax(s, red[w]) : fmin(s, red[w]);
  return s;
}

__global__ void k_occupations(int nk, int nb, const double *__restrict__ eig, const double *__restrict__ kw,
                              double nelec, double sigma, double gs, int iters, double *__restrict__ occ,
                              double *__restrict__ mu_out) {
  __shared__ double red[32];
  const int n = nk * nb;
  double lo_v = 1e300, hi_v = -1e300;
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    lo_v = fmin(lo_v, eig[t]);
    hi_v = fmax(hi_v, eig[t]);
  }
  double lo = block_minmax(lo_v, red, false) - 30.0 * sigma - 1.0;
  double hi = block_minmax(hi_v, red, true) + 30.0 * sigma + 1.0;
  for (int it = 0; it < iters; ++it) {
    const double mid = 0.5 * (lo + hi);
    double s = 0.0;
    for (int t = threadIdx.x; t < n; t += blockDim.x) s += kw[t / nb] * sigmoid((mid - eig[t]) / sigma);
    const double ne = block_sum(s, red) * gs;
    if (ne > nelec) hi = mid; else lo = mid;
  }
  const double mu = 0.5 * (lo + hi);
  for (int t = threadIdx.x; t < n; t += blockDim.x) occ[t] = sigmoid((mu - eig[t]) / sigma);
  if (threadIdx.x == 0) *mu_out = mu;
}

}  // namespace addft

using namespace addft;

extern "C" addft_status addft_occupations(int nk, int nb, const double *eig, const double *kweights,
                                          double nelec, double sigma, double spin_deg, int iters,
                                          double *occ, double *mu, void *stream) {
  ADDFT_REQUIRE(nk >= 1 && nb >= 1 && eig && kweights && occ && mu && sigma > 0 && iters >= 0,
                ADDFT_INVALID_ARG, "occupations: bad arguments");
  k_occupations<<<1, 256, 0, as_stream(stream)>>>(nk, nb, eig, kweights, nelec, sigma, spin_deg, iters, occ, mu);
  return check_launch("k_occupations");
}
