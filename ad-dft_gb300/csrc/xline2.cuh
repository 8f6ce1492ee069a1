// Two-pass register FFT along x for the H psi and density x-line stage.
//
// For n1 = P Q, an x-line (fixed i2, i3) of the slab is transformed with the
// data held in registers and one shared-memory exchange per direction.  Lanes
// are tile columns (i3), warps index the sub-transforms:
//   inverse pass 1 (warp b < Q):  x[b + Q a], a < P, straight from the slab
//                                 rows -> DFT_P -> * W_N^{-b k1} -> smem row k1 Q + b
//   inverse pass 2 (warp k1 < P): smem rows k1 Q + b -> DFT_Q -> y at x = k1 + P k2
// For H psi the same registers then take V(r) and start the forward transform
// (the stride-P subsequence x = q + P p is exactly what warp k1 holds):
//   forward pass 2 (warp q < P):  DFT_Q -> * W_N^{q j1} -> smem row j1 P + q
//   forward pass 3 (warp j1 < Q): smem rows j1 P + q -> DFT_P -> X at x = j1 + Q j2,
//                                 written to the slab rows pass 1 read.
// Rows of inactive x-planes are skipped on load (zero) and on store.
#pragma once
#include "transforms.cuh"

namespace addft {

template <typename R, int P, int Q, int MODE>
__global__ void __launch_bounds__(512)
k_xline2(PlanDev pd, XArgs<R> a) {
  using C = typename Cx<R>::T;
  constexpr int N = P * Q;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *buf = reinterpret_cast<C *>(smem_raw);   // N rows x 32 lanes
  C *twN = buf + N * 32;                      // e^{-2 pi i t / N}
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int n2 = pd.n2, n3 = pd.n3, n2n3 = n2 * n3;
  const int T = a.t3;
  const int i2 = blockIdx.x / a.ntile3;
  const int c0 = (blockIdx.x - i2 * a.ntile3) * T;
  const int tw_ = min(T, n3 - c0);
  const bool col = lane < tw_;
  const C *g1 = twiddles<R>(pd, 0);
  for (int i = threadIdx.x; i < N; i += blockDim.x) twN[i] = g1[i];
  const C z = czero<C>();
  const int colofs = i2 * n3 + c0 + lane;     // offset of this lane's column within a plane / x-row

  // inverse pass 1 for slab band bb (warps < Q)
  auto pass1 = [&](int bb) {
    if (w < Q) {
      const int b = w;
      const C *Wb = a.W + (size_t)bb * pd.np * n2n3 + colofs;
      C v[P];
#pragma unroll
      for (int aa = 0; aa < P; ++aa) {
        const int p = pd.plane_of_i1[b + Q * aa];
        v[aa] = (p >= 0 && col) ? Wb[p * n2n3] : z;
      }
      dft_reg<P, true>(v);
#pragma unroll
      for (int k1 = 0; k1 < P; ++k1) buf[(k1 * Q + b) * 32 + lane] = cmulc(v[k1], twN[b * k1]);
    }
  };

  if (MODE == XM_DENSITY) {
    double acc[Q];
#pragma unroll
    for (int k2 = 0; k2 < Q; ++k2) acc[k2] = 0.0;
    const int per = (a.nbatch + a.nsplit - 1) / a.nsplit;
    const int bb0 = blockIdx.y * per, bb1 = min(a.nbatch, bb0 + per);
    __syncthreads();
    for (int bb = bb0; bb < bb1; ++bb) {
      pass1(bb);
      __syncthreads();
      if (w < P) {
        const int k1 = w;
        C y[Q];
#pragma unroll
        for (int b = 0; b < Q; ++b) y[b] = buf[(k1 * Q + b) * 32 + lane];
        dft_reg<Q, true>(y);
        const double wb = a.wocc[bb] * a.dscale;
#pragma unroll
        for (int k2 = 0; k2 < Q; ++k2)
          acc[k2] += wb * ((double)y[k2].x * (double)y[k2].x + (double)y[k2].y * (double)y[k2].y);
      }
      __syncthreads();
    }
    if (w < P && col) {
      double *dst = (a.nsplit > 1 ? a.part + (size_t)blockIdx.y * a.N : a.rho) + colofs;
      const int acc_mode = a.nsplit > 1 ? 0 : a.rho_acc;
#pragma unroll
      for (int k2 = 0; k2 < Q; ++k2) {
        double *d = dst + (size_t)(w + P * k2) * n2n3;
        *d = acc_mode ? *d + acc[k2] : acc[k2];
      }
    }
    return;
  }

  // H psi: inverse, V(r), forward
  const int bb = blockIdx.y;
  __syncthreads();
  pass1(bb);
  __syncthreads();
  C y[Q];
  if (w < P) {
    const int k1 = w;
#pragma unroll
    for (int b = 0; b < Q; ++b) y[b] = buf[(k1 * Q + b) * 32 + lane];
    dft_reg<Q, true>(y);
    const R *v = a.v + colofs;
#pragma unroll
    for (int k2 = 0; k2 < Q; ++k2) {
      const R s = col ? v[(size_t)(k1 + P * k2) * n2n3] * a.vscale : (R)0;
      y[k2] = cscale(y[k2], s);
    }
    dft_reg<Q, false>(y);
#pragma unroll
    for (int j1 = 0; j1 < Q; ++j1) y[j1] = cmul(y[j1], twN[k1 * j1]);
  }
  __syncthreads();
  if (w < P) {
#pragma unroll
    for (int j1 = 0; j1 < Q; ++j1) buf[(j1 * P + w) * 32 + lane] = y[j1];
  }
  __syncthreads();
  if (w < Q) {
    const int j1 = w;
    C v[P];
#pragma unroll
    for (int q = 0; q < P; ++q) v[q] = buf[(j1 * P + q) * 32 + lane];
    dft_reg<P, false>(v);
    C *Wb = a.W + (size_t)bb * pd.np * n2n3 + colofs;
    if (col) {
#pragma unroll
      for (int j2 = 0; j2 < P; ++j2) {
        const int p = pd.plane_of_i1[j1 + Q * j2];
        if (p >= 0) Wb[p * n2n3] = v[j2];
      }
    }
  }
}

// Launches the two-pass x-line kernel if (P, Q) of the x axis is instantiated;
// returns ADDFT_UNSUPPORTED otherwise (the caller falls back to k_xline).
template <typename R, int MODE>
addft_status launch_xline2(const PlanDev &pd, int nbatch, XArgs<R> a, cudaStream_t st);

}  // namespace addft
