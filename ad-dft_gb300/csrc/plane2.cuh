// Two-pass register FFTs for the plane kernels (y and z directions).
//
// Same scheme as the x-line kernel (xline2.cuh): for a length N = P Q the
// line is transformed in two register passes with one shared-memory exchange.
// y-lines (columns i3) map lanes to columns; z-lines (rows i2, only the rows
// that carry sphere points) map lanes to rows, which the odd row pitch keeps
// bank-conflict-free.  The y pass that touches the slab reads (P2) or writes
// (P1) global memory directly, so no separate copy pass remains.  P1 runs all
// of its shared-memory passes in place on one tile per CTA.
#pragma once
#include "transforms.cuh"

namespace addft {

// One radix pass over a batch of lines in shared memory.
//   pass 1 (sub < Q): x[b + Q a] -> DFT_P -> * W_N^{+-b k1} -> dst[k1 Q + b]
//   pass 2 (sub < P): src[k1 Q + b] -> DFT_Q -> dst[k1 + P k2]   (natural order)
// Line `l` addresses element e at base(l) + e * es.
template <int P, int Q, bool INV, typename C>
__device__ __forceinline__ void pass1_line(const C *src, C *dst, int base, int es, int b, const C *twN) {
  constexpr int N = P * Q;
  (void)N;
  C v[P];
#pragma unroll
  for (int a = 0; a < P; ++a) v[a] = src[base + (b + Q * a) * es];
  dft_reg<P, INV>(v);
#pragma unroll
  for (int k1 = 0; k1 < P; ++k1) {
    const C w = twN[b * k1];
    dst[base + (k1 * Q + b) * es] = INV ? cmulc(v[k1], w) : cmul(v[k1], w);
  }
}

template <int P, int Q, bool INV, typename C>
__device__ __forceinline__ void pass2_line(const C *src, C *dst, int base, int es, int k1) {
  C y[Q];
#pragma unroll
  for (int b = 0; b < Q; ++b) y[b] = src[base + (k1 * Q + b) * es];
  dft_reg<Q, INV>(y);
#pragma unroll
  for (int k2 = 0; k2 < Q; ++k2) dst[base + (k1 + P * k2) * es] = y[k2];
}

// z-direction (rows) of a plane tile, active rows only: A -> B -> A
template <int P, int Q, bool INV, typename C>
__device__ __forceinline__ void zfft_rows(C *A, C *B, const int *rows, int nrow, int p3, const C *tw3) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int ngrp = (nrow + 31) >> 5;
  for (int it = w; it < ngrp * Q; it += nw) {
    const int grp = it / Q, b = it - grp * Q;
    const int r = grp * 32 + lane;
    if (r < nrow) pass1_line<P, Q, INV>(A, B, rows[r] * p3, 1, b, tw3);
  }
  __syncthreads();
  for (int it = w; it < ngrp * P; it += nw) {
    const int grp = it / P, k1 = it - grp * P;
    const int r = grp * 32 + lane;
    if (r < nrow) pass2_line<P, Q, INV>(B, A, rows[r] * p3, 1, k1);
  }
  __syncthreads();
}

// Digit-reversed storage.  Pass 2 run in place leaves the element of natural
// index n = k1 + P k2 of a length N = P Q transform at position k1 Q + k2.  P1
// keeps the z direction in this order inside its tile and undoes it in the
// store to the slab, so that one tile per CTA suffices (twice the resident CTAs
// of the two-tile form) and the slab stays in natural order.  (The same scheme
// for P2, with the gather through the permutation, measured slower than the
// two-tile form at every register budget, so P2 keeps two tiles.)
template <int P, int Q>
__device__ __forceinline__ int dr_nat(int s) { return s / Q + P * (s % Q); }   // position -> natural

// CTAs per SM the register budget of P1 is sized for (512 threads each): the largest
// radix sets the register need (FP32: 32 registers at radix <= 9, 42 at 10,
// 64 at 15; FP64 about twice that).
template <typename R, int P2, int Q2, int P3, int Q3>
constexpr int plane2_min_blocks() {
  constexpr int m1 = P2 > Q2 ? P2 : Q2, m2 = P3 > Q3 ? P3 : Q3;
  constexpr int r = m1 > m2 ? m1 : m2;
  constexpr bool r88 = P2 == 8 && Q2 == 8;
  if (sizeof(R) == 4) return r <= 9 && !r88 ? 4 : r <= 10 ? 3 : 2;
  return r <= 10 ? 2 : 1;
}

// Pass 2 in place: A[k1 Q + b] (b < Q) -> DFT_Q -> A[k1 Q + k2].
template <int P, int Q, bool INV, typename C>
__device__ __forceinline__ void pass2_line_ip(C *A, int base, int es, int k1) {
  C y[Q];
#pragma unroll
  for (int b = 0; b < Q; ++b) y[b] = A[base + (k1 * Q + b) * es];
  dft_reg<Q, INV>(y);
#pragma unroll
  for (int k2 = 0; k2 < Q; ++k2) A[base + (k1 * Q + k2) * es] = y[k2];
}

// z-direction (rows) of a plane tile in place, active rows only: natural z in,
// digit-reversed z out.
template <int P, int Q, bool INV, typename C>
__device__ __forceinline__ void zfft_rows_ip(C *A, const int *rows, int nrow, int p3, const C *tw3) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int ngrp = (nrow + 31) >> 5;
  for (int it = w; it < ngrp * Q; it += nw) {
    const int grp = it / Q, b = it - grp * Q;
    const int r = grp * 32 + lane;
    if (r < nrow) pass1_line<P, Q, INV>(A, A, rows[r] * p3, 1, b, tw3);
  }
  __syncthreads();
  for (int it = w; it < ngrp * P; it += nw) {
    const int grp = it / P, k1 = it - grp * P;
    const int r = grp * 32 + lane;
    if (r < nrow) pass2_line_ip<P, Q, INV>(A, rows[r] * p3, 1, k1);
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// P1: sphere -> slab.  Scatter, z inverse (rows, in place: z digit-reversed),
// y inverse pass 1 in place (columns), y pass 2 from the tile straight to the
// global slab plane in natural (y, z) order.
// ---------------------------------------------------------------------------
template <typename R, int P2, int Q2, int P3, int Q3>
__global__ void __launch_bounds__(512, (plane2_min_blocks<R, P2, Q2, P3, Q3>()))
k_plane_inv2(PlanDev pd, const typename Cx<R>::T *__restrict__ psi, long ld_psi, R scale,
             typename Cx<R>::T *__restrict__ W) {
  using C = typename Cx<R>::T;
  constexpr int N2 = P2 * Q2, N3 = P3 * Q3;
  constexpr int p3 = N3 | 1;   // odd row pitch
  constexpr int SP = N2 * p3;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *A = reinterpret_cast<C *>(smem_raw);
  C *tw2 = A + SP;
  C *tw3 = tw2 + N2;
  const int p = blockIdx.x, band = blockIdx.y;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const C z = czero<C>();
  for (int i = threadIdx.x; i < SP; i += blockDim.x) A[i] = z;
  const C *g2 = twiddles<R>(pd, 1), *g3 = twiddles<R>(pd, 2);
  for (int i = threadIdx.x; i < N2; i += blockDim.x) tw2[i] = g2[i];
  for (int i = threadIdx.x; i < N3; i += blockDim.x) tw3[i] = g3[i];
  __syncthreads();
  const int g0 = pd.gptr[p], g1 = pd.gptr[p + 1];
  const C *src = psi + (size_t)band * ld_psi;
  for (int k = g0 + threadIdx.x; k < g1; k += blockDim.x) A[pd.sp_pos[k]] = cscale(src[pd.sp_g[k]], scale);
  __syncthreads();
  const int r0 = pd.rptr[p], nrow = pd.rptr[p + 1] - r0;
  zfft_rows_ip<P3, Q3, true>(A, pd.row_i2 + r0, nrow, p3, tw3);
  // y inverse: columns (lanes = tile column), pass 1 in place, pass 2 -> global slab plane
  const int ncg = (N3 + 31) >> 5;
  for (int it = w; it < ncg * Q2; it += nw) {
    const int grp = it / Q2, b = it - grp * Q2;
    const int col = grp * 32 + lane;
    if (col < N3) pass1_line<P2, Q2, true>(A, A, col, p3, b, tw2);
  }
  __syncthreads();
  C *dst = W + ((size_t)band * pd.np + p) * (size_t)(N2 * N3);
  for (int it = w; it < ncg * P2; it += nw) {
    const int grp = it / P2, k1 = it - grp * P2;
    const int col = grp * 32 + lane;
    if (col < N3) {
      const int i3 = dr_nat<P3, Q3>(col);
      C y[Q2];
#pragma unroll
      for (int b = 0; b < Q2; ++b) y[b] = A[(k1 * Q2 + b) * p3 + col];
      dft_reg<Q2, true>(y);
#pragma unroll
      for (int k2 = 0; k2 < Q2; ++k2) dst[(k1 + P2 * k2) * N3 + i3] = y[k2];
    }
  }
}

// ---------------------------------------------------------------------------
// P2: slab -> sphere.  y forward (columns) with the first pass reading the slab
// plane straight from global memory, z forward (rows), gather + kinetic.
// ---------------------------------------------------------------------------
template <typename R, int P2, int Q2, int P3, int Q3, int MODE>
__global__ void __launch_bounds__(512)
k_plane_fwd2(PlanDev pd, const typename Cx<R>::T *__restrict__ W, R scale, typename Cx<R>::T *__restrict__ out,
             long ld_out, const typename Cx<R>::T *__restrict__ psi_in, const R *__restrict__ kin, int nb_per_k,
             int batch0) {
  using C = typename Cx<R>::T;
  constexpr int N2 = P2 * Q2, N3 = P3 * Q3;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int p3 = odd_pitch(N3);
  const int SP = N2 * p3;
  C *A = reinterpret_cast<C *>(smem_raw);
  C *B = A + SP;
  C *tw2 = B + SP;
  C *tw3 = tw2 + N2;
  const int p = blockIdx.x, band = blockIdx.y;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const C *g2 = twiddles<R>(pd, 1), *g3 = twiddles<R>(pd, 2);
  for (int i = threadIdx.x; i < N2; i += blockDim.x) tw2[i] = g2[i];
  for (int i = threadIdx.x; i < N3; i += blockDim.x) tw3[i] = g3[i];
  __syncthreads();
  const C *srcw = W + ((size_t)band * pd.np + p) * (size_t)(N2 * N3);
  const int ncg = (N3 + 31) >> 5;
  // y forward pass 1 straight from the slab: x[b + Q2 a][col] -> B[k1 Q2 + b][col]
  for (int it = w; it < ncg * Q2; it += nw) {
    const int grp = it / Q2, b = it - grp * Q2;
    const int col = grp * 32 + lane;
    if (col < N3) {
      C v[P2];
#pragma unroll
      for (int a = 0; a < P2; ++a) v[a] = srcw[(b + Q2 * a) * N3 + col];
      dft_reg<P2, false>(v);
#pragma unroll
      for (int k1 = 0; k1 < P2; ++k1) B[(k1 * Q2 + b) * p3 + col] = cmul(v[k1], tw2[b * k1]);
    }
  }
  __syncthreads();
  for (int it = w; it < ncg * P2; it += nw) {
    const int grp = it / P2, k1 = it - grp * P2;
    const int col = grp * 32 + lane;
    if (col < N3) pass2_line<P2, Q2, false>(B, A, col, p3, k1);
  }
  __syncthreads();
  const int r0 = pd.rptr[p], nrow = pd.rptr[p + 1] - r0;
  zfft_rows<P3, Q3, false>(A, B, pd.row_i2 + r0, nrow, p3, tw3);
  const int g0 = pd.gptr[p], g1 = pd.gptr[p + 1];
  C *dst = out + (size_t)band * ld_out;
  if (MODE == PM_HPSI) {
    const int gb = batch0 + band;
    const R *kk = kin + (size_t)(gb / nb_per_k) * pd.nG;
    const C *pin = psi_in + (size_t)band * ld_out;
    for (int k = g0 + threadIdx.x; k < g1; k += blockDim.x) {
      const int g = pd.sp_g[k];
      dst[g] = cadd(cscale(A[pd.sp_pos[k]], scale), cscale(pin[g], kk[g]));
    }
  } else {
    for (int k = g0 + threadIdx.x; k < g1; k += blockDim.x) dst[pd.sp_g[k]] = cscale(A[pd.sp_pos[k]], scale);
  }
}

}  // namespace addft
