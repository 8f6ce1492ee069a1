// Column pipeline of the local part of H psi: (T + V(r)) psi for bands on a
// G-sphere, in three kernels that keep every intermediate in the smallest
// layout the sphere allows.
//
//   K1 k_colz_inv   one CTA per (group of 32 columns, band).  A column is an
//                   (i1, i2) pair that holds sphere points.  The CTA scatters
//                   the group's points into a zeroed n3 x 33 tile, runs the
//                   inverse z transform of the 32 columns (lanes = columns,
//                   two register passes, one shared-memory exchange) and
//                   writes the columns z-major to the column buffer
//                   W[band][z][column] (32 consecutive columns per store).
//   K2 k_plane_xy   one CTA per (z-plane, band).  Loads the plane's row of the
//                   column buffer (contiguous), scatters it into an n1 x n2
//                   tile, and in shared memory runs: y inverse on the active
//                   x-rows, x inverse on every y, V(r) in registers, x forward,
//                   y forward on the active x-rows; gathers the columns back.
//                   Two axes out, the potential and two axes back in one pass.
//   K3 k_colz_fwd   the forward z transform of K1's groups, then the gather
//                   onto the sphere fused with the kinetic term:
//                   hpsi[G] = FFT(...)[G] + kin[G] psi[G], with kin psi stored by
//                   K1 (which gathers psi anyway) in sorted-point order, so K3
//                   reads it coalesced and only its final store is scattered.
//
// Every line transform of length N = P Q is two register passes (DFT_P,
// twiddle, exchange, DFT_Q) and runs in place on its tile: pass 1 reads and
// writes one residue class mod Q, pass 2 one block of Q, which leaves the
// natural index k1 + P k2 at position k1 Q + k2 (digit-reversed).  The y axis
// stays digit-reversed between the inverse and the forward transform (the
// forward transform is decomposed the other way round and returns natural
// order); the x inverse's second pass, V(r) and the x forward's first pass
// share registers.  The potential is read as Vt[z][x][s] (s = digit-reversed
// y position), prepared once per call by k_vxy.
//
// Tiles use odd row pitches (n2 | 1 in K2, 33 per z-row of 32 columns in K1/K3),
// so every pass and the z-strided scatter are free of shared-memory bank conflicts.  Data volumes per
// band: column buffer n3 x ncols (72^3 microbench sphere: 1.9 MB FP32) against
// the plane slab np x n2 x n3 (2.7 MB) of the plane / x-line pipeline.
// Replaces ops/hpsi.py:29-32 (potential_apply) with the kinetic term of
// hpsi.py:18-26 fused into K3.
#pragma once
#include "plane2.cuh"

namespace addft {

template <int P, int Q>
__host__ __device__ constexpr int cmax() { return P > Q ? P : Q; }

// Sphere points handled per thread and round of the scatter / gather loops: all
// index loads of a round are issued before any data load, and all data loads
// before any store, so a thread keeps kGatherUnroll independent requests in flight.
constexpr int kGatherUnroll = 8;

// Zeroes n bytes of shared memory (16-byte aligned) with 16-byte stores.
__device__ __forceinline__ void smem_zero(void *p, int nbytes) {
  float4 *q = reinterpret_cast<float4 *>(p);
  const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int i = threadIdx.x; i < (nbytes >> 4); i += blockDim.x) q[i] = z;
  float *r = reinterpret_cast<float *>(p);
  for (int i = ((nbytes >> 4) << 2) + threadIdx.x; i < (nbytes >> 2); i += blockDim.x) r[i] = 0.f;
}

// ---------------------------------------------------------------------------
// The kinetic diagonal of every k point in sorted-point order, once per call: the
// factor is shared by all bands of a k point, so K1 reads it contiguously instead
// of gathering it per band.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void k_kinsort(PlanDev pd, const R *__restrict__ kin, int nk, R *__restrict__ kin_s) {
  const long total = (long)nk * pd.nG;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const int k = (int)(t / pd.nG), j = (int)(t - (long)k * pd.nG);
    kin_s[t] = kin[(size_t)k * pd.nG + pd.sp_g[j]];
  }
}

// ---------------------------------------------------------------------------
// K1: sphere -> columns (inverse z)
// ---------------------------------------------------------------------------
template <typename R, int P, int Q>
__global__ void __launch_bounds__(32 * cmax<P, Q>())
k_colz_inv(PlanDev pd, const typename Cx<R>::T *__restrict__ psi, long ld_psi, typename Cx<R>::T *__restrict__ W,
           const R *__restrict__ kin, int nb_per_k, int batch0, typename Cx<R>::T *__restrict__ KP) {
  using C = typename Cx<R>::T;
  constexpr int N = P * Q;
  constexpr int G = kColPitch;
  __shared__ __align__(16) C T[N * G];
  __shared__ C tw[N];
  const int j = blockIdx.x, band = blockIdx.y;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  smem_zero(T, (int)sizeof(T));
  const C *g3 = twiddles<R>(pd, 2);
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = g3[i];
  __syncthreads();
  const int k0 = pd.cgptr[j], k1e = pd.cgptr[j + 1];
  const C *src = psi + (size_t)band * ld_psi;
  const R *kk = kin + (size_t)((batch0 + band) / nb_per_k) * pd.nG;   // sorted-point order (k_kinsort)
  C *kp = KP + (size_t)band * pd.nG;
  for (int kb = k0 + threadIdx.x; kb < k1e; kb += kGatherUnroll * blockDim.x) {
    int gi[kGatherUnroll], pos[kGatherUnroll];
    C val[kGatherUnroll];
    R kv[kGatherUnroll];
#pragma unroll
    for (int u = 0; u < kGatherUnroll; ++u) {
      const int k = kb + u * blockDim.x;
      gi[u] = k < k1e ? pd.sp_g[k] : -1;
      pos[u] = k < k1e ? pd.pt_pos[k] : 0;
    }
#pragma unroll
    for (int u = 0; u < kGatherUnroll; ++u)
      if (gi[u] >= 0) {
        val[u] = src[gi[u]];
        kv[u] = kk[kb + u * blockDim.x];
      }
#pragma unroll
    for (int u = 0; u < kGatherUnroll; ++u)
      if (gi[u] >= 0) {
        T[pos[u]] = val[u];
        kp[kb + u * blockDim.x] = cscale(val[u], kv[u]);   // kinetic term, sorted-point order
      }
  }
  __syncthreads();
  if (w < Q) {   // pass 1 (residue class b = w), in place
    C v[P];
#pragma unroll
    for (int a = 0; a < P; ++a) v[a] = T[(w + Q * a) * G + lane];
    dft_reg<P, true>(v);
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) T[(k1 * Q + w) * G + lane] = cmulc(v[k1], tw[w * k1]);
  }
  __syncthreads();
  if (w < P) {   // pass 2 (block k1 = w) -> natural z = k1 + P k2, z-major store
    C y[Q];
#pragma unroll
    for (int b = 0; b < Q; ++b) y[b] = T[(w * Q + b) * G + lane];
    dft_reg<Q, true>(y);
    C *dst = W + (size_t)band * N * pd.ncols_pad + (size_t)j * kColGroup + lane;
#pragma unroll
    for (int k2 = 0; k2 < Q; ++k2) dst[(size_t)(w + P * k2) * pd.ncols_pad] = y[k2];
  }
}

// ---------------------------------------------------------------------------
// K3: columns -> sphere (forward z), gather + kinetic
// ---------------------------------------------------------------------------
template <typename R, int P, int Q>
__global__ void __launch_bounds__(32 * cmax<P, Q>())
k_colz_fwd(PlanDev pd, const typename Cx<R>::T *__restrict__ W, typename Cx<R>::T *__restrict__ out, long ld_out,
           const typename Cx<R>::T *__restrict__ KP) {
  using C = typename Cx<R>::T;
  constexpr int N = P * Q;
  constexpr int G = kColPitch;
  __shared__ __align__(16) C T[N * G];
  __shared__ C tw[N];
  const int j = blockIdx.x, band = blockIdx.y;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const C *g3 = twiddles<R>(pd, 2);
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = g3[i];
  __syncthreads();
  if (w < Q) {   // pass 1 (residue class b = w) straight from the z-major column buffer
    const C *srcw = W + (size_t)band * N * pd.ncols_pad + (size_t)j * kColGroup + lane;
    C v[P];
#pragma unroll
    for (int a = 0; a < P; ++a) v[a] = srcw[(size_t)(w + Q * a) * pd.ncols_pad];
    dft_reg<P, false>(v);
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) T[(k1 * Q + w) * G + lane] = cmul(v[k1], tw[w * k1]);
  }
  __syncthreads();
  C y[Q];
  if (w < P) {
#pragma unroll
    for (int b = 0; b < Q; ++b) y[b] = T[(w * Q + b) * G + lane];
    dft_reg<Q, false>(y);
  }
  __syncthreads();
  if (w < P) {
#pragma unroll
    for (int k2 = 0; k2 < Q; ++k2) T[(w + P * k2) * G + lane] = y[k2];
  }
  __syncthreads();
  const int k0 = pd.cgptr[j], k1e = pd.cgptr[j + 1];
  const C *kp = KP + (size_t)band * pd.nG;
  C *dst = out + (size_t)band * ld_out;
  for (int k = k0 + threadIdx.x; k < k1e; k += blockDim.x) dst[pd.sp_g[k]] = cadd(T[pd.pt_pos[k]], kp[k]);
}

// ---------------------------------------------------------------------------
// K2: one z-plane of the column buffer: y, x inverse; V; x, y forward
// ---------------------------------------------------------------------------
// threads per CTA the xy-plane kernel is compiled for (FP64 radix-15 lines need the registers of 512)
template <typename R>
__host__ __device__ constexpr int xy_max_threads() { return sizeof(R) == 8 ? 512 : kXYMaxThreads; }

// Column of the active x-plane with first column cb and runs (nlo, nhi) holding y, or -1.
template <int N2>
__device__ __forceinline__ int xy_col(int cb, int lohi, int y) {
  const int nlo = lohi & 0xffff, nhi = lohi >> 16;
  return y < nlo ? cb + y : (y >= N2 - nhi ? cb + nlo + y - (N2 - nhi) : -1);
}

// DIRECT: the y inverse's first pass loads the plane's columns straight from the
// column buffer and the y forward's second pass stores them straight back (lanes
// = residue classes of consecutive y, so both are coalesced runs of columns); only
// the inactive x-rows of the tile are zeroed.  Needs pd.xy_direct.  Otherwise the
// tile is zeroed, the columns scattered into it and gathered back from it.
template <typename R, int P1, int Q1, int P2, int Q2, bool DIRECT>
__global__ void __launch_bounds__(xy_max_threads<R>())
k_plane_xy(PlanDev pd, typename Cx<R>::T *__restrict__ W, const R *__restrict__ Vt) {
  using C = typename Cx<R>::T;
  constexpr int N1 = P1 * Q1, N2 = P2 * Q2, p2 = N2 | 1, SP = N1 * p2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C *A = reinterpret_cast<C *>(smem_raw);
  C *tw1 = A + SP;
  C *tw2 = tw1 + N1;
  int *rb = reinterpret_cast<int *>(tw2 + N2);   // tile offset of each active x-row
  const int z = blockIdx.x, band = blockIdx.y;
  const int nt = blockDim.x, tid = threadIdx.x;
  const int nr = pd.np, ncols = pd.nrows;
  const FastDiv dnr((unsigned)nr);
  const C zero = czero<C>();
  C *Wz = W + ((size_t)band * pd.n3 + z) * pd.ncols_pad;
  const C *g1 = twiddles<R>(pd, 0), *g2 = twiddles<R>(pd, 1);
  for (int i = tid; i < N1; i += nt) tw1[i] = g1[i];
  for (int i = tid; i < N2; i += nt) tw2[i] = g2[i];
  for (int i = tid; i < nr; i += nt) rb[i] = pd.plane_i1[i] * p2;
  if (DIRECT) {
    // zero the inactive x-rows only: a warp per row, lanes along the row
    const int lane = tid & 31, nw = nt >> 5;
    for (int x = tid >> 5; x < N1; x += nw)
      if (pd.plane_of_i1[x] < 0)
        for (int c = lane; c < p2; c += 32) A[x * p2 + c] = zero;
    __syncthreads();
    // y inverse pass 1 from the column buffer: lane (row r, residue class b), b fastest
    for (int i = tid; i < nr * Q2; i += nt) {
      const int r = i / Q2, b = i - r * Q2;
      const int cb = pd.rptr[r], lohi = pd.row_lohi[r];
      C v[P2];
#pragma unroll
      for (int a = 0; a < P2; ++a) {
        const int c = xy_col<N2>(cb, lohi, b + Q2 * a);
        v[a] = c >= 0 ? Wz[c] : zero;
      }
      dft_reg<P2, true>(v);
#pragma unroll
      for (int k1 = 0; k1 < P2; ++k1) A[rb[r] + k1 * Q2 + b] = cmulc(v[k1], tw2[b * k1]);
    }
  } else {
    smem_zero(A, SP * (int)sizeof(C));
    __syncthreads();
    for (int c = tid; c < ncols; c += nt) A[pd.col_xy[c]] = Wz[c];
    __syncthreads();
    // y inverse, active rows: pass 1 (residue classes)
    for (int i = tid; i < nr * Q2; i += nt) {
      const int b = dnr.div(i), r = i - b * nr;
      pass1_line<P2, Q2, true>(A, A, rb[r], 1, b, tw2);
    }
  }
  __syncthreads();
  // y inverse pass 2 (blocks, digit-reversed y)
  for (int i = tid; i < nr * P2; i += nt) {
    const int k1 = dnr.div(i), r = i - k1 * nr;
    pass2_line_ip<P2, Q2, true>(A, rb[r], 1, k1);
  }
  __syncthreads();
  // x inverse pass 1 on every y position s
  for (int i = tid; i < N2 * Q1; i += nt) {
    const int b = i / N2, s = i - b * N2;
    pass1_line<P1, Q1, true>(A, A, s, p2, b, tw1);
  }
  __syncthreads();
  // x inverse pass 2 -> natural x = k1 + P1 k2; times V; forward DFT over the same
  // stride-P1 subsequence (x = q + P1 p with q = k1); twiddle; back into block k1
  const R *Vz = Vt + (size_t)z * N1 * N2;
  for (int i = tid; i < N2 * P1; i += nt) {
    const int k1 = i / N2, s = i - k1 * N2;
    C y[Q1];
#pragma unroll
    for (int b = 0; b < Q1; ++b) y[b] = A[(k1 * Q1 + b) * p2 + s];
    dft_reg<Q1, true>(y);
#pragma unroll
    for (int k2 = 0; k2 < Q1; ++k2) y[k2] = cscale(y[k2], Vz[(k1 + P1 * k2) * N2 + s]);
    dft_reg<Q1, false>(y);
#pragma unroll
    for (int j1 = 0; j1 < Q1; ++j1) A[(k1 * Q1 + j1) * p2 + s] = cmul(y[j1], tw1[k1 * j1]);
  }
  __syncthreads();
  // x forward pass B (residue class j1): natural x-frequency j1 + Q1 j2 at position j2 Q1 + j1
  for (int i = tid; i < N2 * Q1; i += nt) {
    const int j1 = i / N2, s = i - j1 * N2;
    C v[P1];
#pragma unroll
    for (int q = 0; q < P1; ++q) v[q] = A[(q * Q1 + j1) * p2 + s];
    dft_reg<P1, false>(v);
#pragma unroll
    for (int j2 = 0; j2 < P1; ++j2) A[(j2 * Q1 + j1) * p2 + s] = v[j2];
  }
  __syncthreads();
  // y forward on the active rows: position q Q2 + p holds natural y = q + P2 p
  for (int i = tid; i < nr * P2; i += nt) {
    const int q = dnr.div(i), r = i - q * nr;
    C *row = A + rb[r] + q * Q2;
    C y[Q2];
#pragma unroll
    for (int p = 0; p < Q2; ++p) y[p] = row[p];
    dft_reg<Q2, false>(y);
#pragma unroll
    for (int j1 = 0; j1 < Q2; ++j1) row[j1] = cmul(y[j1], tw2[q * j1]);
  }
  __syncthreads();
  if (DIRECT) {   // y forward pass B straight into the column buffer: lane (row r, j1), j1 fastest
    for (int i = tid; i < nr * Q2; i += nt) {
      const int r = i / Q2, j1 = i - r * Q2;
      const C *row = A + rb[r] + j1;
      const int cb = pd.rptr[r], lohi = pd.row_lohi[r];
      C v[P2];
#pragma unroll
      for (int q = 0; q < P2; ++q) v[q] = row[q * Q2];
      dft_reg<P2, false>(v);
#pragma unroll
      for (int j2 = 0; j2 < P2; ++j2) {
        const int c = xy_col<N2>(cb, lohi, j1 + Q2 * j2);
        if (c >= 0) Wz[c] = v[j2];
      }
    }
    return;
  }
  for (int i = tid; i < nr * Q2; i += nt) {
    const int j1 = dnr.div(i), r = i - j1 * nr;
    C *row = A + rb[r] + j1;
    C v[P2];
#pragma unroll
    for (int q = 0; q < P2; ++q) v[q] = row[q * Q2];
    dft_reg<P2, false>(v);
#pragma unroll
    for (int j2 = 0; j2 < P2; ++j2) row[j2 * Q2] = v[j2];
  }
  __syncthreads();
  for (int c = tid; c < ncols; c += nt) Wz[c] = A[pd.col_xy[c]];
}

// Vt[z][x][s] = V[x][y(s)][z] * vscale with y(s) the natural y at digit-reversed
// position s = k1 Q2 + k2 (y = k1 + P2 k2).
template <typename R, int P2, int Q2>
__global__ void k_vxy(PlanDev pd, const R *__restrict__ V, R vscale, R *__restrict__ Vt) {
  constexpr int N2 = P2 * Q2;
  const long total = (long)pd.n1 * N2 * pd.n3;
  for (long f = blockIdx.x * (long)blockDim.x + threadIdx.x; f < total; f += (long)gridDim.x * blockDim.x) {
    const int s = (int)(f % N2);
    const long t = f / N2;
    const int x = (int)(t % pd.n1);
    const int zz = (int)(t / pd.n1);
    const int y = dr_nat<P2, Q2>(s);
    Vt[f] = V[((long)x * N2 + y) * pd.n3 + zz] * vscale;
  }
}

// Launches the column pipeline for nbatch bands if the box is instantiated;
// returns kPlane2NotHandled otherwise (the caller keeps the plane pipeline).
// W: nbatch column buffers (n3 x ncols_pad), KP: nbatch x nG (kin psi in sorted-point order);
// kin_s: the kinetic diagonal of every k point in sorted-point order (k_kinsort).
template <typename R>
addft_status launch_colfft_hpsi(const PlanDev &pd, int nbatch, const typename Cx<R>::T *psi, long ld,
                                const R *v_r, R vscale, R *Vt, bool make_vt, typename Cx<R>::T *W,
                                typename Cx<R>::T *KP, typename Cx<R>::T *out, const R *kin_s, int nb_per_k, int batch0,
                                cudaStream_t st);
template <typename R>
addft_status launch_kinsort(const PlanDev &pd, const R *kin, int nk, R *kin_s, cudaStream_t st) {
  const long total = (long)nk * pd.nG;
  const int blocks = (int)std::min<long>((total + 255) / 256, 4 * 152);
  k_kinsort<R><<<blocks, 256, 0, st>>>(pd, kin, nk, kin_s);
  return check_launch("k_kinsort");
}
// V(r) into the xy-plane kernel's layout Vt[z][x][digit-reversed y] (k_vxy) alone.
template <typename R>
addft_status launch_vxy_only(const PlanDev &pd, const R *v_r, R vscale, R *Vt, cudaStream_t st);
// True if launch_colfft_hpsi handles this plan's box.
template <typename R>
bool colfft_handles(const PlanDev &pd);

// colfused_f32.cu: the same pipeline as one persistent kernel (colfused.cuh), FP32, cubic boxes
// with direct column access.  ctr: device scratch of colfused_ctr_ints(nbatch) ints (zeroed by the
// launch).  Returns kPlane2NotHandled where not instantiated.
inline size_t colfused_ctr_ints(int nbatch) { return 1 + 2 * (size_t)nbatch; }
bool colfused_handles(const PlanDev &pd);
addft_status launch_colfused_hpsi(const PlanDev &pd, int nbatch, const float2 *psi, long ld, float2 *W, float2 *KP,
                                  const float *Vt, float2 *out, const float *kin_s, int nb_per_k, int batch0,
                                  int *ctr, cudaStream_t st);

}  // namespace addft
