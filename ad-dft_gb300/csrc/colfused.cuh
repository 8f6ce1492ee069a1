// The column pipeline of the local H psi as one persistent kernel.
//
// The three kernels of colfft.cuh (K1 sphere -> columns + inverse z, K2 one
// xy-plane with V(r), K3 forward z + gather + kinetic) run as work items of
// one launch.  CTAs take tickets from a counter in order; ticket t is item r
// of step s = t / S, S = 2 ng + nz (ng column groups, nz z-planes), with a lag
// of L steps between the stages of one band:
//   r <  ng            K1 item r of band s
//   r <  ng + nz       K2 item r - ng (z-plane) of band s - L
//   otherwise          K3 item r - ng - nz of band s - 2 L
// A K2 item of band b waits until the ng K1 items of band b are done, a K3
// item until the nz K2 items are.  The interleaving means that by the time a
// CTA holds a dependent ticket, the tickets it depends on were handed out L
// whole steps earlier; only CTAs that hold tickets are waited on, so the
// schedule cannot deadlock whatever the number of resident CTAs.
//
// What this aims at: only the bands in flight (2 L + 1) touch the column
// buffer and the kin psi side buffer, so those stay in L2 (instead of crossing
// HBM four and two times), and the latency-bound sphere gather / scatter of K1
// and K3 shares the SMs with the issue-bound plane transforms of K2.  Measured
// on the 72^3 microbench (64 bands, FP32 H psi): 0.420 ms at L = 8 (0.61 /
// 0.44 / 0.43 ms at L = 1 / 4 / 16) against 0.400 ms for the three kernels, so
// it is not the default (tuning "colfft" = 2 selects it).  288 threads per CTA
// (nine warps: the radix-9 passes of the z items get a warp per block) at four
// CTAs per SM.
//
// Memory ordering: a finished item's threads fence, the CTA synchronises and
// one thread increments the band's counter; a waiting CTA spins on the
// counter (volatile loads, bounded), fences and synchronises.  Column-buffer
// and kin psi loads written by other CTAs bypass L1 (ld.global.cg).  Every
// wait has an iteration limit: on expiry (or once another CTA has flagged
// one) it records bit 0 of addft_hpsi_fused_status and goes on, so a fault
// in the schedule gives wrong numbers and a status bit, never a hang.
#pragma once
#include "colfft.cuh"

namespace addft {

constexpr int kFusedThreads = 288;
constexpr int kFusedWaitLimit = 1 << 20;
// sphere points per thread and round of the K1 gather (the three kernels use 8; fewer here keep
// the persistent kernel's registers at the xy-plane transform's level)
constexpr int kFusedUnroll = 4;

// bit 0: a dependency wait of the fused kernel ran out (read by addft_hpsi_fused_status)
static __device__ unsigned g_fused_error = 0;

__device__ __forceinline__ unsigned *fused_error_word() { return &g_fused_error; }

template <typename C>
__device__ __forceinline__ C ldcg(const C *p) { return __ldcg(p); }

// Spins until *cnt >= target (thread 0), then makes the producers' writes visible to the CTA.
__device__ __forceinline__ void fused_wait(const int *cnt, int target) {
  if (threadIdx.x == 0) {
    volatile unsigned *err = fused_error_word();
    bool ok = false;
    for (int it = 0; it < kFusedWaitLimit; ++it) {
      if (*(volatile const int *)cnt >= target) {
        ok = true;
        break;
      }
      if (*err) break;
      __nanosleep(64);
    }
    if (!ok) atomicOr((unsigned *)err, 1u);
    __threadfence();
  }
  __syncthreads();
}

// Publishes this CTA's writes of the finished item and counts it.
__device__ __forceinline__ void fused_signal(int *cnt) {
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) atomicAdd(cnt, 1);
}

// K1 item: column group j of one band (as k_colz_inv, any number of warps).
template <typename R, int P, int Q>
__device__ __forceinline__ void fz_inv(const PlanDev &pd, int j, int band, const typename Cx<R>::T *__restrict__ psi,
                                       long ld_psi, typename Cx<R>::T *__restrict__ W, const R *__restrict__ kin,
                                       int nb_per_k, int batch0, typename Cx<R>::T *__restrict__ KP,
                                       typename Cx<R>::T *T, const typename Cx<R>::T *tw) {
  using C = typename Cx<R>::T;
  constexpr int N = P * Q, G = kColPitch;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  smem_zero(T, N * G * (int)sizeof(C));
  __syncthreads();
  const int k0 = pd.cgptr[j], k1e = pd.cgptr[j + 1];
  const C *src = psi + (size_t)band * ld_psi;
  const R *kk = kin + (size_t)((batch0 + band) / nb_per_k) * pd.nG;
  C *kp = KP + (size_t)band * pd.nG;
  for (int kb = k0 + threadIdx.x; kb < k1e; kb += kFusedUnroll * blockDim.x) {
    int gi[kFusedUnroll], pos[kFusedUnroll];
    C val[kFusedUnroll];
    R kv[kFusedUnroll];
#pragma unroll
    for (int u = 0; u < kFusedUnroll; ++u) {
      const int k = kb + u * blockDim.x;
      gi[u] = k < k1e ? pd.sp_g[k] : -1;
      pos[u] = k < k1e ? pd.pt_pos[k] : 0;
    }
#pragma unroll
    for (int u = 0; u < kFusedUnroll; ++u)
      if (gi[u] >= 0) {
        val[u] = src[gi[u]];
        kv[u] = kk[kb + u * blockDim.x];
      }
#pragma unroll
    for (int u = 0; u < kFusedUnroll; ++u)
      if (gi[u] >= 0) {
        T[pos[u]] = val[u];
        kp[kb + u * blockDim.x] = cscale(val[u], kv[u]);
      }
  }
  __syncthreads();
  for (int b = w; b < Q; b += nw) {   // pass 1, residue class b, in place
    C v[P];
#pragma unroll
    for (int a = 0; a < P; ++a) v[a] = T[(b + Q * a) * G + lane];
    dft_reg<P, true>(v);
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) T[(k1 * Q + b) * G + lane] = cmulc(v[k1], tw[b * k1]);
  }
  __syncthreads();
  C *dst = W + (size_t)band * N * pd.ncols_pad + (size_t)j * kColGroup + lane;
  for (int k1 = w; k1 < P; k1 += nw) {   // pass 2, block k1 -> natural z, z-major store
    C y[Q];
#pragma unroll
    for (int b = 0; b < Q; ++b) y[b] = T[(k1 * Q + b) * G + lane];
    dft_reg<Q, true>(y);
#pragma unroll
    for (int k2 = 0; k2 < Q; ++k2) dst[(size_t)(k1 + P * k2) * pd.ncols_pad] = y[k2];
  }
}

// K3 item: column group j of one band (as k_colz_fwd; pass 2 out of place into T2).
template <typename R, int P, int Q>
__device__ __forceinline__ void fz_fwd(const PlanDev &pd, int j, int band, const typename Cx<R>::T *W,
                                       typename Cx<R>::T *__restrict__ out, long ld_out,
                                       const typename Cx<R>::T *KP, typename Cx<R>::T *T, typename Cx<R>::T *T2,
                                       const typename Cx<R>::T *tw) {
  using C = typename Cx<R>::T;
  constexpr int N = P * Q, G = kColPitch;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const C *srcw = W + (size_t)band * N * pd.ncols_pad + (size_t)j * kColGroup + lane;
  for (int b = w; b < Q; b += nw) {   // pass 1 straight from the column buffer
    C v[P];
#pragma unroll
    for (int a = 0; a < P; ++a) v[a] = ldcg(srcw + (size_t)(b + Q * a) * pd.ncols_pad);
    dft_reg<P, false>(v);
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) T[(k1 * Q + b) * G + lane] = cmul(v[k1], tw[b * k1]);
  }
  __syncthreads();
  for (int k1 = w; k1 < P; k1 += nw) {
    C y[Q];
#pragma unroll
    for (int b = 0; b < Q; ++b) y[b] = T[(k1 * Q + b) * G + lane];
    dft_reg<Q, false>(y);
#pragma unroll
    for (int k2 = 0; k2 < Q; ++k2) T2[(k1 + P * k2) * G + lane] = y[k2];
  }
  __syncthreads();
  const int k0 = pd.cgptr[j], k1e = pd.cgptr[j + 1];
  const C *kp = KP + (size_t)band * pd.nG;
  C *dst = out + (size_t)band * ld_out;
  for (int k = k0 + threadIdx.x; k < k1e; k += blockDim.x) dst[pd.sp_g[k]] = cadd(T2[pd.pt_pos[k]], ldcg(kp + k));
}

// K2 item: z-plane z of one band (as k_plane_xy with the direct column loads / stores).
template <typename R, int P1, int Q1>
__device__ __forceinline__ void fxy(const PlanDev &pd, int z, int band, typename Cx<R>::T *__restrict__ W,
                                    const R *__restrict__ Vt, typename Cx<R>::T *A, const typename Cx<R>::T *tw1,
                                    const int *rb) {
  using C = typename Cx<R>::T;
  constexpr int P2 = P1, Q2 = Q1;
  constexpr int N1 = P1 * Q1, N2 = P2 * Q2, p2 = N2 | 1;
  const C *tw2 = tw1;
  const int nt = blockDim.x, tid = threadIdx.x;
  const int nr = pd.np;
  const FastDiv dnr((unsigned)nr);
  const C zero = czero<C>();
  C *Wz = W + ((size_t)band * pd.n3 + z) * pd.ncols_pad;
  {
    const int lane = tid & 31, nw = nt >> 5;
    for (int x = tid >> 5; x < N1; x += nw)
      if (pd.plane_of_i1[x] < 0)
        for (int c = lane; c < p2; c += 32) A[x * p2 + c] = zero;
  }
  __syncthreads();
  for (int i = tid; i < nr * Q2; i += nt) {   // y inverse pass 1 from the column buffer
    const int r = i / Q2, b = i - r * Q2;
    const int cb = pd.rptr[r], lohi = pd.row_lohi[r];
    C v[P2];
#pragma unroll
    for (int a = 0; a < P2; ++a) {
      const int c = xy_col<N2>(cb, lohi, b + Q2 * a);
      v[a] = c >= 0 ? ldcg(Wz + c) : zero;
    }
    dft_reg<P2, true>(v);
#pragma unroll
    for (int k1 = 0; k1 < P2; ++k1) A[rb[r] + k1 * Q2 + b] = cmulc(v[k1], tw2[b * k1]);
  }
  __syncthreads();
  for (int i = tid; i < nr * P2; i += nt) {   // y inverse pass 2
    const int k1 = dnr.div(i), r = i - k1 * nr;
    pass2_line_ip<P2, Q2, true>(A, rb[r], 1, k1);
  }
  __syncthreads();
  for (int i = tid; i < N2 * Q1; i += nt) {   // x inverse pass 1
    const int b = i / N2, s = i - b * N2;
    pass1_line<P1, Q1, true>(A, A, s, p2, b, tw1);
  }
  __syncthreads();
  const R *Vz = Vt + (size_t)z * N1 * N2;
  for (int i = tid; i < N2 * P1; i += nt) {   // x inverse pass 2, V, x forward pass A
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
  for (int i = tid; i < N2 * Q1; i += nt) {   // x forward pass B
    const int j1 = i / N2, s = i - j1 * N2;
    C v[P1];
#pragma unroll
    for (int q = 0; q < P1; ++q) v[q] = A[(q * Q1 + j1) * p2 + s];
    dft_reg<P1, false>(v);
#pragma unroll
    for (int j2 = 0; j2 < P1; ++j2) A[(j2 * Q1 + j1) * p2 + s] = v[j2];
  }
  __syncthreads();
  for (int i = tid; i < nr * P2; i += nt) {   // y forward pass A on the active rows
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
  for (int i = tid; i < nr * Q2; i += nt) {   // y forward pass B straight into the column buffer
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
}

// Shared-memory bytes of the fused kernel for a cubic box n = P Q with np active x-planes.
template <typename R, int P, int Q>
__host__ __device__ constexpr size_t fused_smem_fixed() {
  using C = typename Cx<R>::T;
  constexpr int N = P * Q;
  constexpr size_t area = (size_t)N * (N | 1) > (size_t)2 * N * kColPitch ? (size_t)N * (N | 1)
                                                                           : (size_t)2 * N * kColPitch;
  return sizeof(C) * (2 * (size_t)N + area);
}

// The persistent kernel: one launch = the whole column pipeline for nbatch bands of a cubic box.
// ctr: [0] ticket, [1 + b] K1 items done of band b, [1 + nbatch + b] K2 items done of band b.
template <typename R, int P, int Q>
__global__ void __launch_bounds__(kFusedThreads, 4)
k_hpsi_colfused(PlanDev pd, int nbatch, const typename Cx<R>::T *__restrict__ psi, long ld,
                typename Cx<R>::T *__restrict__ W, typename Cx<R>::T *__restrict__ KP, const R *__restrict__ Vt,
                typename Cx<R>::T *__restrict__ out, const R *__restrict__ kin, int nb_per_k, int batch0,
                int lag, int *__restrict__ ctr) {
  using C = typename Cx<R>::T;
  constexpr int N = P * Q;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_ticket;
  C *tw_xy = reinterpret_cast<C *>(smem_raw);   // x and y twiddles (square plane)
  C *tw_z = tw_xy + N;
  C *area = tw_z + N;
  int *rb = reinterpret_cast<int *>(area + (fused_smem_fixed<R, P, Q>() / sizeof(C) - 2 * N));
  const int tid = threadIdx.x;
  {
    const C *g1 = twiddles<R>(pd, 0), *g3 = twiddles<R>(pd, 2);
    for (int i = tid; i < N; i += blockDim.x) {
      tw_xy[i] = g1[i];
      tw_z[i] = g3[i];
    }
    for (int i = tid; i < pd.np; i += blockDim.x) rb[i] = pd.plane_i1[i] * (N | 1);
  }
  const int ng = pd.ncols_pad / kColGroup, nz = pd.n3;
  const int step = 2 * ng + nz;
  const int total = (nbatch + 2 * lag) * step;
  int *done1 = ctr + 1, *done2 = ctr + 1 + nbatch;
  for (;;) {
    __syncthreads();   // the previous item is finished with shared memory
    if (tid == 0) s_ticket = atomicAdd(ctr, 1);
    __syncthreads();
    const int t = s_ticket;
    if (t >= total) break;
    const int s = t / step, r = t - s * step;
    if (r < ng) {
      const int band = s;
      if (band >= nbatch) continue;
      fz_inv<R, P, Q>(pd, r, band, psi, ld, W, kin, nb_per_k, batch0, KP, area, tw_z);
      fused_signal(done1 + band);
    } else if (r < ng + nz) {
      const int band = s - lag;
      if (band < 0 || band >= nbatch) continue;
      fused_wait(done1 + band, ng);
      fxy<R, P, Q>(pd, r - ng, band, W, Vt, area, tw_xy, rb);
      fused_signal(done2 + band);
    } else {
      const int band = s - 2 * lag;
      if (band < 0 || band >= nbatch) continue;
      fused_wait(done2 + band, nz);
      fz_fwd<R, P, Q>(pd, r - ng - nz, band, W, out, ld, KP, area, area + N * kColPitch, tw_z);
    }
  }
}

}  // namespace addft
