// Sphere-aware 3D FFT pipeline for plane-wave coefficients (GB300, sm_103a).
//
// A band lives on a G-sphere of nG points inside an n1 x n2 x n3 box.  The
// inverse transform (G -> r) runs in three kernels:
//   P1  (k_plane_inv)  one CTA per (active x-plane p, band b): scatter the
//        plane's sphere points into a zeroed n2 x n3 tile in shared memory,
//        FFT along z on the active rows only, FFT along y on every column,
//        store the tile to the slab buffer W[b][p] (coalesced);
//   X   (k_xline)      one CTA per (y-row i2, z-tile, band): gather the
//        active planes' rows, FFT along x.  Depending on the mode the CTA then
//        multiplies by V(r) and transforms back (H psi), writes psi(r), or
//        accumulates sum_b w_b |psi_b(r)|^2 (density);
//   P2  (k_plane_fwd)  the forward mirror of P1 ending in the gather onto the
//        sphere, fused with the kinetic term for H psi.
// Boxes whose yz-plane tiles do not fit a CTA's shared memory run P1 / P2 as two
// kernels each (z on groups of 32 sphere columns, y on tiles of one plane) through
// the same slab.  Only planes and rows that carry sphere points are transformed in the
// sparse directions, and the intermediate slabs stay L2-resident for the
// band chunk in flight.  Replaces psi_to_real / real_to_psi / potential_apply
// (src/addft/geometry/basis.py:205-254, src/addft/ops/hpsi.py:29-32) and the
// scatter/gather kernels of native/pack.cu:16-38.
#include <stdlib.h>

#include "colfft.cuh"
#include "transforms.cuh"

namespace addft {
// ---------------------------------------------------------------------------
// P1: sphere -> slab (z and y inverse transforms)
// Shared tiles use an odd row pitch p3 = n3 | 1 (bank-conflict-free lines).
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(kFftMaxThreads)
k_plane_inv(PlanDev pd, const typename Cx<R>::T *__restrict__ psi, long ld_psi, R scale,
            typename Cx<R>::T *__restrict__ W) {
  using C = typename Cx<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int S = pd.n2 * pd.n3;
  const int p3 = odd_pitch(pd.n3);
  const int SP = pd.n2 * p3;
  C *A = reinterpret_cast<C *>(smem_raw);
  C *B = A + SP;
  C *tw2 = B + SP;
  C *tw3 = tw2 + pd.n2;
  const int p = blockIdx.x;
  const int b = blockIdx.y;
  const C z = czero<C>();
  for (int i = threadIdx.x; i < SP; i += blockDim.x) { A[i] = z; B[i] = z; }
  const C *g2 = twiddles<R>(pd, 1), *g3 = twiddles<R>(pd, 2);
  for (int i = threadIdx.x; i < pd.n2; i += blockDim.x) tw2[i] = g2[i];
  for (int i = threadIdx.x; i < pd.n3; i += blockDim.x) tw3[i] = g3[i];
  __syncthreads();
  const int g0 = pd.gptr[p], g1 = pd.gptr[p + 1];
  const C *src = psi + (size_t)b * ld_psi;
  for (int k = g0 + threadIdx.x; k < g1; k += blockDim.x)
    A[pd.sp_pos[k]] = cscale(src[pd.sp_g[k]], scale);
  __syncthreads();
  const int r0 = pd.rptr[p], nrow = pd.rptr[p + 1] - r0;
  C *cur = fft_lines<true>(A, B, pd.ax[2], tw3, nrow, pd.row_i2 + r0, p3, 1);
  C *oth = cur == A ? B : A;
  C *res = fft_lines<true>(cur, oth, pd.ax[1], tw2, pd.n3, nullptr, 1, p3);
  C *dst = W + ((size_t)b * pd.np + p) * S;
  const int lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
  for (int y = threadIdx.x >> 5; y < pd.n2; y += nwarp)
    for (int x = lane; x < pd.n3; x += 32) dst[y * pd.n3 + x] = res[y * p3 + x];
}

// ---------------------------------------------------------------------------
// P2: slab -> sphere (y and z forward transforms, gather, kinetic)
// ---------------------------------------------------------------------------
template <typename R, int MODE>
__global__ void __launch_bounds__(kFftMaxThreads)
k_plane_fwd(PlanDev pd, const typename Cx<R>::T *__restrict__ W, R scale,
            typename Cx<R>::T *__restrict__ out, long ld_out,
            const typename Cx<R>::T *__restrict__ psi_in, const R *__restrict__ kin, int nb_per_k,
            int batch0) {
  using C = typename Cx<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int S = pd.n2 * pd.n3;
  const int p3 = odd_pitch(pd.n3);
  const int SP = pd.n2 * p3;
  C *A = reinterpret_cast<C *>(smem_raw);
  C *B = A + SP;
  C *tw2 = B + SP;
  C *tw3 = tw2 + pd.n2;
  const int p = blockIdx.x;
  const int b = blockIdx.y;
  const C *srcw = W + ((size_t)b * pd.np + p) * S;
  {
    const int lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
    for (int y = threadIdx.x >> 5; y < pd.n2; y += nwarp)
      for (int x = lane; x < pd.n3; x += 32) A[y * p3 + x] = srcw[y * pd.n3 + x];
  }
  const C *g2 = twiddles<R>(pd, 1), *g3 = twiddles<R>(pd, 2);
  for (int i = threadIdx.x; i < pd.n2; i += blockDim.x) tw2[i] = g2[i];
  for (int i = threadIdx.x; i < pd.n3; i += blockDim.x) tw3[i] = g3[i];
  __syncthreads();
  C *cur = fft_lines<false>(A, B, pd.ax[1], tw2, pd.n3, nullptr, 1, p3);
  C *oth = cur == A ? B : A;
  const int r0 = pd.rptr[p], nrow = pd.rptr[p + 1] - r0;
  C *res = fft_lines<false>(cur, oth, pd.ax[2], tw3, nrow, pd.row_i2 + r0, p3, 1);
  const int g0 = pd.gptr[p], g1 = pd.gptr[p + 1];
  C *dst = out + (size_t)b * ld_out;
  if (MODE == PM_HPSI) {
    const int gb = batch0 + b;
    const R *kk = kin + (size_t)(gb / nb_per_k) * pd.nG;
    const C *pin = psi_in + (size_t)b * ld_out;
    for (int k = g0 + threadIdx.x; k < g1; k += blockDim.x) {
      const int g = pd.sp_g[k];
      const C v = cscale(res[pd.sp_pos[k]], scale);
      const C x = pin[g];
      const R t = kk[g];
      dst[g] = cadd(v, cscale(x, t));
    }
  } else {
    for (int k = g0 + threadIdx.x; k < g1; k += blockDim.x)
      dst[pd.sp_g[k]] = cscale(res[pd.sp_pos[k]], scale);
  }
}

// ---------------------------------------------------------------------------
// Split P1 / P2 for yz-planes whose two n2 x (n3 | 1) tiles exceed a CTA's shared
// memory (n2 n3 above ~7,200 in FP64, ~14,400 in FP32): the z transform runs on
// groups of 32 columns (the (i1, i2) rows of the sphere, in the plan's column
// tables: tile n3 x 33, as the column pipeline's K1 / K3) and the y transform on
// tiles of T z-positions of one x-plane.  Both read and write the same band slab
// W[b][p][i2][i3] as P1 / P2, so the x-line stage between them is unchanged.
// ---------------------------------------------------------------------------
// Z1: sphere -> inverse z on 32 columns -> the columns' slab rows (active rows only)
template <typename R>
__global__ void __launch_bounds__(kFftMaxThreads)
k_zcols_inv(PlanDev pd, const typename Cx<R>::T *__restrict__ psi, long ld_psi, R scale,
            typename Cx<R>::T *__restrict__ W) {
  using C = typename Cx<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n3 = pd.n3, SP = n3 * kColPitch;
  C *A = reinterpret_cast<C *>(smem_raw);
  C *B = A + SP;
  C *tw3 = B + SP;
  const int j = blockIdx.x, b = blockIdx.y;
  const C zero = czero<C>();
  for (int i = threadIdx.x; i < SP; i += blockDim.x) A[i] = zero;
  const C *g3 = twiddles<R>(pd, 2);
  for (int i = threadIdx.x; i < n3; i += blockDim.x) tw3[i] = g3[i];
  __syncthreads();
  const C *src = psi + (size_t)b * ld_psi;
  const int k1e = pd.cgptr[j + 1];
  for (int k = pd.cgptr[j] + threadIdx.x; k < k1e; k += blockDim.x) A[pd.pt_pos[k]] = cscale(src[pd.sp_g[k]], scale);
  __syncthreads();
  const C *res = fft_lines<true>(A, B, pd.ax[2], tw3, kColGroup, nullptr, 1, kColPitch);
  const int lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
  const int p2 = pd.n2 | 1;
  const size_t S = (size_t)pd.n2 * n3;
  for (int t = threadIdx.x >> 5; t < kColGroup; t += nwarp) {   // a warp per column, lanes along z
    const int c = j * kColGroup + t;
    if (c >= pd.nrows) break;
    const int xy = pd.col_xy[c];
    const int i1 = xy / p2, i2 = xy - i1 * p2;
    C *dst = W + ((size_t)b * pd.np + pd.plane_of_i1[i1]) * S + (size_t)i2 * n3;
    for (int zz = lane; zz < n3; zz += 32) dst[zz] = res[zz * kColPitch + t];
  }
}

// Y: y transform of x-plane p on the z-positions z0 .. z0 + T - 1.  Inverse: loads the
// plane's active rows (the rest of the tile is zero) and stores every row; forward:
// loads every row and stores the active rows (the only ones Z2 reads).
template <typename R, bool INV>
__global__ void __launch_bounds__(kFftMaxThreads)
k_ytile(PlanDev pd, typename Cx<R>::T *__restrict__ W, int T, int ntile) {
  using C = typename Cx<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n2 = pd.n2, n3 = pd.n3, pT = odd_pitch(T), SP = n2 * pT;
  C *A = reinterpret_cast<C *>(smem_raw);
  C *B = A + SP;
  C *tw2 = B + SP;
  const int p = blockIdx.x / ntile;
  const int z0 = (blockIdx.x - p * ntile) * T;
  const int tv = min(T, n3 - z0);   // valid z-positions of this tile
  const int b = blockIdx.y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const C zero = czero<C>();
  const C *g2 = twiddles<R>(pd, 1);
  for (int i = threadIdx.x; i < n2; i += blockDim.x) tw2[i] = g2[i];
  C *Wp = W + ((size_t)b * pd.np + p) * (size_t)n2 * n3 + z0;
  const int r0 = pd.rptr[p], r1 = pd.rptr[p + 1];
  if (INV) {
    for (int i = threadIdx.x; i < SP; i += blockDim.x) A[i] = zero;
    __syncthreads();
    for (int r = r0 + warp; r < r1; r += nwarp) {
      const int y = pd.row_i2[r];
      for (int t = lane; t < tv; t += 32) A[y * pT + t] = Wp[(size_t)y * n3 + t];
    }
  } else {
    for (int y = warp; y < n2; y += nwarp)
      for (int t = lane; t < T; t += 32) A[y * pT + t] = t < tv ? Wp[(size_t)y * n3 + t] : zero;
  }
  __syncthreads();
  const C *res = fft_lines<INV>(A, B, pd.ax[1], tw2, T, nullptr, 1, pT);
  if (INV) {
    for (int y = warp; y < n2; y += nwarp)
      for (int t = lane; t < tv; t += 32) Wp[(size_t)y * n3 + t] = res[y * pT + t];
  } else {
    for (int r = r0 + warp; r < r1; r += nwarp) {
      const int y = pd.row_i2[r];
      for (int t = lane; t < tv; t += 32) Wp[(size_t)y * n3 + t] = res[y * pT + t];
    }
  }
}

// Z2: the columns' slab rows -> forward z on 32 columns -> gather onto the sphere
// (PM_HPSI: plus kin[G] psi[G], as P2)
template <typename R, int MODE>
__global__ void __launch_bounds__(kFftMaxThreads)
k_zcols_fwd(PlanDev pd, const typename Cx<R>::T *__restrict__ W, R scale, typename Cx<R>::T *__restrict__ out,
            long ld_out, const typename Cx<R>::T *__restrict__ psi_in, const R *__restrict__ kin, int nb_per_k,
            int batch0) {
  using C = typename Cx<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n3 = pd.n3, SP = n3 * kColPitch;
  C *A = reinterpret_cast<C *>(smem_raw);
  C *B = A + SP;
  C *tw3 = B + SP;
  const int j = blockIdx.x, b = blockIdx.y;
  const C zero = czero<C>();
  const int lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
  const int p2 = pd.n2 | 1;
  const size_t S = (size_t)pd.n2 * n3;
  const C *g3 = twiddles<R>(pd, 2);
  for (int i = threadIdx.x; i < n3; i += blockDim.x) tw3[i] = g3[i];
  for (int t = threadIdx.x >> 5; t < kColGroup; t += nwarp) {   // a warp per column, lanes along z
    const int c = j * kColGroup + t;
    if (c < pd.nrows) {
      const int xy = pd.col_xy[c];
      const int i1 = xy / p2, i2 = xy - i1 * p2;
      const C *srcw = W + ((size_t)b * pd.np + pd.plane_of_i1[i1]) * S + (size_t)i2 * n3;
      for (int zz = lane; zz < n3; zz += 32) A[zz * kColPitch + t] = srcw[zz];
    } else {
      for (int zz = lane; zz < n3; zz += 32) A[zz * kColPitch + t] = zero;
    }
  }
  __syncthreads();
  const C *res = fft_lines<false>(A, B, pd.ax[2], tw3, kColGroup, nullptr, 1, kColPitch);
  C *dst = out + (size_t)b * ld_out;
  const int k0 = pd.cgptr[j], k1e = pd.cgptr[j + 1];
  if (MODE == PM_HPSI) {
    const R *kk = kin + (size_t)((batch0 + b) / nb_per_k) * pd.nG;
    const C *pin = psi_in + (size_t)b * ld_out;
    for (int k = k0 + threadIdx.x; k < k1e; k += blockDim.x) {
      const int g = pd.sp_g[k];
      dst[g] = cadd(cscale(res[pd.pt_pos[k]], scale), cscale(pin[g], kk[g]));
    }
  } else {
    for (int k = k0 + threadIdx.x; k < k1e; k += blockDim.x) dst[pd.sp_g[k]] = cscale(res[pd.pt_pos[k]], scale);
  }
}

// ---------------------------------------------------------------------------
// X: x-line transforms over a (i2, i3-tile) column block; tile pitch pT = T | 1
// ---------------------------------------------------------------------------
// V(r) multiply fused into the last inverse stage: line = tile column t, pos = x (i1)
template <typename R>
struct VMulEpi {
  const R *v;      // V at (x, i2, c0 + t): v[x * n2n3 + t]
  int n2n3;
  int tw;          // valid columns
  R scale;
  template <typename C>
  __device__ __forceinline__ C operator()(C val, int line, int pos) const {
    const R s = line < tw ? v[pos * n2n3 + line] * scale : (R)0;
    return cscale(val, s);
  }
};

template <typename R, int MODE>
__global__ void __launch_bounds__(kFftMaxThreads)
k_xline(PlanDev pd, XArgs<R> a) {
  using C = typename Cx<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n1 = pd.n1, n2 = pd.n2, n3 = pd.n3;
  const int T = a.t3;
  const int S = n1 * T;
  const int pT = odd_pitch(T);
  const int SP = n1 * pT;
  C *A = reinterpret_cast<C *>(smem_raw);
  C *B = A + SP;
  C *tw1 = B + SP;
  const int i2 = blockIdx.x / a.ntile3;
  const int c0 = (blockIdx.x - i2 * a.ntile3) * T;
  const int tw_ = min(T, n3 - c0);   // valid columns in this tile
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int n2n3 = n2 * n3;
  const C *g1 = twiddles<R>(pd, 0);
  for (int i = threadIdx.x; i < n1; i += blockDim.x) tw1[i] = g1[i];
  const C z = czero<C>();

  // one warp per x-row: row x of the tile <- slab row (plane(x), i2, c0 .. c0 + tw_)
  auto load_slab = [&](int bb) {
    const C *Wb = a.W + (size_t)bb * pd.np * n2n3 + i2 * n3 + c0;
    for (int x = warp; x < n1; x += nwarp) {
      const int p = pd.plane_of_i1[x];
      C *row = A + x * pT;
      if (p >= 0) {
        const C *src = Wb + p * n2n3;
        for (int t = lane; t < T; t += 32) row[t] = t < tw_ ? src[t] : z;
      } else {
        for (int t = lane; t < T; t += 32) row[t] = z;
      }
    }
  };

  if (MODE == XM_DENSITY) {
    // bands [bb0, bb1) of this chunk; |psi|^2 accumulated in shared memory (f64)
    double *acc = reinterpret_cast<double *>(tw1 + n1);
    for (int i = threadIdx.x; i < S; i += blockDim.x) acc[i] = 0.0;
    const int per = (a.nbatch + a.nsplit - 1) / a.nsplit;
    const int bb0 = blockIdx.y * per, bb1 = min(a.nbatch, bb0 + per);
    for (int bb = bb0; bb < bb1; ++bb) {
      load_slab(bb);
      __syncthreads();
      C *res = fft_lines<true>(A, B, pd.ax[0], tw1, T, nullptr, 1, pT);
      const double wb = a.wocc[bb] * a.dscale;
      for (int x = warp; x < n1; x += nwarp)
        for (int t = lane; t < T; t += 32) {
          const C v = res[x * pT + t];
          acc[x * T + t] += wb * ((double)v.x * (double)v.x + (double)v.y * (double)v.y);
        }
      __syncthreads();
    }
    double *dst = (a.nsplit > 1 ? a.part + (size_t)blockIdx.y * a.N : a.rho) + i2 * n3 + c0;
    const int acc_mode = a.nsplit > 1 ? 0 : a.rho_acc;
    for (int x = warp; x < n1; x += nwarp)
      for (int t = lane; t < tw_; t += 32) {
        double *d = dst + (size_t)x * n2n3 + t;
        *d = acc_mode ? *d + acc[x * T + t] : acc[x * T + t];
      }
    return;
  }

  const int b = blockIdx.y;
  if (MODE == XM_FROM_REAL) {
    const size_t off = (size_t)b * a.rstride + i2 * n3 + c0;
    for (int x = warp; x < n1; x += nwarp) {
      C *row = A + x * pT;
      for (int t = lane; t < T; t += 32) {
        C val = z;
        if (t < tw_) {
          const size_t f = off + (size_t)x * n2n3 + t;
          if (a.rin_is_real) {
            val.x = ((const R *)a.rin)[f] * a.rscale;
          } else {
            val = cscale(((const C *)a.rin)[f], a.rscale);
          }
        }
        row[t] = val;
      }
    }
  } else {
    load_slab(b);
  }
  __syncthreads();
  C *res;
  if (MODE == XM_FROM_REAL) {
    res = fft_lines<false>(A, B, pd.ax[0], tw1, T, nullptr, 1, pT);
  } else if (MODE == XM_HPSI) {
    VMulEpi<R> epi{a.v + i2 * n3 + c0, n2n3, tw_, a.vscale};
    res = fft_lines<true>(A, B, pd.ax[0], tw1, T, nullptr, 1, pT, epi);
    C *oth = res == A ? B : A;
    res = fft_lines<false>(res, oth, pd.ax[0], tw1, T, nullptr, 1, pT);
  } else {
    res = fft_lines<true>(A, B, pd.ax[0], tw1, T, nullptr, 1, pT);
  }
  if (MODE == XM_HPSI || MODE == XM_FROM_REAL) {
    C *Wb = a.W + (size_t)b * pd.np * n2n3 + i2 * n3 + c0;
    for (int x = warp; x < n1; x += nwarp) {
      const int p = pd.plane_of_i1[x];
      if (p < 0) continue;
      C *dst = Wb + p * n2n3;
      const C *row = res + x * pT;
      for (int t = lane; t < tw_; t += 32) dst[t] = row[t];
    }
  } else {  // TO_REAL / TO_REAL_RE
    const size_t off = (size_t)b * a.rstride + i2 * n3 + c0;
    for (int x = warp; x < n1; x += nwarp) {
      const C *row = res + x * pT;
      for (int t = lane; t < tw_; t += 32) {
        const size_t f = off + (size_t)x * n2n3 + t;
        if (MODE == XM_TO_REAL_RE)
          ((R *)a.rout)[f] = row[t].x * a.rscale;
        else
          ((C *)a.rout)[f] = cscale(row[t], a.rscale);
      }
    }
  }
}

const FftTuning &fft_tuning() {
  static const FftTuning tun = [] {
    FftTuning t;
    t.threads_plane = 256;
    t.threads_x = 256;
    t.xtile_kb = 48;
    t.slab_chunk_bytes = size_t(200) << 20;
    t.xline2 = 1;
    t.plane2 = 1;
    t.threads_plane2 = 512;
    t.colfft = 1;
    t.threads_xy = 0;
    t.xy_direct = 1;
    t.plane_split = 0;
    auto env = [](const char *k, long dflt) {
      const char *v = getenv(k);
      return v ? atol(v) : dflt;
    };
    t.threads_plane = (int)env("ADDFT_FFT_THREADS", t.threads_plane);
    t.threads_x = (int)env("ADDFT_FFT_THREADS_X", t.threads_x);
    t.xtile_kb = (int)env("ADDFT_XTILE_KB", t.xtile_kb);
    t.slab_chunk_bytes = (size_t)env("ADDFT_SLAB_MB", (long)(t.slab_chunk_bytes >> 20)) << 20;
    t.xline2 = (int)env("ADDFT_XLINE2", t.xline2);
    t.plane2 = (int)env("ADDFT_PLANE2", t.plane2);
    t.threads_plane2 = (int)env("ADDFT_PLANE2_THREADS", t.threads_plane2);
    t.colfft = (int)std::min(std::max(env("ADDFT_COLFFT", t.colfft), 0L), 2L);
    t.threads_xy = (int)env("ADDFT_XY_THREADS", t.threads_xy);
    t.xy_direct = env("ADDFT_XY_DIRECT", t.xy_direct) ? 1 : 0;
    t.plane_split = env("ADDFT_PLANE_SPLIT", t.plane_split) ? 1 : 0;
    if (t.threads_xy != 0) t.threads_xy = std::min(std::max(t.threads_xy / 32 * 32, 64), kXYMaxThreads);
    auto clampthreads = [](int x) { x = (x / 32) * 32; return x < 64 ? 64 : (x > kFftMaxThreads ? kFftMaxThreads : x); };
    t.threads_plane = clampthreads(t.threads_plane);
    t.threads_x = clampthreads(t.threads_x);
    t.threads_plane2 = clampthreads(t.threads_plane2);
    if (t.xtile_kb < 8) t.xtile_kb = 8;
    if (t.xtile_kb > 200) t.xtile_kb = 200;
    return t;
  }();
  return tun;
}

// rho[f] (+)= sum_s part[s][f]
__global__ void k_density_reduce(const double *__restrict__ part, int nsplit, long N, double *__restrict__ rho,
                                 int acc) {
  for (long f = blockIdx.x * (long)blockDim.x + threadIdx.x; f < N; f += (long)gridDim.x * blockDim.x) {
    double s = acc ? rho[f] : 0.0;
    for (int j = 0; j < nsplit; ++j) s += part[(size_t)j * N + f];
    rho[f] = s;
  }
}

// ---------------------------------------------------------------------------
// host-side launch helpers
// ---------------------------------------------------------------------------
// The split P1 / P2 runs where the plane tiles do not fit (or the plan forces it).
template <typename R>
bool use_plane_split(const PlanDev &pd) {
  if (pd.tun.plane_split) return true;
  int dev = 0, maxb = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&maxb, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return false;   // the plane launch reports the error
  return plane_smem<R>(pd) > (size_t)maxb;
}

template <typename R>
size_t zcols_smem(const PlanDev &pd) {
  return sizeof(typename Cx<R>::T) * (2 * (size_t)pd.n3 * kColPitch + pd.n3);
}

// z-positions per y tile: two n2 x (T | 1) tiles within 64 KB, T <= 32
template <typename R>
int ytile_width(const PlanDev &pd) {
  int t = (int)((size_t(64) << 10) / (2 * sizeof(typename Cx<R>::T) * ((size_t)pd.n2 + 1)));
  t = std::min(std::min(t, 32), pd.n3);
  return t < 1 ? 1 : t;
}

template <typename R>
size_t ytile_smem(const PlanDev &pd, int T) {
  return sizeof(typename Cx<R>::T) * (2 * (size_t)pd.n2 * odd_pitch(T) + pd.n2);
}

template <typename R, bool INV>
addft_status launch_ytile(const PlanDev &pd, int nbatch, typename Cx<R>::T *W, cudaStream_t st) {
  const int T = ytile_width<R>(pd), ntile = (pd.n3 + T - 1) / T;
  const size_t sm = ytile_smem<R>(pd, T);
  ADDFT_TRY(smem_optin(k_ytile<R, INV>, sm));
  k_ytile<R, INV><<<dim3(pd.np * ntile, nbatch), pd.tun.threads_plane, sm, st>>>(pd, W, T, ntile);
  return check_launch("k_ytile");
}

template <typename R>
addft_status launch_split_inv(const PlanDev &pd, int nbatch, const typename Cx<R>::T *psi, long ld, R scale,
                              typename Cx<R>::T *W, cudaStream_t st) {
  const size_t sm = zcols_smem<R>(pd);
  ADDFT_TRY(smem_optin(k_zcols_inv<R>, sm));
  k_zcols_inv<R><<<dim3(pd.ncols_pad / kColGroup, nbatch), pd.tun.threads_plane, sm, st>>>(pd, psi, ld, scale, W);
  ADDFT_TRY(check_launch("k_zcols_inv"));
  return launch_ytile<R, true>(pd, nbatch, W, st);
}

template <typename R, int MODE>
addft_status launch_split_fwd(const PlanDev &pd, int nbatch, typename Cx<R>::T *W, R scale,
                              typename Cx<R>::T *out, long ld, const typename Cx<R>::T *psi_in, const R *kin,
                              int nb_per_k, int batch0, cudaStream_t st) {
  ADDFT_TRY((launch_ytile<R, false>(pd, nbatch, W, st)));
  const size_t sm = zcols_smem<R>(pd);
  ADDFT_TRY(smem_optin(k_zcols_fwd<R, MODE>, sm));
  k_zcols_fwd<R, MODE><<<dim3(pd.ncols_pad / kColGroup, nbatch), pd.tun.threads_plane, sm, st>>>(
      pd, W, scale, out, ld, psi_in, kin, nb_per_k, batch0);
  return check_launch("k_zcols_fwd");
}

template <typename R>
addft_status launch_plane_inv(const PlanDev &pd, int nbatch, const typename Cx<R>::T *psi,
                              long ld, R scale, typename Cx<R>::T *W, cudaStream_t st) {
  if (use_plane_split<R>(pd)) return launch_split_inv<R>(pd, nbatch, psi, ld, scale, W, st);
  if (pd.tun.plane2) {
    const addft_status s = launch_plane_inv2<R>(pd, nbatch, psi, ld, scale, W, st);
    if (s != kPlane2NotHandled) return s;
  }
  const size_t sm = plane_smem<R>(pd);
  ADDFT_TRY(smem_optin(k_plane_inv<R>, sm));
  dim3 grid(pd.np, nbatch);
  k_plane_inv<R><<<grid, pd.tun.threads_plane, sm, st>>>(pd, psi, ld, scale, W);
  return check_launch("k_plane_inv");
}

template <typename R, int MODE>
addft_status launch_plane_fwd(const PlanDev &pd, int nbatch, const typename Cx<R>::T *W, R scale,
                              typename Cx<R>::T *out, long ld, const typename Cx<R>::T *psi_in,
                              const R *kin, int nb_per_k, int batch0, cudaStream_t st) {
  // the split form transforms the slab in place (every caller's slab is scratch, rewritten before reuse)
  if (use_plane_split<R>(pd))
    return launch_split_fwd<R, MODE>(pd, nbatch, const_cast<typename Cx<R>::T *>(W), scale, out, ld, psi_in, kin,
                                     nb_per_k, batch0, st);
  if constexpr (MODE == PM_HPSI) {
    if (pd.tun.plane2) {
      const addft_status s = launch_plane_fwd2<R, MODE>(pd, nbatch, W, scale, out, ld, psi_in, kin, nb_per_k,
                                                        batch0, st);
      if (s != kPlane2NotHandled) return s;
    }
  }
  const size_t sm = plane_smem<R>(pd);
  ADDFT_TRY(smem_optin(k_plane_fwd<R, MODE>, sm));
  dim3 grid(pd.np, nbatch);
  k_plane_fwd<R, MODE><<<grid, pd.tun.threads_plane, sm, st>>>(pd, W, scale, out, ld, psi_in, kin,
                                                      nb_per_k, batch0);
  return check_launch("k_plane_fwd");
}

template <typename R>
inline int pick_t3(const PlanDev &pd, int mode, int nbatch) {
  using C = typename Cx<R>::T;
  (void)nbatch;
  // two ping-pong tiles (+ the f64 accumulator for the density) within ~96 / 64 KB
  const size_t per_col = mode == XM_DENSITY ? (2 * sizeof(C) + sizeof(double)) * pd.n1 : 2 * sizeof(C) * pd.n1;
  int t = (int)((size_t)(mode == XM_DENSITY ? 64 : pd.tun.xtile_kb) * 1024 / per_col);
  if (t > pd.n3) t = pd.n3;
  if (t < 1) t = 1;
  return t;
}

template <typename R, int MODE>
addft_status launch_xline(const PlanDev &pd, int nbatch, XArgs<R> a, cudaStream_t st) {
  if constexpr (MODE == XM_HPSI || MODE == XM_DENSITY) {
    if (pd.tun.xline2) {
      const addft_status s = launch_xline2<R, MODE>(pd, nbatch, a, st);
      if (s != kXline2NotHandled) return s;
    }
  }
  a.t3 = pick_t3<R>(pd, MODE, nbatch);
  a.ntile3 = (pd.n3 + a.t3 - 1) / a.t3;
  size_t sm = xline_smem<R>(pd, a.t3);
  if (MODE == XM_DENSITY) sm += sizeof(double) * (size_t)pd.n1 * a.t3;
  ADDFT_TRY(smem_optin(k_xline<R, MODE>, sm));
  dim3 grid(pd.n2 * a.ntile3, MODE == XM_DENSITY ? a.nsplit : nbatch);
  k_xline<R, MODE><<<grid, pd.tun.threads_x, sm, st>>>(pd, a);
  return check_launch("k_xline");
}

template <typename R>
XArgs<R> xargs_default(void *W) {
  XArgs<R> a;
  memset(&a, 0, sizeof(a));
  a.W = (typename Cx<R>::T *)W;
  a.vscale = 1;
  a.rscale = 1;
  return a;
}

// ---------------------------------------------------------------------------
// entry-point bodies
// ---------------------------------------------------------------------------
template <typename R>
addft_status psi_to_real_t(addft_plan plan, int nbatch, double omega, const void *psi, void *psi_r,
                           void *work, size_t bytes, cudaStream_t st) {
  using C = typename Cx<R>::T;
  const PlanDev &pd = plan->dev;
  Work w;
  ADDFT_TRY(split_work(pd, sizeof(C), work, bytes, w));
  const long N = (long)pd.n1 * pd.n2 * pd.n3;
  const R scale = (R)(1.0 / sqrt(omega));
  for (int b0 = 0; b0 < nbatch; b0 += w.nbfit) {
    const int nbc = min(w.nbfit, nbatch - b0);
    ADDFT_TRY(launch_plane_inv<R>(pd, nbc, (const C *)psi + (size_t)b0 * pd.nG, pd.nG, scale,
                                  (C *)w.W, st));
    XArgs<R> a = xargs_default<R>(w.W);
    a.rout = (C *)psi_r + (size_t)b0 * N;
    a.rstride = N;
    ADDFT_TRY((launch_xline<R, XM_TO_REAL>(pd, nbc, a, st)));
  }
  return ADDFT_OK;
}

template <typename R>
addft_status real_to_psi_t(addft_plan plan, int nbatch, double omega, const void *psi_r, void *psi,
                           void *work, size_t bytes, cudaStream_t st) {
  using C = typename Cx<R>::T;
  const PlanDev &pd = plan->dev;
  Work w;
  ADDFT_TRY(split_work(pd, sizeof(C), work, bytes, w));
  const long N = (long)pd.n1 * pd.n2 * pd.n3;
  const R scale = (R)(sqrt(omega) / (double)N);
  for (int b0 = 0; b0 < nbatch; b0 += w.nbfit) {
    const int nbc = min(w.nbfit, nbatch - b0);
    XArgs<R> a = xargs_default<R>(w.W);
    a.rin = (const C *)psi_r + (size_t)b0 * N;
    a.rin_is_real = 0;
    a.rstride = N;
    ADDFT_TRY((launch_xline<R, XM_FROM_REAL>(pd, nbc, a, st)));
    ADDFT_TRY((launch_plane_fwd<R, PM_PLAIN>(pd, nbc, (const C *)w.W, scale,
                                             (C *)psi + (size_t)b0 * pd.nG, pd.nG, nullptr,
                                             nullptr, 1, 0, st)));
  }
  return ADDFT_OK;
}

// Local part of H psi: kin*psi + FFT^-1[ V(r) FFT[psi] ] (scales cancel to 1/N).
template <typename R>
addft_status hpsi_local_t(addft_plan plan, int nk, int nb, const void *psi, const void *kin,
                          const void *v_r, void *hpsi, void *work, size_t bytes, cudaStream_t st) {
  using C = typename Cx<R>::T;
  const PlanDev &pd = plan->dev;
  if (pd.tun.colfft && colfft_handles<R>(pd) && work != nullptr && ((uintptr_t)work & 255) == 0) {
    // column pipeline: [partials 1 MB | Vt (N reals) | column buffers, n3 x ncols_pad per band]
    const size_t red = size_t(1) << 20;
    const long N = (long)pd.n1 * pd.n2 * pd.n3;
    const size_t vt = ((size_t)N * sizeof(R) + 255) & ~size_t(255);
    const size_t colb = ((size_t)pd.n3 * pd.ncols_pad * sizeof(C) + 255) & ~size_t(255);
    const size_t per = colb + (((size_t)pd.nG * sizeof(C) + 255) & ~size_t(255));
    const size_t ks = ((size_t)nk * pd.nG * sizeof(R) + 255) & ~size_t(255);   // sorted kinetic diagonals
    if (bytes >= red + vt + ks + per) {
      size_t fit = (bytes - red - vt - ks) / per;
      size_t cap = pd.tun.slab_chunk_bytes / per;
      if (cap < 1) cap = 1;
      if (fit > cap) fit = cap;
      const int nbfit = fit > (size_t)(1 << 30) ? (1 << 30) : (int)fit;
      R *Vt = (R *)((char *)work + red);
      R *kin_s = (R *)((char *)work + red + vt);
      C *W = (C *)((char *)work + red + vt + ks);
      C *KP = (C *)((char *)W + (size_t)nbfit * colb);
      ADDFT_TRY(launch_kinsort<R>(pd, (const R *)kin, nk, kin_s, st));
      const int nbatch = nk * nb;
      // colfft = 2: the pipeline as one persistent kernel (FP32, cubic boxes); its dependency
      // counters live in the head of the work buffer (the 1 MB reduction area, unused here)
      const bool fused = sizeof(R) == 4 && pd.tun.colfft == 2 && colfused_handles(pd) &&
                         colfused_ctr_ints(nbfit) * sizeof(int) <= red;
      for (int b0 = 0; b0 < nbatch; b0 += nbfit) {
        const int nbc = min(nbfit, nbatch - b0);
        const C *pin = (const C *)psi + (size_t)b0 * pd.nG;
        if constexpr (sizeof(R) == 4) {
          if (fused) {
            if (b0 == 0) ADDFT_TRY(launch_vxy_only<R>(pd, (const R *)v_r, (R)(1.0 / (double)N), Vt, st));
            const addft_status fs = launch_colfused_hpsi(pd, nbc, (const float2 *)pin, pd.nG, (float2 *)W,
                                                         (float2 *)KP, (const float *)Vt,
                                                         (float2 *)hpsi + (size_t)b0 * pd.nG, (const float *)kin_s,
                                                         nb, b0, (int *)work, st);
            if (fs != kPlane2NotHandled) {
              ADDFT_TRY(fs);
              continue;
            }
          }
        }
        ADDFT_TRY(launch_colfft_hpsi<R>(pd, nbc, pin, pd.nG, (const R *)v_r, (R)(1.0 / (double)N), Vt, b0 == 0,
                                        W, KP, (C *)hpsi + (size_t)b0 * pd.nG, kin_s, nb, b0, st));
      }
      return ADDFT_OK;
    }
  }
  Work w;
  ADDFT_TRY(split_work(pd, sizeof(C), work, bytes, w));
  const long N = (long)pd.n1 * pd.n2 * pd.n3;
  const int nbatch = nk * nb;
  for (int b0 = 0; b0 < nbatch; b0 += w.nbfit) {
    const int nbc = min(w.nbfit, nbatch - b0);
    const C *pin = (const C *)psi + (size_t)b0 * pd.nG;
    ADDFT_TRY(launch_plane_inv<R>(pd, nbc, pin, pd.nG, (R)1, (C *)w.W, st));
    XArgs<R> a = xargs_default<R>(w.W);
    a.v = (const R *)v_r;
    a.vscale = (R)(1.0 / (double)N);
    ADDFT_TRY((launch_xline<R, XM_HPSI>(pd, nbc, a, st)));
    ADDFT_TRY((launch_plane_fwd<R, PM_HPSI>(pd, nbc, (const C *)w.W, (R)1,
                                            (C *)hpsi + (size_t)b0 * pd.nG, pd.nG, pin,
                                            (const R *)kin, nb, b0, st)));
  }
  return ADDFT_OK;
}

template <typename R>
addft_status density_t(addft_plan plan, int nk, int nb, double omega, const void *psi,
                       const double *wocc, double *rho, void *work, size_t bytes, cudaStream_t st) {
  using C = typename Cx<R>::T;
  const PlanDev &pd = plan->dev;
  const int nbatch = nk * nb;
  const long N = (long)pd.n1 * pd.n2 * pd.n3;
  if (nbatch == 0) {
    ADDFT_CUDA(cudaMemsetAsync(rho, 0, sizeof(double) * N, st));
    return ADDFT_OK;
  }
  // split the bands across CTAs so the x-line stage has >= 4 CTAs per SM
  const int t3 = pick_t3<R>(pd, XM_DENSITY, nbatch);
  const int tiles = pd.n2 * ((pd.n3 + t3 - 1) / t3);
  int nsplit = (4 * 152 + tiles - 1) / tiles;
  if (nsplit > 8) nsplit = 8;
  if (nsplit > nbatch) nsplit = nbatch;
  if (nsplit < 1) nsplit = 1;
  size_t part_bytes = nsplit > 1 ? (((size_t)nsplit * N * sizeof(double)) + 255) & ~size_t(255) : 0;
  const size_t slab1 = (size_t(1) << 20) + (size_t)pd.np * pd.n2 * pd.n3 * sizeof(C);
  if (part_bytes && (work == nullptr || bytes < part_bytes + slab1)) {
    nsplit = 1;
    part_bytes = 0;
  }
  Work w;
  ADDFT_TRY(split_work(pd, sizeof(C), (char *)work + part_bytes, bytes - part_bytes, w));
  double *part = (double *)work;
  for (int b0 = 0; b0 < nbatch; b0 += w.nbfit) {
    const int nbc = min(w.nbfit, nbatch - b0);
    ADDFT_TRY(launch_plane_inv<R>(pd, nbc, (const C *)psi + (size_t)b0 * pd.nG, pd.nG, (R)1,
                                  (C *)w.W, st));
    XArgs<R> a = xargs_default<R>(w.W);
    a.nbatch = nbc;
    a.wocc = wocc + b0;
    a.dscale = 1.0 / omega;
    a.rho = rho;
    a.rho_acc = b0 > 0;
    a.nsplit = min(nsplit, nbc);
    a.part = part;
    a.N = N;
    ADDFT_TRY((launch_xline<R, XM_DENSITY>(pd, nbc, a, st)));
    if (a.nsplit > 1) {
      k_density_reduce<<<(int)std::min<long>((N + 255) / 256, 2048), 256, 0, st>>>(part, a.nsplit, N, rho,
                                                                                    b0 > 0);
      ADDFT_TRY(check_launch("k_density_reduce"));
    }
  }
  return ADDFT_OK;
}

// instantiations used by other translation units
template addft_status launch_plane_inv<double>(const PlanDev &, int, const double2 *, long, double,
                                               double2 *, cudaStream_t);
template addft_status launch_plane_fwd<double, PM_PLAIN>(const PlanDev &, int, const double2 *,
                                                         double, double2 *, long, const double2 *,
                                                         const double *, int, int, cudaStream_t);
template addft_status launch_xline<double, XM_FROM_REAL>(const PlanDev &, int, XArgs<double>,
                                                         cudaStream_t);
template addft_status launch_xline<double, XM_TO_REAL_RE>(const PlanDev &, int, XArgs<double>,
                                                          cudaStream_t);
template XArgs<double> xargs_default<double>(void *);
template addft_status hpsi_local_t<float>(addft_plan, int, int, const void *, const void *,
                                          const void *, void *, void *, size_t, cudaStream_t);
template addft_status hpsi_local_t<double>(addft_plan, int, int, const void *, const void *,
                                           const void *, void *, void *, size_t, cudaStream_t);

}  // namespace addft

using namespace addft;

extern "C" {

addft_status addft_psi_to_real(addft_plan plan, addft_dtype dt, int nbatch, double omega,
                               const void *psi, void *psi_r, void *work, size_t work_bytes,
                               void *stream) {
  ADDFT_REQUIRE(plan && nbatch >= 0 && omega > 0 && (nbatch == 0 || (psi && psi_r)), ADDFT_INVALID_ARG,
                "psi_to_real: bad arguments");
  if (nbatch == 0) return ADDFT_OK;
  return dt == ADDFT_F64
             ? psi_to_real_t<double>(plan, nbatch, omega, psi, psi_r, work, work_bytes, as_stream(stream))
             : psi_to_real_t<float>(plan, nbatch, omega, psi, psi_r, work, work_bytes, as_stream(stream));
}

addft_status addft_real_to_psi(addft_plan plan, addft_dtype dt, int nbatch, double omega,
                               const void *psi_r, void *psi, void *work, size_t work_bytes,
                               void *stream) {
  ADDFT_REQUIRE(plan && nbatch >= 0 && omega > 0 && (nbatch == 0 || (psi && psi_r)), ADDFT_INVALID_ARG,
                "real_to_psi: bad arguments");
  if (nbatch == 0) return ADDFT_OK;
  return dt == ADDFT_F64
             ? real_to_psi_t<double>(plan, nbatch, omega, psi_r, psi, work, work_bytes, as_stream(stream))
             : real_to_psi_t<float>(plan, nbatch, omega, psi_r, psi, work, work_bytes, as_stream(stream));
}

addft_status addft_density(addft_plan plan, addft_dtype dt, int nk, int nb, double omega,
                           const void *psi, const double *wocc, double *rho, void *work,
                           size_t work_bytes, void *stream) {
  ADDFT_REQUIRE(plan && rho && nk >= 0 && nb >= 0 && omega > 0, ADDFT_INVALID_ARG,
                "density: bad arguments");
  ADDFT_REQUIRE(nk * nb == 0 || (psi && wocc), ADDFT_INVALID_ARG, "density: null psi/wocc");
  return dt == ADDFT_F64
             ? density_t<double>(plan, nk, nb, omega, psi, wocc, rho, work, work_bytes, as_stream(stream))
             : density_t<float>(plan, nk, nb, omega, psi, wocc, rho, work, work_bytes, as_stream(stream));
}

}  // extern "C"
