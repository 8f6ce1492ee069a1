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
// Only planes and rows that carry sphere points are transformed in the
// sparse directions, and the intermediate slabs stay L2-resident for the
// band chunk in flight.  Replaces psi_to_real / real_to_psi / potential_apply
// (src/addft/geometry/basis.py:205-254, src/addft/ops/hpsi.py:29-32) and the
// scatter/gather kernels of native/pack.cu:16-38.
#include "transforms.cuh"

namespace addft {
// ---------------------------------------------------------------------------
// P1: sphere -> slab (z and y inverse transforms)
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(kFftThreads)
k_plane_inv(PlanDev pd, const typename Cx<R>::T *__restrict__ psi, long ld_psi, R scale,
            typename Cx<R>::T *__restrict__ W) {
  using C = typename Cx<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int S = pd.n2 * pd.n3;
  C *A = reinterpret_cast<C *>(smem_raw);
  C *B = A + S;
  C *tw2 = B + S;
  C *tw3 = tw2 + pd.n2;
  const int p = blockIdx.x;
  const int b = blockIdx.y;
  const C z = czero<C>();
  for (int i = threadIdx.x; i < S; i += blockDim.x) { A[i] = z; B[i] = z; }
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
  C *cur = fft_lines<true>(A, B, pd.ax[2], tw3, nrow, pd.row_i2 + r0, pd.n3, 1);
  C *oth = cur == A ? B : A;
  C *res = fft_lines<true>(cur, oth, pd.ax[1], tw2, pd.n3, nullptr, 1, pd.n3);
  C *dst = W + ((size_t)b * pd.np + p) * S;
  for (int i = threadIdx.x; i < S; i += blockDim.x) dst[i] = res[i];
}

// ---------------------------------------------------------------------------
// P2: slab -> sphere (y and z forward transforms, gather, kinetic)
// ---------------------------------------------------------------------------
template <typename R, int MODE>
__global__ void __launch_bounds__(kFftThreads)
k_plane_fwd(PlanDev pd, const typename Cx<R>::T *__restrict__ W, R scale,
            typename Cx<R>::T *__restrict__ out, long ld_out,
            const typename Cx<R>::T *__restrict__ psi_in, const R *__restrict__ kin, int nb_per_k,
            int batch0) {
  using C = typename Cx<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int S = pd.n2 * pd.n3;
  C *A = reinterpret_cast<C *>(smem_raw);
  C *B = A + S;
  C *tw2 = B + S;
  C *tw3 = tw2 + pd.n2;
  const int p = blockIdx.x;
  const int b = blockIdx.y;
  const C *srcw = W + ((size_t)b * pd.np + p) * S;
  for (int i = threadIdx.x; i < S; i += blockDim.x) A[i] = srcw[i];
  const C *g2 = twiddles<R>(pd, 1), *g3 = twiddles<R>(pd, 2);
  for (int i = threadIdx.x; i < pd.n2; i += blockDim.x) tw2[i] = g2[i];
  for (int i = threadIdx.x; i < pd.n3; i += blockDim.x) tw3[i] = g3[i];
  __syncthreads();
  C *cur = fft_lines<false>(A, B, pd.ax[1], tw2, pd.n3, nullptr, 1, pd.n3);
  C *oth = cur == A ? B : A;
  const int r0 = pd.rptr[p], nrow = pd.rptr[p + 1] - r0;
  C *res = fft_lines<false>(cur, oth, pd.ax[2], tw3, nrow, pd.row_i2 + r0, pd.n3, 1);
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
// X: x-line transforms over a (i2, i3-tile) column block
// ---------------------------------------------------------------------------


template <typename R, int MODE>
__global__ void __launch_bounds__(kFftThreads)
k_xline(PlanDev pd, XArgs<R> a) {
  using C = typename Cx<R>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n1 = pd.n1, n2 = pd.n2, n3 = pd.n3;
  const int T = a.t3;
  const int S = n1 * T;
  C *A = reinterpret_cast<C *>(smem_raw);
  C *B = A + S;
  C *tw1 = B + S;
  const int i2 = blockIdx.x / a.ntile3;
  const int c0 = (blockIdx.x - i2 * a.ntile3) * T;
  const int tw_ = min(T, n3 - c0);   // valid columns in this tile
  const C *g1 = twiddles<R>(pd, 0);
  for (int i = threadIdx.x; i < n1; i += blockDim.x) tw1[i] = g1[i];
  const C z = czero<C>();

  auto load_slab = [&](int b) {
    const C *Wb = a.W + (size_t)b * pd.np * n2 * n3;
    for (int i = threadIdx.x; i < S; i += blockDim.x) {
      const int x = i / T, t = i - x * T;
      const int p = pd.plane_of_i1[x];
      C val = z;
      if (p >= 0 && t < tw_) val = Wb[((size_t)p * n2 + i2) * n3 + c0 + t];
      A[i] = val;
    }
  };

  if (MODE == XM_DENSITY) {
    double acc[kDensSlots];
#pragma unroll
    for (int s = 0; s < kDensSlots; ++s) acc[s] = 0.0;
    for (int b = 0; b < a.nbatch; ++b) {
      load_slab(b);
      __syncthreads();
      C *res = fft_lines<true>(A, B, pd.ax[0], tw1, T, nullptr, 1, T);
      const double wb = a.wocc[b] * a.dscale;
#pragma unroll
      for (int s = 0; s < kDensSlots; ++s) {
        const int i = threadIdx.x + s * blockDim.x;
        if (i < S) {
          const C v = res[i];
          acc[s] += wb * ((double)v.x * (double)v.x + (double)v.y * (double)v.y);
        }
      }
      __syncthreads();
    }
#pragma unroll
    for (int s = 0; s < kDensSlots; ++s) {
      const int i = threadIdx.x + s * blockDim.x;
      if (i < S) {
        const int x = i / T, t = i - x * T;
        if (t < tw_) {
          const size_t f = ((size_t)x * n2 + i2) * n3 + c0 + t;
          a.rho[f] = a.rho_acc ? a.rho[f] + acc[s] : acc[s];
        }
      }
    }
    return;
  }

  const int b = blockIdx.y;
  if (MODE == XM_FROM_REAL) {
    for (int i = threadIdx.x; i < S; i += blockDim.x) {
      const int x = i / T, t = i - x * T;
      C val = z;
      if (t < tw_) {
        const size_t f = (size_t)b * a.rstride + ((size_t)x * n2 + i2) * n3 + c0 + t;
        if (a.rin_is_real) {
          val.x = ((const R *)a.rin)[f] * a.rscale;
        } else {
          val = cscale(((const C *)a.rin)[f], a.rscale);
        }
      }
      A[i] = val;
    }
  } else {
    load_slab(b);
  }
  __syncthreads();
  C *res;
  if (MODE == XM_FROM_REAL) {
    res = fft_lines<false>(A, B, pd.ax[0], tw1, T, nullptr, 1, T);
  } else {
    res = fft_lines<true>(A, B, pd.ax[0], tw1, T, nullptr, 1, T);
  }
  if (MODE == XM_HPSI) {
    for (int i = threadIdx.x; i < S; i += blockDim.x) {
      const int x = i / T, t = i - x * T;
      R vv = 0;
      if (t < tw_) vv = a.v[((size_t)x * n2 + i2) * n3 + c0 + t] * a.vscale;
      res[i] = cscale(res[i], vv);
    }
    __syncthreads();
    C *oth = res == A ? B : A;
    res = fft_lines<false>(res, oth, pd.ax[0], tw1, T, nullptr, 1, T);
  }
  if (MODE == XM_HPSI || MODE == XM_FROM_REAL) {
    C *Wb = a.W + (size_t)b * pd.np * n2 * n3;
    for (int i = threadIdx.x; i < S; i += blockDim.x) {
      const int x = i / T, t = i - x * T;
      const int p = pd.plane_of_i1[x];
      if (p >= 0 && t < tw_) Wb[((size_t)p * n2 + i2) * n3 + c0 + t] = res[i];
    }
  } else {  // TO_REAL / TO_REAL_RE
    for (int i = threadIdx.x; i < S; i += blockDim.x) {
      const int x = i / T, t = i - x * T;
      if (t < tw_) {
        const size_t f = (size_t)b * a.rstride + ((size_t)x * n2 + i2) * n3 + c0 + t;
        if (MODE == XM_TO_REAL_RE)
          ((R *)a.rout)[f] = res[i].x * a.rscale;
        else
          ((C *)a.rout)[f] = cscale(res[i], a.rscale);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// host-side launch helpers
// ---------------------------------------------------------------------------
template <typename R>
addft_status launch_plane_inv(const PlanDev &pd, int nbatch, const typename Cx<R>::T *psi,
                              long ld, R scale, typename Cx<R>::T *W, cudaStream_t st) {
  const size_t sm = plane_smem<R>(pd);
  ADDFT_TRY(smem_optin(k_plane_inv<R>, sm));
  dim3 grid(pd.np, nbatch);
  k_plane_inv<R><<<grid, kFftThreads, sm, st>>>(pd, psi, ld, scale, W);
  return check_launch("k_plane_inv");
}

template <typename R, int MODE>
addft_status launch_plane_fwd(const PlanDev &pd, int nbatch, const typename Cx<R>::T *W, R scale,
                              typename Cx<R>::T *out, long ld, const typename Cx<R>::T *psi_in,
                              const R *kin, int nb_per_k, int batch0, cudaStream_t st) {
  const size_t sm = plane_smem<R>(pd);
  ADDFT_TRY(smem_optin(k_plane_fwd<R, MODE>, sm));
  dim3 grid(pd.np, nbatch);
  k_plane_fwd<R, MODE><<<grid, kFftThreads, sm, st>>>(pd, W, scale, out, ld, psi_in, kin,
                                                      nb_per_k, batch0);
  return check_launch("k_plane_fwd");
}

template <typename R>
inline int pick_t3(const PlanDev &pd, int mode, int nbatch) {
  if (mode == XM_DENSITY) {
    // register accumulator bound, and >= ~2 CTAs per SM of column tiles
    int t = (kDensSlots * kFftThreads) / pd.n1;
    if (t > pd.n3) t = pd.n3;
    const int want_tiles = (304 + pd.n2 - 1) / pd.n2;
    int t2 = (pd.n3 + want_tiles - 1) / want_tiles;
    if (t2 < 8) t2 = 8;
    if (t2 < t) t = t2;
    if (t < 1) t = 1;
    return t;
  }
  (void)nbatch;
  // keep the two ping-pong tiles within ~96 KB
  using C = typename Cx<R>::T;
  int t = (int)((96 * 1024) / (2 * sizeof(C) * pd.n1));
  if (t > pd.n3) t = pd.n3;
  if (t < 1) t = 1;
  return t;
}

template <typename R, int MODE>
addft_status launch_xline(const PlanDev &pd, int nbatch, XArgs<R> a, cudaStream_t st) {
  a.t3 = pick_t3<R>(pd, MODE, nbatch);
  a.ntile3 = (pd.n3 + a.t3 - 1) / a.t3;
  if (MODE == XM_DENSITY)
    ADDFT_REQUIRE(pd.n1 * a.t3 <= kDensSlots * kFftThreads, ADDFT_UNSUPPORTED,
                  "density accumulator: n1 = %d too large", pd.n1);
  const size_t sm = xline_smem<R>(pd, a.t3);
  ADDFT_TRY(smem_optin(k_xline<R, MODE>, sm));
  dim3 grid(pd.n2 * a.ntile3, MODE == XM_DENSITY ? 1 : nbatch);
  k_xline<R, MODE><<<grid, kFftThreads, sm, st>>>(pd, a);
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
  Work w;
  ADDFT_TRY(split_work(pd, sizeof(C), work, bytes, w));
  const int nbatch = nk * nb;
  const long N = (long)pd.n1 * pd.n2 * pd.n3;
  if (nbatch == 0) {
    ADDFT_CUDA(cudaMemsetAsync(rho, 0, sizeof(double) * N, st));
    return ADDFT_OK;
  }
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
    ADDFT_TRY((launch_xline<R, XM_DENSITY>(pd, nbc, a, st)));
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
  ADDFT_REQUIRE(plan && psi && psi_r && nbatch >= 0 && omega > 0, ADDFT_INVALID_ARG,
                "psi_to_real: bad arguments");
  if (nbatch == 0) return ADDFT_OK;
  return dt == ADDFT_F64
             ? psi_to_real_t<double>(plan, nbatch, omega, psi, psi_r, work, work_bytes, as_stream(stream))
             : psi_to_real_t<float>(plan, nbatch, omega, psi, psi_r, work, work_bytes, as_stream(stream));
}

addft_status addft_real_to_psi(addft_plan plan, addft_dtype dt, int nbatch, double omega,
                               const void *psi_r, void *psi, void *work, size_t work_bytes,
                               void *stream) {
  ADDFT_REQUIRE(plan && psi && psi_r && nbatch >= 0 && omega > 0, ADDFT_INVALID_ARG,
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
