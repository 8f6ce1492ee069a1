// Declarations shared by the translation units that drive the sphere-aware
// FFT pipeline (kernels and launch helpers live in transforms.cu).
#pragma once
#include <algorithm>

#include "fft.cuh"

namespace addft {


enum XMode { XM_HPSI = 0, XM_TO_REAL = 1, XM_TO_REAL_RE = 2, XM_FROM_REAL = 3, XM_DENSITY = 4 };
enum PMode { PM_PLAIN = 0, PM_HPSI = 1 };

constexpr int kFftMaxThreads = 512;   // launch bound of the FFT pipeline kernels
constexpr int kXYMaxThreads = 1024;   // launch bound of the xy-plane kernel of the column pipeline

// Process defaults of the launch tunables (FftTuning, common.cuh); every plan
// starts from them and may override them with addft_plan_set_tuning.
const FftTuning &fft_tuning();

template <typename R>
struct XArgs {
  using C = typename Cx<R>::T;
  C *W;
  int t3;                 // columns per CTA (tile width along i3)
  int ntile3;             // ceil(n3 / t3)
  const R *v;             // XM_HPSI: V(r), (N,)
  R vscale;
  const void *rin;        // XM_FROM_REAL: input field (batch, N)
  int rin_is_real;        //   1: real R, 0: complex C
  void *rout;             // XM_TO_REAL(_RE): output (batch, N)
  long rstride;           // batch stride (elements) of rin / rout
  R rscale;               // scale applied on load (FROM_REAL) or store (TO_REAL)
  int nbatch;             // XM_DENSITY: bands in this chunk
  const double *wocc;     // XM_DENSITY: weights of the chunk's bands
  double dscale;          // XM_DENSITY: |psi|^2 scale (1/omega)
  double *rho;            // XM_DENSITY: output
  int rho_acc;            //   add into rho (1) or overwrite (0)
  int nsplit;             // XM_DENSITY: band splits across CTAs (grid.y)
  double *part;           // XM_DENSITY: per-split partial slabs (nsplit x N) when nsplit > 1
  long N;                 // XM_DENSITY: points in the box
};

struct Work {
  double *partial;   // reduction partials (1 MB)
  void *W;           // slabs
  int nbfit;         // bands per chunk
};

inline addft_status split_work(const PlanDev &pd, size_t csz, void *work, size_t bytes, Work &w) {
  const size_t red = size_t(1) << 20;
  const size_t per = (size_t)pd.np * pd.n2 * pd.n3 * csz;
  ADDFT_REQUIRE(work != nullptr && bytes >= red + per, ADDFT_INVALID_ARG,
                "work buffer of %zu B too small (need >= %zu B)", bytes, red + per);
  ADDFT_REQUIRE(((uintptr_t)work & 255) == 0, ADDFT_INVALID_ARG, "work buffer must be 256-byte aligned");
  w.partial = (double *)work;
  w.W = (char *)work + red;
  size_t fit = (bytes - red) / per;
  size_t l2fit = pd.tun.slab_chunk_bytes / per;
  if (l2fit < 1) l2fit = 1;
  if (fit > l2fit) fit = l2fit;
  w.nbfit = fit > (size_t)(1 << 30) ? (1 << 30) : (int)fit;
  return ADDFT_OK;
}

template <typename R>
inline size_t plane_smem(const PlanDev &pd) {
  using C = typename Cx<R>::T;
  return sizeof(C) * (2 * (size_t)pd.n2 * odd_pitch(pd.n3) + pd.n2 + pd.n3);
}

// the two-pass inverse plane kernel works in place on one tile
template <typename R>
inline size_t plane2_smem(const PlanDev &pd) {
  using C = typename Cx<R>::T;
  return sizeof(C) * ((size_t)pd.n2 * odd_pitch(pd.n3) + pd.n2 + pd.n3);
}

template <typename R>
inline size_t xline_smem(const PlanDev &pd, int t3) {
  using C = typename Cx<R>::T;
  return sizeof(C) * (2 * (size_t)pd.n1 * odd_pitch(t3) + pd.n1);
}


template <typename R>
addft_status launch_plane_inv(const PlanDev &pd, int nbatch, const typename Cx<R>::T *psi,
                              long ld, R scale, typename Cx<R>::T *W, cudaStream_t st);
template <typename R, int MODE>
addft_status launch_plane_fwd(const PlanDev &pd, int nbatch, const typename Cx<R>::T *W, R scale,
                              typename Cx<R>::T *out, long ld, const typename Cx<R>::T *psi_in,
                              const R *kin, int nb_per_k, int batch0, cudaStream_t st);
template <typename R, int MODE>
addft_status launch_xline(const PlanDev &pd, int nbatch, XArgs<R> a, cudaStream_t st);
template <typename R>
XArgs<R> xargs_default(void *W);
// returned by launch_xline2 / launch_plane_*2 when there is no two-pass instantiation
constexpr addft_status kXline2NotHandled = -1;
constexpr addft_status kPlane2NotHandled = -1;
template <typename R>
addft_status launch_plane_inv2(const PlanDev &pd, int nbatch, const typename Cx<R>::T *psi, long ld, R scale,
                               typename Cx<R>::T *W, cudaStream_t st);
template <typename R, int MODE>
addft_status launch_plane_fwd2(const PlanDev &pd, int nbatch, const typename Cx<R>::T *W, R scale,
                               typename Cx<R>::T *out, long ld, const typename Cx<R>::T *psi_in, const R *kin,
                               int nb_per_k, int batch0, cudaStream_t st);
template <typename R, int MODE>
addft_status launch_xline2(const PlanDev &pd, int nbatch, XArgs<R> a, cudaStream_t st);
template <typename R>
addft_status hpsi_local_t(addft_plan plan, int nk, int nb, const void *psi, const void *kin,
                          const void *v_r, void *hpsi, void *work, size_t bytes, cudaStream_t st);

}  // namespace addft
