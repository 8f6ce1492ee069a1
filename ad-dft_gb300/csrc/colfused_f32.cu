// Instantiations and launch of the fused column pipeline (colfused.cuh), FP32.
#include <cstdlib>

#include "colfused.cuh"

namespace addft {

// cubic boxes n = P Q of the fused kernel: 72, 48, 75, 60, 30, 32, 24
#define CFU_CASES(X) X(9, 8) X(8, 6) X(15, 5) X(10, 6) X(6, 5) X(8, 4) X(6, 4)

namespace {

bool axis_pq(const AxisPlan &ax, int &P, int &Q) {
  if (ax.nst != 2) return false;
  P = ax.rad[0];
  Q = ax.rad[1];
  return true;
}

template <int P, int Q>
addft_status fused_go(const PlanDev &pd, int nbatch, const float2 *psi, long ld, float2 *W, float2 *KP,
                      const float *Vt, float2 *out, const float *kin_s, int nb_per_k, int batch0, int *ctr,
                      cudaStream_t st) {
  auto kern = k_hpsi_colfused<float, P, Q>;
  const size_t sm = fused_smem_fixed<float, P, Q>() + sizeof(int) * (size_t)pd.np;
  ADDFT_TRY(smem_optin(kern, sm));
  int dev = 0, nsm = 0, per_sm = 0;
  ADDFT_CUDA(cudaGetDevice(&dev));
  ADDFT_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  ADDFT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFusedThreads, sm));
  ADDFT_REQUIRE(per_sm >= 1, ADDFT_UNSUPPORTED, "fused H psi kernel does not fit on an SM");
  // steps between the stages of one band (ADDFT_FUSED_LAG, read once per process)
  static const int lag = [] {
    const char *v = getenv("ADDFT_FUSED_LAG");
    const int x = v ? atoi(v) : 8;
    return x >= 1 && x <= 16 ? x : 8;
  }();
  const long total = (long)(nbatch + 2 * lag) * (2 * (pd.ncols_pad / kColGroup) + pd.n3);
  ADDFT_REQUIRE(total < (1L << 30), ADDFT_UNSUPPORTED, "fused H psi: too many work items");
  const int grid = (int)std::max(1L, std::min<long>((long)per_sm * nsm, total));
  ADDFT_CUDA(cudaMemsetAsync(ctr, 0, sizeof(int) * colfused_ctr_ints(nbatch), st));
  kern<<<grid, kFusedThreads, sm, st>>>(pd, nbatch, psi, ld, W, KP, Vt, out, kin_s, nb_per_k, batch0, lag, ctr);
  return check_launch("k_hpsi_colfused");
}

}  // namespace

bool colfused_handles(const PlanDev &pd) {
  int P1, Q1, P2, Q2, P3, Q3;
  if (!pd.xy_direct || !pd.tun.xy_direct) return false;
  if (!axis_pq(pd.ax[0], P1, Q1) || !axis_pq(pd.ax[1], P2, Q2) || !axis_pq(pd.ax[2], P3, Q3)) return false;
  if (P1 != P2 || P1 != P3 || Q1 != Q2 || Q1 != Q3) return false;
  switch (P1 * 100 + Q1) {
#define CFU_K(p, q) case p * 100 + q:
    CFU_CASES(CFU_K)
#undef CFU_K
    return true;
    default: return false;
  }
}

addft_status launch_colfused_hpsi(const PlanDev &pd, int nbatch, const float2 *psi, long ld, float2 *W, float2 *KP,
                                  const float *Vt, float2 *out, const float *kin_s, int nb_per_k, int batch0,
                                  int *ctr, cudaStream_t st) {
  if (!colfused_handles(pd)) return kPlane2NotHandled;
  switch (pd.ax[0].rad[0] * 100 + pd.ax[0].rad[1]) {
#define CFU_GO(p, q) \
  case p * 100 + q: return fused_go<p, q>(pd, nbatch, psi, ld, W, KP, Vt, out, kin_s, nb_per_k, batch0, ctr, st);
    CFU_CASES(CFU_GO)
#undef CFU_GO
    default: return kPlane2NotHandled;
  }
}

}  // namespace addft

extern "C" {

// Device error bits of the fused H psi kernel since the last call (bit 0: a bounded
// dependency wait ran out; that launch's results are not valid); reading clears them.
// Synchronises with the device.
unsigned addft_hpsi_fused_status(void) {
  unsigned v = 0, z = 0;
  if (cudaMemcpyFromSymbol(&v, addft::g_fused_error, sizeof(v)) != cudaSuccess) return 0xffffffffu;
  cudaMemcpyToSymbol(addft::g_fused_error, &z, sizeof(z));
  return v;
}

}  // extern "C"
