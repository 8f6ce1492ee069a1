// Density-side kernels (f64): LDA PZ81 exchange-correlation with its VJP,
// Hartree in G space on the wavefunction shell, the local pseudopotential,
// and the density terms of the envelope gradients (local and Hartree).
//
// Reference: src/addft/physics/xc.py:139-212 (PZ81, the native
// custom_vjp), native/xc_lda.cu:8-54, physics/hartree.py:21-48,
// physics/local.py:21-39, solver/scf.py:81-92 (effective_potential).
#include "radial.cuh"
#include "transforms.cuh"
#include "xc.cuh"

namespace addft {

constexpr int kMaxAtomsP = 256;

// sums: [0] sum n eps_x, [1] sum n eps_c, [2] sum v_xc rho_dc
__global__ void __launch_bounds__(kRedThreads)
k_xc_lda(int n, const double *__restrict__ rho, const double *__restrict__ rho_dc,
         const double *__restrict__ v_loc, const double *__restrict__ v_h, double *__restrict__ v_xc,
         double *__restrict__ v_eff, double *__restrict__ partial) {
  double acc[3] = {0.0, 0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double r = rho[i];
    const XcPoint x = pz81(r);
    const double nn = fmax(r, 1e-14);
    acc[0] += nn * x.ex;
    acc[1] += nn * x.ec;
    acc[2] += x.v * (rho_dc ? rho_dc[i] : r);
    if (v_xc) v_xc[i] = x.v;
    if (v_eff) v_eff[i] = x.v + (v_loc ? v_loc[i] : 0.0) + (v_h ? v_h[i] : 0.0);
  }
  block_reduce_store<3>(acc, partial);
}

__global__ void k_xc_vjp(int n, const double *__restrict__ rho, const double *__restrict__ g,
                         double *__restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = pz81(rho[i]).f * g[i];
}

// ---------------------------------------------------------------------------
// G-shell helpers
// ---------------------------------------------------------------------------
struct ShellGeo {
  double B[9];
  double omega;
  int nat;
  double pos[kMaxAtomsP * 3];
  double vamp, vsig;
  int kind, nrad;      // kind 1: tabulated smooth part (function nrad of rt) + Coulomb tail
  RadialTab rt;
  double g0, zval;
};

// v~_loc(q) and d v~_loc / dq (psp.py:92-95 analytic; psp.py:102-119 UPF)
__device__ __forceinline__ void vloc_eval(const ShellGeo &sg, double q, double &v0, double &v1) {
  if (sg.kind == 0) {
    v0 = -sg.vamp * exp(-0.5 * (q * sg.vsig) * (q * sg.vsig));
    v1 = -q * sg.vsig * sg.vsig * v0;
    return;
  }
  if (q <= 1e-12) {
    v0 = sg.g0;
    v1 = 0.0;
    return;
  }
  double s, ds;
  radial_eval(sg.rt, sg.nrad, q, s, ds);
  const double fz = 4.0 * 3.14159265358979323846 * sg.zval * exp(-0.25 * q * q);
  v0 = s - fz / (q * q);
  v1 = ds + fz * (0.5 / q + 2.0 / (q * q * q));
}

__device__ __forceinline__ void gvec(const PlanDev &pd, const ShellGeo &sg, int g, double *G) {
  const double m1 = pd.miller[3 * g], m2 = pd.miller[3 * g + 1], m3 = pd.miller[3 * g + 2];
  G[0] = m1 * sg.B[0] + m2 * sg.B[3] + m3 * sg.B[6];
  G[1] = m1 * sg.B[1] + m2 * sg.B[4] + m3 * sg.B[7];
  G[2] = m1 * sg.B[2] + m2 * sg.B[5] + m3 * sg.B[8];
}

// Hartree in G: V = 4 pi n / G^2 (G != 0), E partial = Re(n V*) ; also dE_H/deps partials
// partial layout [10][nblk]: [0] sum_{G} 4 pi |n|^2/G^2, [1..9] sum 4 pi |n|^2 G_a G_b / G^4
__global__ void __launch_bounds__(kRedThreads)
k_hartree_g(PlanDev pd, ShellGeo sg, const double2 *__restrict__ ng, double2 *__restrict__ vg,
            double *__restrict__ partial) {
  double acc[10];
#pragma unroll
  for (int j = 0; j < 10; ++j) acc[j] = 0.0;
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < pd.nG; g += gridDim.x * blockDim.x) {
    double G[3];
    gvec(pd, sg, g, G);
    const double q2 = G[0] * G[0] + G[1] * G[1] + G[2] * G[2];
    const double2 n = ng[g];
    double2 v = make_double2(0.0, 0.0);
    if (q2 > 1e-14) {
      const double s = 4.0 * 3.14159265358979323846 / q2;
      v = make_double2(n.x * s, n.y * s);
      const double e = (n.x * n.x + n.y * n.y) * s;
      acc[0] += e;
      const double e2 = e / q2;
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) acc[1 + 3 * a + b] += e2 * G[a] * G[b];
    }
    if (vg) vg[g] = v;
  }
  block_reduce_store<10>(acc, partial);
}

// E_H = omega/2 sum, dE_H/deps_ab = -E_H delta + 2 omega sum(...)   (rho ~ 1/omega)
__global__ void k_hartree_final(const double *__restrict__ sums, double omega, double *__restrict__ e_h,
                                double *__restrict__ deps) {
  if (threadIdx.x != 0) return;
  const double E = 0.5 * omega * sums[0];
  if (e_h) *e_h = E;
  if (deps)
    for (int ab = 0; ab < 9; ++ab) deps[ab] = omega * sums[1 + ab] - ((ab % 4 == 0) ? E : 0.0);
}

// V_loc(G) on the density shell: (1/omega) v~(|G|) sum_i e^{-iG.R_i}
__global__ void k_vloc_g(PlanDev pd, ShellGeo sg, double2 *__restrict__ vg) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= pd.nG) return;
  double G[3];
  gvec(pd, sg, g, G);
  const double q2 = G[0] * G[0] + G[1] * G[1] + G[2] * G[2];
  const double q = q2 > 1e-30 ? sqrt(q2) : 0.0;
  double amp, damp;
  vloc_eval(sg, q, amp, damp);
  double re = 0.0, im = 0.0;
  for (int i = 0; i < sg.nat; ++i) {
    double sn, cs;
    sincos(G[0] * sg.pos[3 * i] + G[1] * sg.pos[3 * i + 1] + G[2] * sg.pos[3 * i + 2], &sn, &cs);
    re += cs;
    im -= sn;
  }
  const double s = amp / sg.omega;
  vg[g] = make_double2(re * s, im * s);
}

// Local-energy terms on the density shell, n(G) given:
//   E_loc = Re sum_G v~(|G|) S(G) conj(n),   S = sum_i e^{-iG.R_i}
//   dE/deps_ab = -E_loc delta + sum_G v~'(q) (-G_a G_b / q) Re(S conj n)
// partial [10][nblk]: [0] E_loc, [1..9] second term
__global__ void __launch_bounds__(kRedThreads)
k_local_sums(PlanDev pd, ShellGeo sg, const double2 *__restrict__ ng, double *__restrict__ partial) {
  double acc[10];
#pragma unroll
  for (int j = 0; j < 10; ++j) acc[j] = 0.0;
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < pd.nG; g += gridDim.x * blockDim.x) {
    double G[3];
    gvec(pd, sg, g, G);
    const double q2 = G[0] * G[0] + G[1] * G[1] + G[2] * G[2];
    const double q = q2 > 1e-30 ? sqrt(q2) : 0.0;
    double v0, v1;
    vloc_eval(sg, q, v0, v1);
    double sr = 0.0, si = 0.0;
    for (int i = 0; i < sg.nat; ++i) {
      double sn, cs;
      sincos(G[0] * sg.pos[3 * i] + G[1] * sg.pos[3 * i + 1] + G[2] * sg.pos[3 * i + 2], &sn, &cs);
      sr += cs;
      si -= sn;
    }
    const double2 n = ng[g];
    const double re = sr * n.x + si * n.y;   // Re(S conj(n))
    acc[0] += v0 * re;
    if (q > 0.0) {
      const double c = -v1 * re / q;
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) acc[1 + 3 * a + b] += c * G[a] * G[b];
    }
  }
  block_reduce_store<10>(acc, partial);
}

// local forces: dE/dR_{i,a} = sum_G v~ G_a Im(e^{-iG.R_i} conj(n));  grid (nat, nsplit)
__global__ void __launch_bounds__(kRedThreads)
k_local_force(PlanDev pd, ShellGeo sg, const double2 *__restrict__ ng, int nsplit,
              double *__restrict__ partial) {
  const int i = blockIdx.x, sp = blockIdx.y;
  const int chunk = (pd.nG + nsplit - 1) / nsplit;
  const int ga = sp * chunk, gb = min(pd.nG, ga + chunk);
  double acc[3] = {0.0, 0.0, 0.0};
  for (int g = ga + threadIdx.x; g < gb; g += blockDim.x) {
    double G[3];
    gvec(pd, sg, g, G);
    const double q2 = G[0] * G[0] + G[1] * G[1] + G[2] * G[2];
    const double q = q2 > 1e-30 ? sqrt(q2) : 0.0;
    double v0, v1;
    vloc_eval(sg, q, v0, v1);
    double sn, cs;
    sincos(G[0] * sg.pos[3 * i] + G[1] * sg.pos[3 * i + 1] + G[2] * sg.pos[3 * i + 2], &sn, &cs);
    const double2 n = ng[g];
    // e^{-iGR} conj(n) = (cs - i sn)(nx - i ny) -> Im = -cs ny - sn nx
    const double im = -cs * n.y - sn * n.x;
#pragma unroll
    for (int a = 0; a < 3; ++a) acc[a] += v0 * G[a] * im;
  }
  __shared__ double red[8][3];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    double x = acc[j];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][j] = x;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double s = 0.0;
    for (int w = 0; w < (blockDim.x >> 5); ++w) s += red[w][threadIdx.x];
    partial[((size_t)i * nsplit + sp) * 3 + threadIdx.x] = s;
  }
}

// assemble density-gradient output
// out: [0] E_loc, [1] E_H, [2..4] 0, [5..5+3nat) dE_loc/dR, then deps_H (9), deps_loc (9)
__global__ void k_density_grad_final(const double *__restrict__ hsum, const double *__restrict__ lsum,
                                     const double *__restrict__ fpart, int nat, int nsplit, double omega,
                                     double *__restrict__ out) {
  const double E_H = 0.5 * omega * hsum[0];
  const double E_loc = lsum[0];
  for (int t = threadIdx.x; t < 5 + 3 * nat + 18; t += blockDim.x) {
    double v = 0.0;
    if (t == 0) v = E_loc;
    else if (t == 1) v = E_H;
    else if (t < 5) v = 0.0;
    else if (t < 5 + 3 * nat) {
      const int i = (t - 5) / 3, a = (t - 5) % 3;
      for (int s = 0; s < nsplit; ++s) v += fpart[((size_t)i * nsplit + s) * 3 + a];
    } else if (t < 5 + 3 * nat + 9) {
      const int ab = t - 5 - 3 * nat;
      v = omega * hsum[1 + ab] - ((ab % 4 == 0) ? E_H : 0.0);
    } else {
      const int ab = t - 5 - 3 * nat - 9;
      v = lsum[1 + ab] - ((ab % 4 == 0) ? E_loc : 0.0);
    }
    out[t] = v;
  }
}

// Kerker filter on the full box: d(G) *= alpha q^2 / (q^2 + gg0), 0 at q = 0 (scf.py:215-223)
__global__ void k_kerker_g(PlanDev pd, ShellGeo sg, double alpha, double gg0, double2 *__restrict__ dg) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= pd.nG) return;
  double G[3];
  gvec(pd, sg, g, G);
  const double q2 = G[0] * G[0] + G[1] * G[1] + G[2] * G[2];
  const double f = q2 > 1e-12 ? alpha * q2 / (q2 + gg0) : 0.0;
  const double2 v = dg[g];
  dg[g] = make_double2(v.x * f, v.y * f);
}

inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

inline addft_status make_shell(ShellGeo &sg, const double *bvec, double omega, int nat, const double *pos,
                               const addft_psp *psp) {
  ADDFT_REQUIRE(nat >= 0 && nat <= kMaxAtomsP, ADDFT_UNSUPPORTED, "nat = %d exceeds %d", nat, kMaxAtomsP);
  ADDFT_REQUIRE(omega > 0 && bvec, ADDFT_INVALID_ARG, "bad cell");
  memset(&sg, 0, sizeof(sg));
  for (int i = 0; i < 9; ++i) sg.B[i] = bvec[i];
  sg.omega = omega;
  sg.nat = nat;
  for (int i = 0; i < 3 * nat; ++i) sg.pos[i] = pos[i];
  if (psp) {
    ADDFT_REQUIRE(psp->kind == 0 || (psp->kind == 1 && psp->tab && psp->nq >= 2 && psp->dq > 0),
                  ADDFT_INVALID_ARG, "psp: kind 0, or kind 1 with tab, nq >= 2, dq > 0");
    sg.vamp = psp->vloc_amp;
    sg.vsig = psp->vloc_sigma;
    sg.kind = psp->kind;
    sg.nrad = psp->nrad;
    sg.rt.tab = psp->tab;
    sg.rt.nq = psp->nq;
    sg.rt.dq = psp->dq;
    sg.g0 = psp->vloc_g0;
    sg.zval = psp->zval;
  }
  return ADDFT_OK;
}

// n(G) = fftn(rho)/N gathered on the plan's shell (f64), W = slab scratch
inline addft_status density_to_shell(const PlanDev &pd, const double *rho, double2 *ng, void *W,
                                     cudaStream_t st) {
  const long N = (long)pd.n1 * pd.n2 * pd.n3;
  XArgs<double> a = xargs_default<double>(W);
  a.rin = rho;
  a.rin_is_real = 1;
  a.rstride = N;
  a.rscale = 1.0;
  ADDFT_TRY((launch_xline<double, XM_FROM_REAL>(pd, 1, a, st)));
  return launch_plane_fwd<double, PM_PLAIN>(pd, 1, (const double2 *)W, 1.0 / (double)N, ng, pd.nG,
                                            nullptr, nullptr, 1, 0, st);
}

// v(r) = Re(N ifftn(scatter(vg)))
inline addft_status shell_to_real(const PlanDev &pd, const double2 *vg, double *v, void *W, cudaStream_t st) {
  const long N = (long)pd.n1 * pd.n2 * pd.n3;
  ADDFT_TRY(launch_plane_inv<double>(pd, 1, vg, pd.nG, 1.0, (double2 *)W, st));
  XArgs<double> a = xargs_default<double>(W);
  a.rout = v;
  a.rstride = N;
  a.rscale = 1.0;
  return launch_xline<double, XM_TO_REAL_RE>(pd, 1, a, st);
}

inline size_t slab_bytes(const PlanDev &pd) { return (size_t)pd.np * pd.n2 * pd.n3 * sizeof(double2); }

}  // namespace addft

using namespace addft;

extern "C" {

addft_status addft_xc_lda(int n, const double *rho, const double *rho_dc, const double *v_loc,
                          const double *v_h, double *v_xc, double *v_eff, double *sums, void *work,
                          size_t work_bytes, void *stream) {
  ADDFT_REQUIRE(n >= 0 && rho && sums && work && work_bytes >= 3 * kRedBlocks * sizeof(double),
                ADDFT_INVALID_ARG, "xc_lda: bad arguments (work >= %zu B)", 3 * kRedBlocks * sizeof(double));
  cudaStream_t st = as_stream(stream);
  double *part = (double *)work;
  k_xc_lda<<<kRedBlocks, kRedThreads, 0, st>>>(n, rho, rho_dc, v_loc, v_h, v_xc, v_eff, part);
  ADDFT_TRY(check_launch("k_xc_lda"));
  return finalize_sums(part, 3, kRedBlocks, sums, false, st);
}

addft_status addft_xc_lda_vjp(int n, const double *rho, const double *g, double *out, void *stream) {
  ADDFT_REQUIRE(n >= 0 && (n == 0 || (rho && g && out)), ADDFT_INVALID_ARG, "xc_lda_vjp: bad arguments");
  if (n == 0) return ADDFT_OK;
  k_xc_vjp<<<std::min((n + 255) / 256, 1216), 256, 0, as_stream(stream)>>>(n, rho, g, out);
  return check_launch("k_xc_vjp");
}

addft_status addft_hartree(addft_plan plan, const double *bvec, double omega, const double *rho, double *v_h,
                           double *e_h, void *work, size_t work_bytes, void *stream) {
  ADDFT_REQUIRE(plan && bvec && rho && omega > 0, ADDFT_INVALID_ARG, "hartree: bad arguments");
  const PlanDev &pd = plan->dev;
  cudaStream_t st = as_stream(stream);
  ShellGeo sg;
  ADDFT_TRY(make_shell(sg, bvec, omega, 0, nullptr, nullptr));
  const size_t o_part = 0, o_sum = al256(10 * kRedBlocks * sizeof(double));
  const size_t o_ng = o_sum + al256(16 * sizeof(double));
  const size_t o_vg = o_ng + al256(pd.nG * sizeof(double2));
  const size_t o_w = o_vg + al256(pd.nG * sizeof(double2));
  ADDFT_REQUIRE(work && work_bytes >= o_w + slab_bytes(pd), ADDFT_INVALID_ARG,
                "hartree: work needs %zu B", o_w + slab_bytes(pd));
  char *w = (char *)work;
  double2 *ng = (double2 *)(w + o_ng), *vg = (double2 *)(w + o_vg);
  ADDFT_TRY(density_to_shell(pd, rho, ng, w + o_w, st));
  k_hartree_g<<<kRedBlocks, kRedThreads, 0, st>>>(pd, sg, ng, vg, (double *)(w + o_part));
  ADDFT_TRY(check_launch("k_hartree_g"));
  ADDFT_TRY(finalize_sums((double *)(w + o_part), 10, kRedBlocks, (double *)(w + o_sum), false, st));
  k_hartree_final<<<1, 32, 0, st>>>((double *)(w + o_sum), omega, e_h, nullptr);
  ADDFT_TRY(check_launch("k_hartree_final"));
  if (v_h) ADDFT_TRY(shell_to_real(pd, vg, v_h, w + o_w, st));
  return ADDFT_OK;
}

size_t addft_hartree_work_bytes(addft_plan plan) {
  if (!plan) return 0;
  const PlanDev &pd = plan->dev;
  return al256(10 * kRedBlocks * sizeof(double)) + al256(16 * sizeof(double)) + 2 * al256(pd.nG * sizeof(double2)) +
         slab_bytes(pd);
}

addft_status addft_local_potential(addft_plan rho_plan, const double *bvec, double omega, int nat,
                                   const double *pos, const addft_psp *psp, double *v_loc, void *work,
                                   size_t work_bytes, void *stream) {
  ADDFT_REQUIRE(rho_plan && bvec && psp && v_loc && (nat == 0 || pos), ADDFT_INVALID_ARG,
                "local_potential: bad arguments");
  const PlanDev &pd = rho_plan->dev;
  cudaStream_t st = as_stream(stream);
  ShellGeo sg;
  ADDFT_TRY(make_shell(sg, bvec, omega, nat, pos, psp));
  const size_t o_vg = 0, o_w = al256(pd.nG * sizeof(double2));
  ADDFT_REQUIRE(work && work_bytes >= o_w + slab_bytes(pd), ADDFT_INVALID_ARG,
                "local_potential: work needs %zu B", o_w + slab_bytes(pd));
  char *w = (char *)work;
  k_vloc_g<<<(pd.nG + 255) / 256, 256, 0, st>>>(pd, sg, (double2 *)(w + o_vg));
  ADDFT_TRY(check_launch("k_vloc_g"));
  return shell_to_real(pd, (const double2 *)(w + o_vg), v_loc, w + o_w, st);
}

addft_status addft_kerker(addft_plan full_plan, const double *bvec, const double *in, double alpha, double gg0,
                          double *out, void *work, size_t work_bytes, void *stream) {
  ADDFT_REQUIRE(full_plan && bvec && in && out, ADDFT_INVALID_ARG, "kerker: bad arguments");
  const PlanDev &pd = full_plan->dev;
  const long N = (long)pd.n1 * pd.n2 * pd.n3;
  ADDFT_REQUIRE(pd.nG == N, ADDFT_INVALID_ARG, "kerker: plan must cover the full box (nG = %ld)", N);
  cudaStream_t st = as_stream(stream);
  ShellGeo sg;
  ADDFT_TRY(make_shell(sg, bvec, 1.0, 0, nullptr, nullptr));
  const size_t o_g = 0, o_w = al256(pd.nG * sizeof(double2));
  ADDFT_REQUIRE(work && work_bytes >= o_w + slab_bytes(pd), ADDFT_INVALID_ARG, "kerker: work needs %zu B",
                o_w + slab_bytes(pd));
  char *w = (char *)work;
  ADDFT_TRY(density_to_shell(pd, in, (double2 *)(w + o_g), w + o_w, st));
  k_kerker_g<<<(pd.nG + 255) / 256, 256, 0, st>>>(pd, sg, alpha, gg0, (double2 *)(w + o_g));
  ADDFT_TRY(check_launch("k_kerker_g"));
  return shell_to_real(pd, (const double2 *)(w + o_g), out, w + o_w, st);
}

size_t addft_kerker_work_bytes(addft_plan full_plan) {
  if (!full_plan) return 0;
  return al256(full_plan->dev.nG * sizeof(double2)) + slab_bytes(full_plan->dev);
}

size_t addft_local_potential_work_bytes(addft_plan rho_plan) {
  if (!rho_plan) return 0;
  return al256(rho_plan->dev.nG * sizeof(double2)) + slab_bytes(rho_plan->dev);
}

addft_status addft_density_gradients(addft_plan wfc_plan, addft_plan rho_plan, const double *bvec, double omega,
                                     int nat, const double *pos, const addft_psp *psp, const double *rho,
                                     double *out, void *work, size_t work_bytes, void *stream) {
  ADDFT_REQUIRE(wfc_plan && rho_plan && bvec && psp && rho && out && (nat == 0 || pos), ADDFT_INVALID_ARG,
                "density_gradients: bad arguments");
  const PlanDev &pw = wfc_plan->dev, &pr = rho_plan->dev;
  ADDFT_REQUIRE(pw.n1 == pr.n1 && pw.n2 == pr.n2 && pw.n3 == pr.n3, ADDFT_INVALID_ARG,
                "density_gradients: plans on different boxes");
  cudaStream_t st = as_stream(stream);
  ShellGeo sg;
  ADDFT_TRY(make_shell(sg, bvec, omega, nat, pos, psp));
  const int nsplit = 16;
  size_t off = 0;
  auto take = [&](size_t b) { size_t o = off; off += al256(b); return o; };
  const size_t o_hp = take(10 * kRedBlocks * sizeof(double));
  const size_t o_lp = take(10 * kRedBlocks * sizeof(double));
  const size_t o_hs = take(10 * sizeof(double));
  const size_t o_ls = take(10 * sizeof(double));
  const size_t o_fp = take((size_t)(nat > 0 ? nat : 1) * nsplit * 3 * sizeof(double));
  const size_t o_nw = take(pw.nG * sizeof(double2));
  const size_t o_nr = take(pr.nG * sizeof(double2));
  const size_t o_w = take(std::max(slab_bytes(pw), slab_bytes(pr)));
  ADDFT_REQUIRE(work && work_bytes >= off, ADDFT_INVALID_ARG, "density_gradients: work needs %zu B", off);
  char *w = (char *)work;
  ADDFT_TRY(density_to_shell(pw, rho, (double2 *)(w + o_nw), w + o_w, st));
  ADDFT_TRY(density_to_shell(pr, rho, (double2 *)(w + o_nr), w + o_w, st));
  k_hartree_g<<<kRedBlocks, kRedThreads, 0, st>>>(pw, sg, (const double2 *)(w + o_nw), nullptr,
                                                 (double *)(w + o_hp));
  ADDFT_TRY(check_launch("k_hartree_g"));
  ADDFT_TRY(finalize_sums((double *)(w + o_hp), 10, kRedBlocks, (double *)(w + o_hs), false, st));
  k_local_sums<<<kRedBlocks, kRedThreads, 0, st>>>(pr, sg, (const double2 *)(w + o_nr), (double *)(w + o_lp));
  ADDFT_TRY(check_launch("k_local_sums"));
  ADDFT_TRY(finalize_sums((double *)(w + o_lp), 10, kRedBlocks, (double *)(w + o_ls), false, st));
  if (nat > 0) {
    k_local_force<<<dim3(nat, nsplit), kRedThreads, 0, st>>>(pr, sg, (const double2 *)(w + o_nr), nsplit,
                                                            (double *)(w + o_fp));
    ADDFT_TRY(check_launch("k_local_force"));
  }
  k_density_grad_final<<<1, 128, 0, st>>>((const double *)(w + o_hs), (const double *)(w + o_ls),
                                          (const double *)(w + o_fp), nat, nsplit, omega, out);
  return check_launch("k_density_grad_final");
}

size_t addft_density_gradients_work_bytes(addft_plan wfc_plan, addft_plan rho_plan, int nat) {
  if (!wfc_plan || !rho_plan) return 0;
  const PlanDev &pw = wfc_plan->dev, &pr = rho_plan->dev;
  size_t s = 2 * al256(10 * kRedBlocks * sizeof(double)) + 2 * al256(10 * sizeof(double));
  s += al256((size_t)(nat > 0 ? nat : 1) * 16 * 3 * sizeof(double));
  s += al256(pw.nG * sizeof(double2)) + al256(pr.nG * sizeof(double2));
  s += al256(std::max(slab_bytes(pw), slab_bytes(pr)));
  return s;
}

}  // extern "C"
