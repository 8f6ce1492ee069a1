// Nonlocal pseudopotential on GB300: projector tables, the two projector
// contractions of V_NL psi, the nonlocal energy and its envelope gradients,
// and the full matrix-free H psi entry point.
//
// Reference: src/addft/physics/nonlocal_op.py:25-82 (dion_full, projectors,
// becp, vnl_apply, nonlocal_energy), ylm.py:8-26, psp.py:122-128, and
// src/addft/ops/hpsi.py:35-50.
#include "radial.cuh"
#include "transforms.cuh"

namespace addft {

constexpr int kMaxAtoms = 256;
constexpr int kMaxK = 64;
constexpr int kMaxNh = 16;

// Kernel-parameter view of the geometry + pseudopotential (no device allocation).
struct GeoParams {
  double B[9];                 // reciprocal rows
  double inv_sqrt_omega;
  int nat, nh, nk;
  double pos[kMaxAtoms * 3];
  double kpt[kMaxK * 3];
  // per projector channel c in [0, nh): radial index, l, m
  int ch_rad[kMaxNh], ch_l[kMaxNh], ch_m[kMaxNh];
  double w[4], b[4];
  int kind;            // 0 analytic, 1 tabulated (rt)
  RadialTab rt;
};

inline addft_status make_geo(GeoParams &g, const double *bvec, double omega, int nk,
                             const double *kpts, int nat, const double *pos, const addft_psp *psp) {
  ADDFT_REQUIRE(nat >= 0 && nat <= kMaxAtoms, ADDFT_UNSUPPORTED, "nat = %d exceeds %d", nat, kMaxAtoms);
  ADDFT_REQUIRE(nk >= 1 && nk <= kMaxK, ADDFT_UNSUPPORTED, "nk = %d exceeds %d", nk, kMaxK);
  ADDFT_REQUIRE(omega > 0, ADDFT_INVALID_ARG, "omega must be > 0");
  memset(&g, 0, sizeof(g));
  for (int i = 0; i < 9; ++i) g.B[i] = bvec[i];
  g.inv_sqrt_omega = 1.0 / sqrt(omega);
  g.nat = nat;
  g.nk = nk;
  for (int i = 0; i < 3 * nat; ++i) g.pos[i] = pos[i];
  for (int i = 0; i < 3 * nk; ++i) g.kpt[i] = kpts ? kpts[i] : 0.0;
  g.nh = 0;
  if (psp) {
    ADDFT_REQUIRE(psp->nrad >= 0 && psp->nrad <= 4, ADDFT_UNSUPPORTED, "psp nrad > 4");
    ADDFT_REQUIRE(psp->kind == 0 || psp->kind == 1, ADDFT_INVALID_ARG, "psp kind must be 0 or 1");
    if (psp->kind == 1)
      ADDFT_REQUIRE(psp->tab != nullptr && psp->nq >= 2 && psp->dq > 0, ADDFT_INVALID_ARG,
                    "tabulated psp needs tab, nq >= 2, dq > 0");
    g.kind = psp->kind;
    g.rt.tab = psp->tab;
    g.rt.nq = psp->nq;
    g.rt.dq = psp->dq;
    for (int ib = 0; ib < psp->nrad; ++ib) {
      ADDFT_REQUIRE(psp->l[ib] >= 0 && psp->l[ib] <= 2, ADDFT_UNSUPPORTED,
                    "projector l = %d not supported (l <= 2)", psp->l[ib]);
      g.w[ib] = psp->w[ib];
      g.b[ib] = psp->b[ib];
      for (int m = 0; m < 2 * psp->l[ib] + 1; ++m) {
        ADDFT_REQUIRE(g.nh < kMaxNh, ADDFT_UNSUPPORTED, "too many projector channels");
        g.ch_rad[g.nh] = ib;
        g.ch_l[g.nh] = psp->l[ib];
        g.ch_m[g.nh] = m;
        ++g.nh;
      }
    }
  }
  return ADDFT_OK;
}

// beta~(q), d beta~/dq, Y_lm, grad Y_lm, for one channel at v = k+G.
struct ProjEval {
  double beta;       // beta~(q) Y_lm  (phase-free)
  double grad[3];    // d(beta~ Y)/dv
};

__device__ __forceinline__ ProjEval proj_eval(const GeoParams &gp, int c, double vx, double vy,
                                              double vz) {
  const double r2 = vx * vx + vy * vy + vz * vz;
  const bool pos = r2 > 1e-30;
  const double q = pos ? sqrt(r2) : 0.0;        // safe_norm (basis.py:170-179)
  const double rs = pos ? q : 1.0;
  const int ib = gp.ch_rad[c], l = gp.ch_l[c], m = gp.ch_m[c];
  double bq, dbq;
  if (gp.kind == 1) {
    radial_eval(gp.rt, ib, q, bq, dbq);                           // psp.py:130-138
  } else {
    // beta(q) = w q^l exp(-(q b)^2/2), q clamped at 1e-12 (psp.py:122-128);
    // d beta/dq = w exp(..) (l q^(l-1) - q^(l+1) b^2), zero below the clamp
    const double w = gp.w[ib], bb = gp.b[ib];
    const double qq = fmax(q, 1e-12);
    const double e = exp(-0.5 * (qq * bb) * (qq * bb));
    const double qlm1 = l == 0 ? 0.0 : (l == 1 ? 1.0 : qq);       // q^(l-1) for l >= 1
    const double ql = l == 0 ? 1.0 : qlm1 * qq;
    bq = w * ql * e;
    dbq = (q > 1e-12) ? w * e * ((double)l * qlm1 - ql * qq * bb * bb) : 0.0;
  }
  ProjEval out;
  const double c0 = 0.28209479177387814347;   // 1/sqrt(4 pi)
  const double c1 = 0.48860251190291992159;   // sqrt(3/(4 pi))
  const double u[3] = {pos ? vx / rs : 0.0, pos ? vy / rs : 0.0, pos ? vz / rs : 0.0};
  double Y, dY[3] = {0.0, 0.0, 0.0};
  if (l == 0) {
    Y = c0;
  } else if (l == 1) {
    // m = 0: +z, 1: -x, 2: -y  (ABACUS order, ylm.py:15-25)
    const int comp = m == 0 ? 2 : (m == 1 ? 0 : 1);
    const double sgn = m == 0 ? 1.0 : -1.0;
    Y = sgn * c1 * (comp == 0 ? vx : (comp == 1 ? vy : vz)) / rs;
    if (pos) {
      for (int a = 0; a < 3; ++a) dY[a] = sgn * c1 * ((a == comp ? 1.0 : 0.0) - u[comp] * u[a]) / rs;
    }
  } else {
    // l = 2, m = 0, +1, -1, +2, -2 (ylm.py:18-25): Y = P(v) / r^2 with P a quadratic
    // form, dY/dv = grad P / r^2 - 2 P v / r^4
    const double c20 = 0.31539156525252000603;   // sqrt(5/(4 pi)) / 2
    const double c21 = 1.09254843059207907054;   // sqrt(15/(4 pi))
    const double c22 = 0.54627421529603953527;   // sqrt(15/(16 pi))
    const double r2 = rs * rs;
    double P, dP[3];
    switch (m) {
      case 0: P = c20 * (2.0 * vz * vz - vx * vx - vy * vy);
              dP[0] = -2.0 * c20 * vx; dP[1] = -2.0 * c20 * vy; dP[2] = 4.0 * c20 * vz; break;
      case 1: P = -c21 * vx * vz; dP[0] = -c21 * vz; dP[1] = 0.0; dP[2] = -c21 * vx; break;
      case 2: P = -c21 * vy * vz; dP[0] = 0.0; dP[1] = -c21 * vz; dP[2] = -c21 * vy; break;
      case 3: P = c22 * (vx * vx - vy * vy); dP[0] = 2.0 * c22 * vx; dP[1] = -2.0 * c22 * vy; dP[2] = 0.0; break;
      default: P = c21 * vx * vy; dP[0] = c21 * vy; dP[1] = c21 * vx; dP[2] = 0.0; break;
    }
    Y = P / r2;
    if (pos) {
      const double v3[3] = {vx, vy, vz};
      for (int a = 0; a < 3; ++a) dY[a] = dP[a] / r2 - 2.0 * P * v3[a] / (r2 * r2);
    }
  }
  out.beta = bq * Y;
  for (int a = 0; a < 3; ++a) out.grad[a] = dbq * u[a] * Y + bq * dY[a];
  return out;
}

// proj[k][p][g], p = atom * nh + channel
template <typename R>
__global__ void k_projectors(PlanDev pd, GeoParams gp, typename Cx<R>::T *__restrict__ proj) {
  using C = typename Cx<R>::T;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int p = blockIdx.y;
  const int k = blockIdx.z;
  if (g >= pd.nG) return;
  const int i = p / gp.nh, c = p - i * gp.nh;
  const double m1 = pd.miller[3 * g], m2 = pd.miller[3 * g + 1], m3 = pd.miller[3 * g + 2];
  const double vx = m1 * gp.B[0] + m2 * gp.B[3] + m3 * gp.B[6] + gp.kpt[3 * k];
  const double vy = m1 * gp.B[1] + m2 * gp.B[4] + m3 * gp.B[7] + gp.kpt[3 * k + 1];
  const double vz = m1 * gp.B[2] + m2 * gp.B[5] + m3 * gp.B[8] + gp.kpt[3 * k + 2];
  const ProjEval pe = proj_eval(gp, c, vx, vy, vz);
  const double arg = vx * gp.pos[3 * i] + vy * gp.pos[3 * i + 1] + vz * gp.pos[3 * i + 2];
  double sn, cs;
  sincos(arg, &sn, &cs);
  const double a = pe.beta * gp.inv_sqrt_omega;
  C out;
  out.x = (R)(a * cs);
  out.y = (R)(-a * sn);   // e^{-i v.R}
  proj[((size_t)k * gridDim.y + p) * pd.nG + g] = out;
}

// kinetic diagonal 1/2 |k+G|^2
template <typename R>
__global__ void k_kinetic(PlanDev pd, GeoParams gp, R *__restrict__ kin) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  if (g >= pd.nG) return;
  const double m1 = pd.miller[3 * g], m2 = pd.miller[3 * g + 1], m3 = pd.miller[3 * g + 2];
  const double vx = m1 * gp.B[0] + m2 * gp.B[3] + m3 * gp.B[6] + gp.kpt[3 * k];
  const double vy = m1 * gp.B[1] + m2 * gp.B[4] + m3 * gp.B[7] + gp.kpt[3 * k + 1];
  const double vz = m1 * gp.B[2] + m2 * gp.B[5] + m3 * gp.B[8] + gp.kpt[3 * k + 2];
  kin[(size_t)k * pd.nG + g] = (R)(0.5 * (vx * vx + vy * vy + vz * vz));
}

// ---------------------------------------------------------------------------
// becp[k][p][b] = sum_g conj(proj[k][p][g]) psi[k][b][g]
//   CTA tile 32 (p) x 64 (b) over one G chunk (split-K); 256 threads, each
//   2 p x 4 b outputs (p = tp + 16 i, b = tb + 16 j: conflict-free smem reads)
// ---------------------------------------------------------------------------
constexpr int kBP = 32, kBB = 64, kBK = 16;

template <typename R>
__global__ void __launch_bounds__(256)
k_becp(const typename Cx<R>::T *__restrict__ proj, const typename Cx<R>::T *__restrict__ psi,
       int nb, int nG, int nproj, int nsplit, int gchunk, typename Cx<R>::T *__restrict__ out) {
  using C = typename Cx<R>::T;
  __shared__ __align__(16) C sP[2][kBP][kBK + 1];
  __shared__ __align__(16) C sX[2][kBB][kBK + 1];
  const int p0 = blockIdx.y * kBP, b0 = blockIdx.x * kBB;
  const int nkz = gridDim.z / nsplit;
  const int k = blockIdx.z / nsplit, sp = blockIdx.z - k * nsplit;
  const int ga = sp * gchunk, gb = min(nG, ga + gchunk);
  const C *Pk = proj + (size_t)k * nproj * nG;
  const C *Xk = psi + (size_t)k * nb * nG;
  const int tb = threadIdx.x & 15, tp = threadIdx.x >> 4;
  C acc[2][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = czero<C>();
  // 2-stage cp.async pipeline over G steps of kBK
  auto issue = [&](int g0, int buf) {
    for (int i = threadIdx.x; i < (kBP + kBB) * kBK; i += 256) {
      const int r = i / kBK, c = i - r * kBK;
      const int g = g0 + c;
      if (r < kBP) {
        const bool ok = p0 + r < nproj && g < gb;
        cp_async_el(&sP[buf][r][c], ok ? Pk + (size_t)(p0 + r) * nG + g : Pk, ok);
      } else {
        const int rr = r - kBP;
        const bool ok = b0 + rr < nb && g < gb;
        cp_async_el(&sX[buf][rr][c], ok ? Xk + (size_t)(b0 + rr) * nG + g : Xk, ok);
      }
    }
    cp_async_commit();
  };
  int buf = 0;
  if (ga < gb) issue(ga, 0);
  for (int g0 = ga; g0 < gb; g0 += kBK) {
    if (g0 + kBK < gb) {
      issue(g0 + kBK, buf ^ 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
#pragma unroll 4
    for (int c = 0; c < kBK; ++c) {
      C av[2], xv[4];
#pragma unroll
      for (int i = 0; i < 2; ++i) av[i] = sP[buf][tp + 16 * i][c];
#pragma unroll
      for (int j = 0; j < 4; ++j) xv[j] = sX[buf][tb + 16 * j][c];
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          // conj(a) * x
          acc[i][j].x += av[i].x * xv[j].x + av[i].y * xv[j].y;
          acc[i][j].y += av[i].x * xv[j].y - av[i].y * xv[j].x;
        }
    }
    __syncthreads();
    buf ^= 1;
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int p = p0 + tp + 16 * i;
    if (p >= nproj) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int bb = b0 + tb + 16 * j;
      if (bb < nb) out[(((size_t)sp * nkz + k) * nproj + p) * nb + bb] = acc[i][j];
    }
  }
}

// Deterministic two-pass sum over splits, out[i] = sum_s part[s][i]:
//   pass 1 (grid: outputs / 256 x split groups) sums groups of kSplitGroup splits,
//   pass 2 (8 lanes per output) sums the groups: lane l takes groups l, l + 8, ...,
//   then a fixed xor-shuffle tree; every load is coalesced along i.
constexpr int kSplitGroup = 16;
constexpr int kSumLanes = 8;

template <typename C>
__global__ void __launch_bounds__(256) k_sum_splits1(const C *__restrict__ part, int nsplit, size_t n,
                                                     C *__restrict__ tmp) {
  const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int j0 = blockIdx.y * kSplitGroup, j1 = min(nsplit, j0 + kSplitGroup);
  C s = czero<C>();
  for (int j = j0; j < j1; ++j) s = cadd(s, part[(size_t)j * n + i]);
  tmp[(size_t)blockIdx.y * n + i] = s;
}

template <typename C>
__global__ void __launch_bounds__(256) k_sum_splits2(const C *__restrict__ tmp, int ngroup, size_t n,
                                                     C *__restrict__ out) {
  const size_t i = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) / kSumLanes;
  const int l = threadIdx.x % kSumLanes;
  C s = czero<C>();
  if (i < n)
    for (int g = l; g < ngroup; g += kSumLanes) s = cadd(s, tmp[(size_t)g * n + i]);
#pragma unroll
  for (int o = kSumLanes / 2; o > 0; o >>= 1) {
    s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
    s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
  }
  if (i < n && l == 0) out[i] = s;
}

inline int split_groups(int ns) { return (ns + kSplitGroup - 1) / kSplitGroup; }

// DB[k][p][b] = sum_q D[p][q] becp[k][q][b]   (optionally scaled by wocc[k][b])
template <typename R>
__global__ void k_dbecp(const R *__restrict__ D, const typename Cx<R>::T *__restrict__ becp, int nk,
                        int nproj, int nb, const double *__restrict__ wocc,
                        typename Cx<R>::T *__restrict__ out) {
  using C = typename Cx<R>::T;
  const size_t n = (size_t)nk * nproj * nb;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const int b = (int)(t % nb);
    const int p = (int)((t / nb) % nproj);
    const int k = (int)(t / ((size_t)nb * nproj));
    const C *Bk = becp + (size_t)k * nproj * nb;
    C s = czero<C>();
    for (int q = 0; q < nproj; ++q) {
      const R d = D[(size_t)p * nproj + q];
      if (d != (R)0) s = cadd(s, cscale(Bk[(size_t)q * nb + b], d));
    }
    if (wocc) s = cscale(s, (R)wocc[(size_t)k * nb + b]);
    out[t] = s;
  }
}

// out[k][i][g] (+)= sum_j X[k][j, i] op(A[k][j][g]);  X element (j, i) at j*xs_j + i*xs_i
// CTA tile: TG g x 32 i, j in steps of 16 (cp.async double buffer); 256 threads;
// TG = 128: each thread 4 g (lane + 32 u) x 4 i (warp * 4 + v); TG = 32: 1 g x 4 i.
constexpr int kAI = 32, kAJ = 16;

template <typename R, bool CONJ_A, bool ACCUM, int TG>
__global__ void __launch_bounds__(256)
k_apply(const typename Cx<R>::T *__restrict__ Xm, int xs_j, int xs_i, size_t xs_k,
        const typename Cx<R>::T *__restrict__ A, size_t as_k, int nj, int ni, int nG,
        typename Cx<R>::T *__restrict__ out, size_t os_k) {
  using C = typename Cx<R>::T;
  constexpr int U = TG / 32;
  __shared__ __align__(16) C sA[2][kAJ][TG];
  __shared__ __align__(16) C sX[2][kAJ][kAI];
  const int g0 = blockIdx.x * TG, i0 = blockIdx.y * kAI, k = blockIdx.z;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const C *Ak = A + (size_t)k * as_k;
  const C *Xk = Xm + (size_t)k * xs_k;
  C acc[U][4];
#pragma unroll
  for (int u = 0; u < U; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = czero<C>();
  auto issue = [&](int j0, int buf) {
    for (int t = threadIdx.x; t < kAJ * TG; t += 256) {
      const int r = t / TG, c = t - r * TG;
      const bool ok = j0 + r < nj && g0 + c < nG;
      cp_async_el(&sA[buf][r][c], ok ? Ak + (size_t)(j0 + r) * nG + g0 + c : Ak, ok);
    }
    for (int t = threadIdx.x; t < kAJ * kAI; t += 256) {
      const int r = t / kAI, c = t - r * kAI;
      const bool ok = j0 + r < nj && i0 + c < ni;
      cp_async_el(&sX[buf][r][c], ok ? Xk + (size_t)(j0 + r) * xs_j + (size_t)(i0 + c) * xs_i : Xk, ok);
    }
    cp_async_commit();
  };
  int buf = 0;
  issue(0, 0);
  for (int j0 = 0; j0 < nj; j0 += kAJ) {
    if (j0 + kAJ < nj) {
      issue(j0 + kAJ, buf ^ 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
#pragma unroll 4
    for (int r = 0; r < kAJ; ++r) {
      C av[U], xv[4];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        av[u] = sA[buf][r][lane + 32 * u];
        if (CONJ_A) av[u].y = -av[u].y;
      }
#pragma unroll
      for (int v = 0; v < 4; ++v) xv[v] = sX[buf][r][w * 4 + v];
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          acc[u][v].x += av[u].x * xv[v].x - av[u].y * xv[v].y;
          acc[u][v].y += av[u].x * xv[v].y + av[u].y * xv[v].x;
        }
    }
    __syncthreads();
    buf ^= 1;
  }
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const int i = i0 + w * 4 + v;
    if (i >= ni) continue;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int g = g0 + lane + 32 * u;
      if (g < nG) {
        C *o = out + (size_t)k * os_k + (size_t)i * nG + g;
        *o = ACCUM ? cadd(*o, acc[u][v]) : acc[u][v];
      }
    }
  }
}

// E_NL partial per (k, b): wocc * Re(B^H D B); writes partial[k*nb + b]
template <typename R>
__global__ void k_nl_energy(const typename Cx<R>::T *__restrict__ becp,
                            const typename Cx<R>::T *__restrict__ dbecp, int nk, int nproj, int nb,
                            const double *__restrict__ wocc, double *__restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nk * nb) return;
  const int k = t / nb, b = t - k * nb;
  double s = 0.0;
  for (int p = 0; p < nproj; ++p) {
    const auto x = becp[((size_t)k * nproj + p) * nb + b];
    const auto y = dbecp[((size_t)k * nproj + p) * nb + b];
    s += (double)x.x * (double)y.x + (double)x.y * (double)y.y;
  }
  out[t] = wocc[t] * s;
}

// Envelope gradients of E_NL from Y[k][p][g] = sum_b wocc (D B)[p][b] conj(psi_b(g)):
//   dE/dR_{i,a} = sum_{p in i} sum_g 2 v_a Im(beta_p y)
//   dE/deps_ab  = -2 sum_p sum_g Re(Q_pa y) G_b            (the -E_NL delta_ab term is added later)
// one CTA per (k, p); partial[(k*P + p)*12 + j]
template <typename R>
__global__ void __launch_bounds__(256)
k_nl_grad(PlanDev pd, GeoParams gp, const typename Cx<R>::T *__restrict__ Y, int nproj,
          double *__restrict__ partial) {
  const int p = blockIdx.x, k = blockIdx.y;
  const int i = p / gp.nh, c = p - i * gp.nh;
  const auto *Yp = Y + ((size_t)k * nproj + p) * pd.nG;
  double acc[12];
#pragma unroll
  for (int j = 0; j < 12; ++j) acc[j] = 0.0;
  for (int g = threadIdx.x; g < pd.nG; g += blockDim.x) {
    const double m1 = pd.miller[3 * g], m2 = pd.miller[3 * g + 1], m3 = pd.miller[3 * g + 2];
    const double Gx = m1 * gp.B[0] + m2 * gp.B[3] + m3 * gp.B[6];
    const double Gy = m1 * gp.B[1] + m2 * gp.B[4] + m3 * gp.B[7];
    const double Gz = m1 * gp.B[2] + m2 * gp.B[5] + m3 * gp.B[8];
    const double v[3] = {Gx + gp.kpt[3 * k], Gy + gp.kpt[3 * k + 1], Gz + gp.kpt[3 * k + 2]};
    const double G[3] = {Gx, Gy, Gz};
    const ProjEval pe = proj_eval(gp, c, v[0], v[1], v[2]);
    const double arg = v[0] * gp.pos[3 * i] + v[1] * gp.pos[3 * i + 1] + v[2] * gp.pos[3 * i + 2];
    double sn, cs;
    sincos(arg, &sn, &cs);
    const auto yv = Yp[g];
    const double yr = yv.x, yi = yv.y;
    // phase * y = (cs - i sn)(yr + i yi)
    const double pr = (cs * yr + sn * yi) * gp.inv_sqrt_omega;
    const double pim = (cs * yi - sn * yr) * gp.inv_sqrt_omega;
    // beta y = beta~ * (phase y)
    const double im_by = pe.beta * pim;
#pragma unroll
    for (int a = 0; a < 3; ++a) acc[a] += 2.0 * v[a] * im_by;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double re_qy = pe.grad[a] * pr;
#pragma unroll
      for (int b = 0; b < 3; ++b) acc[3 + 3 * a + b] += -2.0 * re_qy * G[b];
    }
  }
  // block reduce 12 values
  __shared__ double red[8][12];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < 12; ++j) {
    double x = acc[j];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][j] = x;
  }
  __syncthreads();
  if (threadIdx.x < 12) {
    double s = 0.0;
    for (int w = 0; w < (blockDim.x >> 5); ++w) s += red[w][threadIdx.x];
    partial[((size_t)k * nproj + p) * 12 + threadIdx.x] = s;
  }
}

// out: [0] E_NL, [1..3nat] dE/dR, [1+3nat..] dE/deps (9)
__global__ void k_nl_grad_final(const double *__restrict__ epart, int nkb,
                                const double *__restrict__ gpart, int nk, int nproj, int nh,
                                int nat, double *__restrict__ out) {
  __shared__ double e_nl;
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int t = 0; t < nkb; ++t) s += epart[t];
    e_nl = s;
    out[0] = s;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < 3 * nat + 9; t += blockDim.x) {
    double s = 0.0;
    if (t < 3 * nat) {
      const int i = t / 3, a = t - 3 * i;
      for (int k = 0; k < nk; ++k)
        for (int c = 0; c < nh; ++c) s += gpart[((size_t)k * nproj + i * nh + c) * 12 + a];
    } else {
      const int ab = t - 3 * nat;
      for (int k = 0; k < nk; ++k)
        for (int p = 0; p < nproj; ++p) s += gpart[((size_t)k * nproj + p) * 12 + 3 + ab];
      if (ab == 0 || ab == 4 || ab == 8) s -= e_nl;
    }
    out[1 + t] = s;
  }
}

// kinetic stress partials: -sum wocc |psi|^2 (k+G)_a G_b
template <typename R>
__global__ void __launch_bounds__(256)
k_kin_stress(PlanDev pd, GeoParams gp, const typename Cx<R>::T *__restrict__ psi, int nb,
             const double *__restrict__ wocc, double *__restrict__ partial) {
  double acc[9];
#pragma unroll
  for (int j = 0; j < 9; ++j) acc[j] = 0.0;
  const size_t total = (size_t)gp.nk * pd.nG;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total;
       t += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(t / pd.nG), g = (int)(t - (size_t)k * pd.nG);
    double p2 = 0.0;
    for (int b = 0; b < nb; ++b) {
      const auto x = psi[((size_t)k * nb + b) * pd.nG + g];
      p2 += wocc[(size_t)k * nb + b] * ((double)x.x * x.x + (double)x.y * x.y);
    }
    const double m1 = pd.miller[3 * g], m2 = pd.miller[3 * g + 1], m3 = pd.miller[3 * g + 2];
    const double G[3] = {m1 * gp.B[0] + m2 * gp.B[3] + m3 * gp.B[6],
                         m1 * gp.B[1] + m2 * gp.B[4] + m3 * gp.B[7],
                         m1 * gp.B[2] + m2 * gp.B[5] + m3 * gp.B[8]};
    const double v[3] = {G[0] + gp.kpt[3 * k], G[1] + gp.kpt[3 * k + 1], G[2] + gp.kpt[3 * k + 2]};
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) acc[3 * a + b] -= p2 * v[a] * G[b];
  }
  block_reduce_store<9>(acc, partial);
}

// ---------------------------------------------------------------------------
// host drivers
// ---------------------------------------------------------------------------
inline int pick_nsplit(int tiles, int nG, int ctas_per_sm = 8) {
  int ns = (ctas_per_sm * 152 + tiles - 1) / tiles;
  const int maxs = (nG + 63) / 64;
  if (ns > maxs) ns = maxs;
  if (ns < 1) ns = 1;
  return ns;
}

// becp_tc.cu: split-precision TF32 tensor-core becp (FP32), same grid and partial layout as k_becp;
// proj_simt.cu: register-tiled FP32 FMA becp, same layout
addft_status launch_becp_tc(int nk, int nb, int nG, int nproj, int nsplit, int gchunk, const float2 *proj,
                            const float2 *psi, float2 *out, cudaStream_t st);
addft_status launch_becp_f32(int nk, int nb, int nG, int nproj, int nsplit, int gchunk, const float2 *proj,
                             const float2 *psi, float2 *out, cudaStream_t st);
// tc05.cu: split-TF32 becp on tcgen05 with a tensor-memory accumulator, same layout
addft_status launch_becp_tc05(int nk, int nb, int nG, int nproj, int nsplit, int gchunk, const float2 *proj,
                              const float2 *psi, float2 *out, cudaStream_t st);

// Kernel of the FP32 projector contractions, read once per process from ADDFT_BECP_TC /
// ADDFT_APPLY_TC: 0 = register-tiled FP32 FMA, 1 = split-TF32 mma.sync tensor cores,
// 2 = the generic SIMT kernels of this file, 3 = split-TF32 tcgen05 with a tensor-memory
// accumulator.  Defaults (the fastest measured on the 72^3 microbench): becp 1 (the
// tcgen05 becp has to transpose its operands through shared memory and is L1-bound),
// apply 3.
static int proj_mode(const char *var, int dflt) {
  const char *v = getenv(var);
  const int m = v ? atoi(v) : dflt;
  return m >= 0 && m <= 3 ? m : dflt;
}
static int becp_mode() {
  static const int m = proj_mode("ADDFT_BECP_TC", 1);
  return m;
}

// CTAs per SM of split-K work for the tensor-core and register-tiled becp kernels
// (ADDFT_BECP_CTAS, 1..8, read once per process; default 4).
static int becp_ctas_per_sm() {
  static const int m = [] {
    const char *v = getenv("ADDFT_BECP_CTAS");
    const int x = v ? atoi(v) : 4;
    return x >= 1 && x <= 8 ? x : 4;
  }();
  return m;
}

template <typename R>
size_t becp_work_bytes(int nk, int nb, int nG, int nproj) {
  using C = typename Cx<R>::T;
  const int tiles = ((nproj + kBP - 1) / kBP) * ((nb + kBB - 1) / kBB) * nk;
  const int ns = pick_nsplit(tiles, nG);
  return ns > 1 ? (size_t)(ns + split_groups(ns)) * nk * nproj * nb * sizeof(C) : 0;
}

template <typename R>
addft_status becp_t(int nk, int nb, int nG, int nproj, const void *proj, const void *psi, void *becp,
                    void *work, size_t bytes, cudaStream_t st) {
  using C = typename Cx<R>::T;
  const int tiles = ((nproj + kBP - 1) / kBP) * ((nb + kBB - 1) / kBB) * nk;
  const int mode = sizeof(R) == 4 ? becp_mode() : 2;
  const bool tc = mode == 1;
  // the tensor-core and register-tiled forms hold 2 / 4 CTAs per SM: 4 per SM of work keeps
  // 1-2 waves of long K chunks
  int ns = pick_nsplit(tiles, nG, mode != 2 ? becp_ctas_per_sm() : 8);
  const size_t per = (size_t)nk * nproj * nb * sizeof(C);
  // partials (ns) + pass-1 group sums (ceil(ns / kSplitGroup)) must fit the work buffer
  while (ns > 1 && (work == nullptr || bytes < per * (size_t)(ns + split_groups(ns)))) --ns;
  if (ns < 1) ns = 1;
  int gchunk = (nG + ns - 1) / ns;
  if (tc) {   // whole 32-G stages per chunk; never more partials than the work buffer holds
    gchunk = (gchunk + 31) / 32 * 32;
    ns = (nG + gchunk - 1) / gchunk;
  }
  dim3 grid((nb + kBB - 1) / kBB, (nproj + kBP - 1) / kBP, nk * ns);
  C *dst = ns > 1 ? (C *)work : (C *)becp;
  bool done = false;
  if constexpr (sizeof(R) == 4) {
    if (tc) {
      ADDFT_TRY(launch_becp_tc(nk, nb, nG, nproj, ns, gchunk, (const float2 *)proj, (const float2 *)psi,
                               (float2 *)dst, st));
      done = true;
    } else if (mode == 0) {
      ADDFT_TRY(launch_becp_f32(nk, nb, nG, nproj, ns, gchunk, (const float2 *)proj, (const float2 *)psi,
                                (float2 *)dst, st));
      done = true;
    } else if (mode == 3) {
      ADDFT_TRY(launch_becp_tc05(nk, nb, nG, nproj, ns, gchunk, (const float2 *)proj, (const float2 *)psi,
                                 (float2 *)dst, st));
      done = true;
    }
  }
  if (!done) {
    k_becp<R><<<grid, 256, 0, st>>>((const C *)proj, (const C *)psi, nb, nG, nproj, ns, gchunk, dst);
    ADDFT_TRY(check_launch("k_becp"));
  }
  if (ns > 1) {
    const size_t n = (size_t)nk * nproj * nb;
    const int ng = split_groups(ns);
    C *tmp = dst + (size_t)ns * n;
    k_sum_splits1<C><<<dim3((unsigned)((n + 255) / 256), ng), 256, 0, st>>>(dst, ns, n, tmp);
    ADDFT_TRY(check_launch("k_sum_splits1"));
    k_sum_splits2<C><<<(unsigned)((n * kSumLanes + 255) / 256), 256, 0, st>>>(tmp, ng, n, (C *)becp);
    ADDFT_TRY(check_launch("k_sum_splits2"));
  }
  return ADDFT_OK;
}

template <typename R>
addft_status dbecp_t(const void *D, const void *becp, int nk, int nproj, int nb, const double *wocc,
                     void *out, cudaStream_t st) {
  using C = typename Cx<R>::T;
  const size_t n = (size_t)nk * nproj * nb;
  k_dbecp<R><<<(int)std::min<size_t>((n + 255) / 256, 1024), 256, 0, st>>>(
      (const R *)D, (const C *)becp, nk, nproj, nb, wocc, (C *)out);
  return check_launch("k_dbecp");
}

// apply_tc.cu: split-precision TF32 tensor-core apply (FP32, no conjugation);
// proj_simt.cu: register-tiled FP32 FMA apply
addft_status launch_apply_tc(bool accum, const float2 *X, int xs_j, int xs_i, size_t xs_k, const float2 *A,
                             size_t as_k, int nk, int nj, int ni, int nG, float2 *out, size_t os_k,
                             cudaStream_t st);
addft_status launch_apply_f32(bool accum, const float2 *X, int xs_j, int xs_i, size_t xs_k, const float2 *A,
                              size_t as_k, int nk, int nj, int ni, int nG, float2 *out, size_t os_k,
                              cudaStream_t st);
// tc05.cu: split-TF32 apply on tcgen05 with a tensor-memory accumulator
addft_status launch_apply_tc05(bool accum, const float2 *X, int xs_j, int xs_i, size_t xs_k, const float2 *A,
                               size_t as_k, int nk, int nj, int ni, int nG, float2 *out, size_t os_k,
                               cudaStream_t st);

static int apply_mode() {
  static const int m = proj_mode("ADDFT_APPLY_TC", 3);
  return m;
}

template <typename R, bool CONJ_A, bool ACCUM>
addft_status apply_t(const void *X, int xs_j, int xs_i, size_t xs_k, const void *A, size_t as_k,
                     int nk, int nj, int ni, int nG, void *out, size_t os_k, cudaStream_t st) {
  using C = typename Cx<R>::T;
  if constexpr (sizeof(R) == 4 && !CONJ_A) {
    if (apply_mode() == 1)
      return launch_apply_tc(ACCUM, (const float2 *)X, xs_j, xs_i, xs_k, (const float2 *)A, as_k, nk, nj, ni, nG,
                             (float2 *)out, os_k, st);
    if (apply_mode() == 0)
      return launch_apply_f32(ACCUM, (const float2 *)X, xs_j, xs_i, xs_k, (const float2 *)A, as_k, nk, nj, ni, nG,
                              (float2 *)out, os_k, st);
    if (apply_mode() == 3)
      return launch_apply_tc05(ACCUM, (const float2 *)X, xs_j, xs_i, xs_k, (const float2 *)A, as_k, nk, nj, ni, nG,
                               (float2 *)out, os_k, st);
  }
  const long ctas128 = (long)((nG + 127) / 128) * ((ni + kAI - 1) / kAI) * nk;
  if (ctas128 >= 4 * 152) {
    dim3 grid((nG + 127) / 128, (ni + kAI - 1) / kAI, nk);
    k_apply<R, CONJ_A, ACCUM, 128><<<grid, 256, 0, st>>>((const C *)X, xs_j, xs_i, xs_k, (const C *)A, as_k, nj,
                                                         ni, nG, (C *)out, os_k);
  } else {
    dim3 grid((nG + 31) / 32, (ni + kAI - 1) / kAI, nk);
    k_apply<R, CONJ_A, ACCUM, 32><<<grid, 256, 0, st>>>((const C *)X, xs_j, xs_i, xs_k, (const C *)A, as_k, nj,
                                                        ni, nG, (C *)out, os_k);
  }
  return check_launch("k_apply");
}

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

template <typename R>
size_t nl_scratch(int nk, int nb, int nG, int nproj) {
  using C = typename Cx<R>::T;
  if (nproj == 0) return 0;
  return align256(2 * (size_t)nk * nproj * nb * sizeof(C)) + align256(becp_work_bytes<R>(nk, nb, nG, nproj));
}

// H psi with the work buffer split as [becp | D becp | becp split-K partials | local FFT scratch].
// The local part needs at least one band of FFT scratch (addft_work_bytes(plan, 1)); the split-K
// partials get what remains beyond that, up to what the default number of splits uses, and becp_t
// lowers the number of splits to fit (down to one, which needs no partials).
// The projector chain (becp, split sums, D becp) only reads psi and the beta tables and
// writes its own part of the work buffer, so it can run beside the local FFT pipeline.
// ADDFT_HPSI_OVERLAP (read once per process): 0 = one stream; 1 (default) = the chain on a
// second stream of the calling thread, forked from and joined back into the caller's stream
// with events (also inside a stream capture); 2 = the same with that stream at the highest
// priority.  72^3 microbench, 64 bands: 0.428 ms (0), 0.399 ms (1), 0.400 ms (2).
static int overlap_mode() {
  static const int m = [] {
    const char *v = getenv("ADDFT_HPSI_OVERLAP");
    const int x = v ? atoi(v) : 1;
    return x >= 0 && x <= 2 ? x : 1;
  }();
  return m;
}

// The calling thread's side stream on the current device (created on first use, kept).
static addft_status side_stream(int prio_mode, cudaStream_t *out) {
  constexpr int kDev = 64;
  static thread_local cudaStream_t side[kDev] = {};
  int dev = 0;
  ADDFT_CUDA(cudaGetDevice(&dev));
  ADDFT_REQUIRE(dev >= 0 && dev < kDev, ADDFT_UNSUPPORTED, "hpsi: device index %d >= %d", dev, kDev);
  if (side[dev] == nullptr) {
    int lo = 0, hi = 0;
    ADDFT_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    ADDFT_CUDA(cudaStreamCreateWithPriority(&side[dev], cudaStreamNonBlocking, prio_mode == 2 ? hi : lo));
  }
  *out = side[dev];
  return ADDFT_OK;
}

template <typename R>
addft_status hpsi_t(addft_plan plan, int nk, int nb, const void *psi, const void *kin, const void *v_r, int nproj,
                    const void *proj, const void *dion, void *hpsi, void *work, size_t work_bytes, cudaStream_t st,
                    bool allow_overlap) {
  using C = typename Cx<R>::T;
  const PlanDev &pd = plan->dev;
  const addft_dtype dt = sizeof(R) == 8 ? ADDFT_F64 : ADDFT_F32;
  const size_t arrays = nproj > 0 ? align256(2 * (size_t)nk * nproj * nb * sizeof(C)) : 0;
  const size_t local_min = addft_work_bytes(plan, 1, dt);
  ADDFT_REQUIRE(work && work_bytes >= arrays + local_min, ADDFT_INVALID_ARG,
                "hpsi: work buffer of %zu B too small (need >= %zu B)", work_bytes, arrays + local_min);
  size_t split = 0;
  if (nproj > 0) {
    const size_t spare = (work_bytes - arrays - local_min) & ~size_t(255);
    split = std::min(align256(becp_work_bytes<R>(nk, nb, pd.nG, nproj)), spare);
  }
  C *becp = (C *)work;
  C *db = becp + (size_t)nk * nproj * nb;
  char *bw = (char *)work + arrays;
  const size_t used = arrays + split;
  if (nproj > 0 && allow_overlap && overlap_mode() != 0) {
    cudaStream_t side = nullptr;
    ADDFT_TRY(side_stream(overlap_mode(), &side));
    cudaEvent_t fork = nullptr, join = nullptr;
    ADDFT_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    cudaError_t e = cudaEventCreateWithFlags(&join, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      cudaEventDestroy(fork);
      ADDFT_CUDA(e);
    }
    // events are released once their work completes; destroying them here is safe
    struct Release {
      cudaEvent_t a, b;
      ~Release() { cudaEventDestroy(a); cudaEventDestroy(b); }
    } release{fork, join};
    ADDFT_CUDA(cudaEventRecord(fork, st));
    ADDFT_CUDA(cudaStreamWaitEvent(side, fork, 0));
    addft_status s = becp_t<R>(nk, nb, pd.nG, nproj, proj, psi, becp, split ? bw : nullptr, split, side);
    if (s == ADDFT_OK) s = dbecp_t<R>(dion, becp, nk, nproj, nb, nullptr, db, side);
    // join even after an error, so a stream capture is never left forked
    ADDFT_CUDA(cudaEventRecord(join, side));
    const addft_status sl = s == ADDFT_OK
                                ? hpsi_local_t<R>(plan, nk, nb, psi, kin, v_r, hpsi, (char *)work + used,
                                                  work_bytes - used, st)
                                : s;
    ADDFT_CUDA(cudaStreamWaitEvent(st, join, 0));
    ADDFT_TRY(sl);
    return apply_t<R, false, true>(db, nb, 1, (size_t)nproj * nb, proj, (size_t)nproj * pd.nG, nk, nproj, nb,
                                   pd.nG, hpsi, (size_t)nb * pd.nG, st);
  }
  if (nproj > 0) {
    ADDFT_TRY(becp_t<R>(nk, nb, pd.nG, nproj, proj, psi, becp, split ? bw : nullptr, split, st));
    ADDFT_TRY(dbecp_t<R>(dion, becp, nk, nproj, nb, nullptr, db, st));
  }
  ADDFT_TRY(hpsi_local_t<R>(plan, nk, nb, psi, kin, v_r, hpsi, (char *)work + used, work_bytes - used, st));
  if (nproj > 0)
    ADDFT_TRY((apply_t<R, false, true>(db, nb, 1, (size_t)nproj * nb, proj, (size_t)nproj * pd.nG, nk, nproj, nb,
                                       pd.nG, hpsi, (size_t)nb * pd.nG, st)));
  return ADDFT_OK;
}

// addft_hpsi on the caller's stream only (no second stream, no events): the form the
// no-allocation entry point runs, which creates no CUDA objects per call.
addft_status hpsi_one_stream(addft_plan plan, addft_dtype dt, int nk, int nb, const void *psi, const void *kin,
                             const void *v_r, int nproj, const void *proj, const void *dion, void *hpsi, void *work,
                             size_t work_bytes, void *stream) {
  ADDFT_REQUIRE(plan && nk >= 1 && nb >= 0 && nproj >= 0, ADDFT_INVALID_ARG, "hpsi: bad arguments");
  if (nb == 0) return ADDFT_OK;   // no bands: the data pointers may be NULL
  ADDFT_REQUIRE(psi && kin && v_r && hpsi, ADDFT_INVALID_ARG, "hpsi: null pointer");
  ADDFT_REQUIRE(nproj == 0 || (proj && dion), ADDFT_INVALID_ARG, "hpsi: null projector tables");
  ADDFT_REQUIRE(psi != hpsi, ADDFT_INVALID_ARG, "hpsi: output aliases input");
  return dt == ADDFT_F64 ? hpsi_t<double>(plan, nk, nb, psi, kin, v_r, nproj, proj, dion, hpsi, work, work_bytes,
                                          as_stream(stream), false)
                         : hpsi_t<float>(plan, nk, nb, psi, kin, v_r, nproj, proj, dion, hpsi, work, work_bytes,
                                         as_stream(stream), false);
}

}  // namespace addft

using namespace addft;

extern "C" {

addft_status addft_kinetic(addft_plan plan, addft_dtype dt, const double *bvec, int nk,
                           const double *kpts, void *kin, void *stream) {
  ADDFT_REQUIRE(plan && bvec && kin && nk >= 1, ADDFT_INVALID_ARG, "kinetic: bad arguments");
  GeoParams gp;
  ADDFT_TRY(make_geo(gp, bvec, 1.0, nk, kpts, 0, nullptr, nullptr));
  dim3 grid((plan->dev.nG + 255) / 256, nk);
  if (dt == ADDFT_F64)
    k_kinetic<double><<<grid, 256, 0, as_stream(stream)>>>(plan->dev, gp, (double *)kin);
  else
    k_kinetic<float><<<grid, 256, 0, as_stream(stream)>>>(plan->dev, gp, (float *)kin);
  return check_launch("k_kinetic");
}

addft_status addft_projectors(addft_plan plan, addft_dtype dt, const double *bvec, double omega, int nk,
                              const double *kpts, int nat, const double *pos, const addft_psp *psp,
                              void *proj, void *stream) {
  ADDFT_REQUIRE(plan && bvec && psp && proj && (nat == 0 || pos), ADDFT_INVALID_ARG,
                "projectors: bad arguments");
  GeoParams gp;
  ADDFT_TRY(make_geo(gp, bvec, omega, nk, kpts, nat, pos, psp));
  if (nat * gp.nh == 0) return ADDFT_OK;
  dim3 grid((plan->dev.nG + 127) / 128, nat * gp.nh, nk);
  if (dt == ADDFT_F64)
    k_projectors<double><<<grid, 128, 0, as_stream(stream)>>>(plan->dev, gp, (double2 *)proj);
  else
    k_projectors<float><<<grid, 128, 0, as_stream(stream)>>>(plan->dev, gp, (float2 *)proj);
  return check_launch("k_projectors");
}

addft_status addft_becp(addft_dtype dt, int nk, int nb, int nG, int nproj, const void *proj,
                        const void *psi, void *becp, void *work, size_t work_bytes, void *stream) {
  ADDFT_REQUIRE(nk >= 0 && nb >= 0 && nG > 0 && nproj >= 0, ADDFT_INVALID_ARG, "becp: bad sizes");
  if (nk * nb * nproj == 0) return ADDFT_OK;
  ADDFT_REQUIRE(proj && psi && becp, ADDFT_INVALID_ARG, "becp: null pointer");
  return dt == ADDFT_F64
             ? becp_t<double>(nk, nb, nG, nproj, proj, psi, becp, work, work_bytes, as_stream(stream))
             : becp_t<float>(nk, nb, nG, nproj, proj, psi, becp, work, work_bytes, as_stream(stream));
}

addft_status addft_vnl_apply(addft_dtype dt, int nk, int nb, int nG, int nproj, const void *proj,
                             const void *dion, const void *becp, void *hpsi, void *work,
                             size_t work_bytes, void *stream) {
  ADDFT_REQUIRE(nk >= 0 && nb >= 0 && nG > 0 && nproj >= 0, ADDFT_INVALID_ARG, "vnl_apply: bad sizes");
  if (nk * nb * nproj == 0) return ADDFT_OK;
  const size_t csz = dt == ADDFT_F64 ? 16 : 8;
  ADDFT_REQUIRE(proj && dion && becp && hpsi && work && work_bytes >= (size_t)nk * nproj * nb * csz,
                ADDFT_INVALID_ARG, "vnl_apply: null pointer or work < nk*nproj*nb complex");
  cudaStream_t st = as_stream(stream);
  const size_t Pk = (size_t)nproj * nG, Xk = (size_t)nproj * nb, Ok = (size_t)nb * nG;
  if (dt == ADDFT_F64) {
    ADDFT_TRY(dbecp_t<double>(dion, becp, nk, nproj, nb, nullptr, work, st));
    return apply_t<double, false, true>(work, nb, 1, Xk, proj, Pk, nk, nproj, nb, nG, hpsi, Ok, st);
  }
  ADDFT_TRY(dbecp_t<float>(dion, becp, nk, nproj, nb, nullptr, work, st));
  return apply_t<float, false, true>(work, nb, 1, Xk, proj, Pk, nk, nproj, nb, nG, hpsi, Ok, st);
}

addft_status addft_nonlocal_energy(addft_dtype dt, int nk, int nb, int nproj, const void *becp,
                                   const void *dion, const double *wocc, double *e_out, void *work,
                                   size_t work_bytes, void *stream) {
  ADDFT_REQUIRE(nk >= 0 && nb >= 0 && nproj >= 0 && e_out, ADDFT_INVALID_ARG, "nonlocal_energy: bad sizes");
  cudaStream_t st = as_stream(stream);
  if (nk * nb * nproj == 0) {
    ADDFT_CUDA(cudaMemsetAsync(e_out, 0, sizeof(double), st));
    return ADDFT_OK;
  }
  const size_t csz = dt == ADDFT_F64 ? 16 : 8;
  const size_t need = align256((size_t)nk * nproj * nb * csz) + (size_t)nk * nb * sizeof(double);
  ADDFT_REQUIRE(becp && dion && wocc && work && work_bytes >= need, ADDFT_INVALID_ARG,
                "nonlocal_energy: null pointer or work < %zu B", need);
  char *w = (char *)work;
  double *ep = (double *)(w + align256((size_t)nk * nproj * nb * csz));
  if (dt == ADDFT_F64) {
    ADDFT_TRY(dbecp_t<double>(dion, becp, nk, nproj, nb, nullptr, w, st));
    k_nl_energy<double><<<(nk * nb + 127) / 128, 128, 0, st>>>((const double2 *)becp, (const double2 *)w,
                                                              nk, nproj, nb, wocc, ep);
  } else {
    ADDFT_TRY(dbecp_t<float>(dion, becp, nk, nproj, nb, nullptr, w, st));
    k_nl_energy<float><<<(nk * nb + 127) / 128, 128, 0, st>>>((const float2 *)becp, (const float2 *)w,
                                                             nk, nproj, nb, wocc, ep);
  }
  ADDFT_TRY(check_launch("k_nl_energy"));
  return finalize_sums(ep, 1, nk * nb, e_out, false, st);
}

addft_status addft_hpsi(addft_plan plan, addft_dtype dt, int nk, int nb, const void *psi, const void *kin,
                        const void *v_r, int nproj, const void *proj, const void *dion, void *hpsi,
                        void *work, size_t work_bytes, void *stream) {
  ADDFT_REQUIRE(plan && nk >= 1 && nb >= 0 && nproj >= 0, ADDFT_INVALID_ARG, "hpsi: bad arguments");
  if (nb == 0) return ADDFT_OK;   // no bands: the data pointers may be NULL
  ADDFT_REQUIRE(psi && kin && v_r && hpsi, ADDFT_INVALID_ARG, "hpsi: null pointer");
  ADDFT_REQUIRE(nproj == 0 || (proj && dion), ADDFT_INVALID_ARG, "hpsi: null projector tables");
  ADDFT_REQUIRE(psi != hpsi, ADDFT_INVALID_ARG, "hpsi: output aliases input");
  return dt == ADDFT_F64 ? hpsi_t<double>(plan, nk, nb, psi, kin, v_r, nproj, proj, dion, hpsi, work, work_bytes,
                                          as_stream(stream), true)
                         : hpsi_t<float>(plan, nk, nb, psi, kin, v_r, nproj, proj, dion, hpsi, work, work_bytes,
                                         as_stream(stream), true);
}

size_t addft_hpsi_work_bytes(addft_plan plan, addft_dtype dt, int nk, int nb, int nproj, int nbatch_chunk) {
  if (!plan) return 0;
  const size_t nls = dt == ADDFT_F64 ? nl_scratch<double>(nk, nb, plan->dev.nG, nproj)
                                     : nl_scratch<float>(nk, nb, plan->dev.nG, nproj);
  return nls + addft_work_bytes(plan, nbatch_chunk < 1 ? 1 : nbatch_chunk, dt);
}

addft_status addft_kinetic_stress(addft_plan plan, addft_dtype dt, const double *bvec, int nk,
                                  const double *kpts, int nb, const void *psi, const double *wocc,
                                  double *out9, void *work, size_t work_bytes, void *stream) {
  ADDFT_REQUIRE(plan && bvec && psi && wocc && out9 && work && work_bytes >= 9 * kRedBlocks * sizeof(double),
                ADDFT_INVALID_ARG, "kinetic_stress: bad arguments");
  GeoParams gp;
  ADDFT_TRY(make_geo(gp, bvec, 1.0, nk, kpts, 0, nullptr, nullptr));
  cudaStream_t st = as_stream(stream);
  double *part = (double *)work;
  if (dt == ADDFT_F64)
    k_kin_stress<double><<<kRedBlocks, 256, 0, st>>>(plan->dev, gp, (const double2 *)psi, nb, wocc, part);
  else
    k_kin_stress<float><<<kRedBlocks, 256, 0, st>>>(plan->dev, gp, (const float2 *)psi, nb, wocc, part);
  ADDFT_TRY(check_launch("k_kin_stress"));
  return finalize_sums(part, 9, kRedBlocks, out9, true, st);
}

addft_status addft_nonlocal_gradients(addft_plan plan, addft_dtype dt, const double *bvec, double omega,
                                      int nk, const double *kpts, int nb, int nat, const double *pos,
                                      const addft_psp *psp, const void *psi, const double *wocc,
                                      const void *dion, double *out, void *work, size_t work_bytes,
                                      void *stream) {
  ADDFT_REQUIRE(plan && bvec && psp && psi && wocc && dion && out && work, ADDFT_INVALID_ARG,
                "nonlocal_gradients: bad arguments");
  GeoParams gp;
  ADDFT_TRY(make_geo(gp, bvec, omega, nk, kpts, nat, pos, psp));
  cudaStream_t st = as_stream(stream);
  const int nproj = nat * gp.nh;
  const int nG = plan->dev.nG;
  if (nproj == 0) {
    ADDFT_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * (1 + 3 * nat + 9), st));
    return ADDFT_OK;
  }
  const size_t csz = dt == ADDFT_F64 ? 16 : 8;
  // layout: proj | becp | DB | Mw | Y | epart | gpart | becp split scratch
  size_t off = 0;
  auto take = [&](size_t b) { size_t o = off; off += align256(b); return o; };
  const size_t o_proj = take((size_t)nk * nproj * nG * csz);
  const size_t o_becp = take((size_t)nk * nproj * nb * csz);
  const size_t o_db = take((size_t)nk * nproj * nb * csz);
  const size_t o_mw = take((size_t)nk * nproj * nb * csz);
  const size_t o_y = take((size_t)nk * nproj * nG * csz);
  const size_t o_ep = take((size_t)nk * nb * sizeof(double));
  const size_t o_gp = take((size_t)nk * nproj * 12 * sizeof(double));
  const size_t bwb = dt == ADDFT_F64 ? becp_work_bytes<double>(nk, nb, nG, nproj)
                                     : becp_work_bytes<float>(nk, nb, nG, nproj);
  const size_t o_bw = take(bwb);
  ADDFT_REQUIRE(work_bytes >= off, ADDFT_INVALID_ARG, "nonlocal_gradients: work needs %zu B, got %zu B",
                off, work_bytes);
  char *w = (char *)work;
  ADDFT_TRY(addft_projectors(plan, dt, bvec, omega, nk, kpts, nat, pos, psp, w + o_proj, stream));
  if (dt == ADDFT_F64) {
    ADDFT_TRY(becp_t<double>(nk, nb, nG, nproj, w + o_proj, psi, w + o_becp, w + o_bw, bwb, st));
    ADDFT_TRY(dbecp_t<double>(dion, w + o_becp, nk, nproj, nb, nullptr, w + o_db, st));
    ADDFT_TRY(dbecp_t<double>(dion, w + o_becp, nk, nproj, nb, wocc, w + o_mw, st));
    ADDFT_TRY((apply_t<double, true, false>(w + o_mw, 1, nb, (size_t)nproj * nb, psi, (size_t)nb * nG, nk, nb,
                                            nproj, nG, w + o_y, (size_t)nproj * nG, st)));
    k_nl_energy<double><<<(nk * nb + 127) / 128, 128, 0, st>>>((const double2 *)(w + o_becp),
                                                              (const double2 *)(w + o_db), nk, nproj, nb,
                                                              wocc, (double *)(w + o_ep));
    ADDFT_TRY(check_launch("k_nl_energy"));
    k_nl_grad<double><<<dim3(nproj, nk), 256, 0, st>>>(plan->dev, gp, (const double2 *)(w + o_y), nproj,
                                                      (double *)(w + o_gp));
  } else {
    ADDFT_TRY(becp_t<float>(nk, nb, nG, nproj, w + o_proj, psi, w + o_becp, w + o_bw, bwb, st));
    ADDFT_TRY(dbecp_t<float>(dion, w + o_becp, nk, nproj, nb, nullptr, w + o_db, st));
    ADDFT_TRY(dbecp_t<float>(dion, w + o_becp, nk, nproj, nb, wocc, w + o_mw, st));
    ADDFT_TRY((apply_t<float, true, false>(w + o_mw, 1, nb, (size_t)nproj * nb, psi, (size_t)nb * nG, nk, nb,
                                           nproj, nG, w + o_y, (size_t)nproj * nG, st)));
    k_nl_energy<float><<<(nk * nb + 127) / 128, 128, 0, st>>>((const float2 *)(w + o_becp),
                                                             (const float2 *)(w + o_db), nk, nproj, nb, wocc,
                                                             (double *)(w + o_ep));
    ADDFT_TRY(check_launch("k_nl_energy"));
    k_nl_grad<float><<<dim3(nproj, nk), 256, 0, st>>>(plan->dev, gp, (const float2 *)(w + o_y), nproj,
                                                     (double *)(w + o_gp));
  }
  ADDFT_TRY(check_launch("k_nl_grad"));
  k_nl_grad_final<<<1, 128, 0, st>>>((const double *)(w + o_ep), nk * nb, (const double *)(w + o_gp), nk,
                                     nproj, gp.nh, nat, out);
  return check_launch("k_nl_grad_final");
}

size_t addft_nonlocal_gradients_work_bytes(addft_dtype dt, int nk, int nb, int nG, int nat, int nh) {
  const size_t csz = dt == ADDFT_F64 ? 16 : 8;
  const int nproj = nat * nh;
  size_t s = 0;
  s += align256((size_t)nk * nproj * nG * csz) * 2;
  s += align256((size_t)nk * nproj * nb * csz) * 3;
  s += align256((size_t)nk * nb * sizeof(double));
  s += align256((size_t)nk * nproj * 12 * sizeof(double));
  s += align256(dt == ADDFT_F64 ? becp_work_bytes<double>(nk, nb, nG, nproj)
                                : becp_work_bytes<float>(nk, nb, nG, nproj));
  return s;
}

}  // extern "C"
