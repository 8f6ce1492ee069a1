// Ewald ion-ion energy with its position and strain derivatives, f64 on the
// device.  Reference: src/addft/physics/ewald.py:34-77 (nmax translations
// per axis in real space, (2 nmax + 5)^3 reciprocal vectors, eta = 0.9
// default), E = E_real + E_recip + E_self + E_bg.
#include "common.cuh"

namespace addft {

constexpr int kMaxAtomsE = 256;

struct EwaldParams {
  double L[9];     // lattice rows
  double B[9];     // reciprocal rows
  double omega, eta;
  int nat, nmax;
  double pos[kMaxAtomsE * 3];
  double z[kMaxAtomsE];
};

// real-space pair (i, j): partial[pair][13] = {E, dE/dR_i (3), dE/deps (9)}
__global__ void __launch_bounds__(256) k_ewald_real(EwaldParams ep, double *__restrict__ partial) {
  const int pair = blockIdx.x;
  const int i = pair / ep.nat, j = pair - i * ep.nat;
  const int side = 2 * ep.nmax + 1;
  const int nt = side * side * side;
  const double zz = ep.z[i] * ep.z[j];
  const double rp = 1.1283791670955125739 * ep.eta;   // 2 eta / sqrt(pi)
  double acc[13];
#pragma unroll
  for (int t = 0; t < 13; ++t) acc[t] = 0.0;
  for (int t = threadIdx.x; t < nt; t += blockDim.x) {
    const int a = t / (side * side) - ep.nmax;
    const int b = (t / side) % side - ep.nmax;
    const int c = t % side - ep.nmax;
    if (i == j && a == 0 && b == 0 && c == 0) continue;
    double d[3];
    for (int x = 0; x < 3; ++x)
      d[x] = ep.pos[3 * i + x] - ep.pos[3 * j + x] + a * ep.L[x] + b * ep.L[3 + x] + c * ep.L[6 + x];
    const double dist = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + 1e-30);
    const double phi = erfc(ep.eta * dist) / dist;
    const double dphi = -phi / dist - rp * exp(-(ep.eta * dist) * (ep.eta * dist)) / dist;
    acc[0] += 0.5 * zz * phi;
    const double f = 0.5 * zz * dphi / dist;
    // pair (i,j) contributes f d to dE/dR_i and -f d to dE/dR_j (handled in finalize)
    for (int x = 0; x < 3; ++x) acc[1 + x] += f * d[x];
    for (int x = 0; x < 3; ++x)
      for (int y = 0; y < 3; ++y) acc[4 + 3 * x + y] += f * d[x] * d[y];
  }
  __shared__ double red[8][13];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int q = 0; q < 13; ++q) {
    double x = acc[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][q] = x;
  }
  __syncthreads();
  if (threadIdx.x < 13) {
    double s = 0.0;
    for (int w = 0; w < (blockDim.x >> 5); ++w) s += red[w][threadIdx.x];
    partial[(size_t)pair * 13 + threadIdx.x] = s;
  }
}

__device__ __forceinline__ void recip_vec(const EwaldParams &ep, int t, double *g, bool &keep) {
  const int M = ep.nmax + 2, side = 2 * M + 1;
  const int a = t / (side * side) - M, b = (t / side) % side - M, c = t % side - M;
  for (int x = 0; x < 3; ++x) g[x] = a * ep.B[x] + b * ep.B[3 + x] + c * ep.B[6 + x];
  keep = (g[0] * g[0] + g[1] * g[1] + g[2] * g[2]) > 1e-12;
}

// reciprocal sums: partial [10][nblk] = {sum w |S|^2, sum coef |S|^2 G_a G_b}
__global__ void __launch_bounds__(kRedThreads) k_ewald_recip(EwaldParams ep, double *__restrict__ partial) {
  const int M = ep.nmax + 2, side = 2 * M + 1, ng = side * side * side;
  double acc[10];
#pragma unroll
  for (int q = 0; q < 10; ++q) acc[q] = 0.0;
  const double e4 = 4.0 * ep.eta * ep.eta;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ng; t += gridDim.x * blockDim.x) {
    double g[3];
    bool keep;
    recip_vec(ep, t, g, keep);
    if (!keep) continue;
    const double g2 = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
    double sr = 0.0, si = 0.0;
    for (int i = 0; i < ep.nat; ++i) {
      double sn, cs;
      sincos(g[0] * ep.pos[3 * i] + g[1] * ep.pos[3 * i + 1] + g[2] * ep.pos[3 * i + 2], &sn, &cs);
      sr += ep.z[i] * cs;
      si -= ep.z[i] * sn;
    }
    const double s2 = sr * sr + si * si;
    const double ex = exp(-g2 / e4);
    acc[0] += ex / g2 * s2;
    const double coef = ex * (1.0 / (e4 * g2) + 1.0 / (g2 * g2)) * 2.0 * s2;
    for (int x = 0; x < 3; ++x)
      for (int y = 0; y < 3; ++y) acc[1 + 3 * x + y] += coef * g[x] * g[y];
  }
  block_reduce_store<10>(acc, partial);
}

// reciprocal forces per atom: dE/dR_i = pref sum_G 2 w Re(conj(S) z_i (-i) e^{-iG.R_i}) G
__global__ void __launch_bounds__(256) k_ewald_recip_force(EwaldParams ep, double *__restrict__ partial) {
  const int i = blockIdx.x;
  const int M = ep.nmax + 2, side = 2 * M + 1, ng = side * side * side;
  const double e4 = 4.0 * ep.eta * ep.eta;
  double acc[3] = {0.0, 0.0, 0.0};
  for (int t = threadIdx.x; t < ng; t += blockDim.x) {
    double g[3];
    bool keep;
    recip_vec(ep, t, g, keep);
    if (!keep) continue;
    const double g2 = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
    double sr = 0.0, si = 0.0, ci = 0.0, snI = 0.0;
    for (int j = 0; j < ep.nat; ++j) {
      double sn, cs;
      sincos(g[0] * ep.pos[3 * j] + g[1] * ep.pos[3 * j + 1] + g[2] * ep.pos[3 * j + 2], &sn, &cs);
      sr += ep.z[j] * cs;
      si -= ep.z[j] * sn;
      if (j == i) { ci = cs; snI = sn; }
    }
    // conj(S) * z_i * (-i) * (cs - i sn) = z_i conj(S) (-sn - i cs)
    const double xr = -snI, xi = -ci;
    const double re = ep.z[i] * (sr * xr + si * xi);
    const double w = exp(-g2 / e4) / g2;
    for (int x = 0; x < 3; ++x) acc[x] += 2.0 * w * re * g[x];
  }
  __shared__ double red[8][3];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int q = 0; q < 3; ++q) {
    double x = acc[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][q] = x;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double s = 0.0;
    for (int w = 0; w < (blockDim.x >> 5); ++w) s += red[w][threadIdx.x];
    partial[(size_t)i * 3 + threadIdx.x] = s;
  }
}

__global__ void k_ewald_final(EwaldParams ep, const double *__restrict__ real_part,
                              const double *__restrict__ rsum, const double *__restrict__ rforce,
                              double *__restrict__ out) {
  const int nat = ep.nat;
  const double pref = 2.0 * 3.14159265358979323846 / ep.omega;
  const double sqpi = 1.7724538509055160273;
  double ztot = 0.0, z2 = 0.0;
  for (int i = 0; i < nat; ++i) { ztot += ep.z[i]; z2 += ep.z[i] * ep.z[i]; }
  const double e_recip = pref * rsum[0];
  const double e_self = -(ep.eta / sqpi) * z2;
  const double e_bg = -(3.14159265358979323846 / (2.0 * ep.omega * ep.eta * ep.eta)) * ztot * ztot;
  for (int t = threadIdx.x; t < 1 + 3 * nat + 9; t += blockDim.x) {
    double v = 0.0;
    if (t == 0) {
      for (int p = 0; p < nat * nat; ++p) v += real_part[(size_t)p * 13];
      v += e_recip + e_self + e_bg;
    } else if (t < 1 + 3 * nat) {
      const int i = (t - 1) / 3, x = (t - 1) % 3;
      for (int j = 0; j < nat; ++j) {
        v += real_part[((size_t)i * nat + j) * 13 + 1 + x];   // pair (i, j): +f d
        v -= real_part[((size_t)j * nat + i) * 13 + 1 + x];   // pair (j, i): -f d for atom i
      }
      v += pref * rforce[(size_t)i * 3 + x];
    } else {
      const int ab = t - 1 - 3 * nat;
      for (int p = 0; p < nat * nat; ++p) v += real_part[(size_t)p * 13 + 4 + ab];
      v += pref * rsum[1 + ab];
      if (ab % 4 == 0) v += -e_recip - e_bg;
    }
    out[t] = v;
  }
}

}  // namespace addft

using namespace addft;

extern "C" {

size_t addft_ewald_work_bytes(int nat) {
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  return al((size_t)nat * nat * 13 * sizeof(double)) + al(10 * kRedBlocks * sizeof(double)) +
         al(16 * sizeof(double)) + al((size_t)(nat > 0 ? nat : 1) * 3 * sizeof(double));
}

addft_status addft_ewald(const double *lattice, int nat, const double *pos, const double *charges, double eta,
                         int nmax, double *out, void *work, size_t work_bytes, void *stream) {
  ADDFT_REQUIRE(lattice && out && nat >= 1 && pos && charges && eta > 0 && nmax >= 0, ADDFT_INVALID_ARG,
                "ewald: bad arguments");
  ADDFT_REQUIRE(nat <= kMaxAtomsE, ADDFT_UNSUPPORTED, "ewald: nat = %d exceeds %d", nat, kMaxAtomsE);
  ADDFT_REQUIRE(work && work_bytes >= addft_ewald_work_bytes(nat), ADDFT_INVALID_ARG,
                "ewald: work needs %zu B", addft_ewald_work_bytes(nat));
  EwaldParams ep;
  memset(&ep, 0, sizeof(ep));
  for (int i = 0; i < 9; ++i) ep.L[i] = lattice[i];
  // B = 2 pi inv(L)^T, Omega = |det L|
  const double *L = lattice;
  const double det = L[0] * (L[4] * L[8] - L[5] * L[7]) - L[1] * (L[3] * L[8] - L[5] * L[6]) +
                     L[2] * (L[3] * L[7] - L[4] * L[6]);
  ADDFT_REQUIRE(fabs(det) > 0, ADDFT_INVALID_ARG, "ewald: singular lattice");
  double inv[9];
  inv[0] = (L[4] * L[8] - L[5] * L[7]) / det;
  inv[1] = (L[2] * L[7] - L[1] * L[8]) / det;
  inv[2] = (L[1] * L[5] - L[2] * L[4]) / det;
  inv[3] = (L[5] * L[6] - L[3] * L[8]) / det;
  inv[4] = (L[0] * L[8] - L[2] * L[6]) / det;
  inv[5] = (L[2] * L[3] - L[0] * L[5]) / det;
  inv[6] = (L[3] * L[7] - L[4] * L[6]) / det;
  inv[7] = (L[1] * L[6] - L[0] * L[7]) / det;
  inv[8] = (L[0] * L[4] - L[1] * L[3]) / det;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) ep.B[3 * r + c] = 2.0 * M_PI * inv[3 * c + r];
  ep.omega = fabs(det);
  ep.eta = eta;
  ep.nat = nat;
  ep.nmax = nmax;
  for (int i = 0; i < 3 * nat; ++i) ep.pos[i] = pos[i];
  for (int i = 0; i < nat; ++i) ep.z[i] = charges[i];
  cudaStream_t st = as_stream(stream);
  auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
  char *w = (char *)work;
  double *real_part = (double *)w;
  double *rpart = (double *)(w + al((size_t)nat * nat * 13 * sizeof(double)));
  double *rsum = (double *)((char *)rpart + al(10 * kRedBlocks * sizeof(double)));
  double *rforce = (double *)((char *)rsum + al(16 * sizeof(double)));
  k_ewald_real<<<nat * nat, 256, 0, st>>>(ep, real_part);
  ADDFT_TRY(check_launch("k_ewald_real"));
  k_ewald_recip<<<kRedBlocks, kRedThreads, 0, st>>>(ep, rpart);
  ADDFT_TRY(check_launch("k_ewald_recip"));
  ADDFT_TRY(finalize_sums(rpart, 10, kRedBlocks, rsum, false, st));
  k_ewald_recip_force<<<nat, 256, 0, st>>>(ep, rforce);
  ADDFT_TRY(check_launch("k_ewald_recip_force"));
  k_ewald_final<<<1, 128, 0, st>>>(ep, real_part, rsum, rforce, out);
  return check_launch("k_ewald_final");
}

}  // extern "C"
