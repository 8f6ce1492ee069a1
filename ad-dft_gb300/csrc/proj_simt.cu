// FP32 projector contractions of V_NL psi on the FP32 FMA pipes, register-tiled.
//
//   becp[k][p][b] = sum_G conj(A[k][p][G]) X[k][b][G]        (nonlocal_op.py:67-70)
//   out[k][i][g] (+)= sum_j X[k][j][i] A[k][j][g]            (nonlocal_op.py:73-76)
//
// Both are exact FP32 complex products (4 FFMA per complex multiply-add) with FP32
// accumulation.  Each thread owns a 4 x 4 block of complex outputs, so every shared-
// memory load feeds four complex multiply-adds: one operand of each inner step is a
// warp-wide broadcast, the other a conflict-free row (odd complex pitch), and the
// FMA pipes, not shared memory, set the pace.
//
// becp: a CTA of 128 threads computes 32 projectors x 64 bands over one chunk of G
//   (split-K, same partial layout as the other becp kernels), staging 32 G per step
//   through a double-buffered cp.async pipeline.
// apply: a CTA of 256 threads computes 64 rows (i) x 64 G over all j, in steps of 32 j;
//   the accumulate form prefetches its output tile with the first step, so the whole
//   read-modify-write costs one memory latency.
#include "common.cuh"

namespace addft {

namespace {
constexpr int kBP = 32, kBB = 64, kBG = 32, kBPit = kBG + 1;   // becp tile and stage
constexpr int kAI = 64, kAG = 64, kAJ = 32, kAPit = 65;        // apply tile and step

__device__ __forceinline__ void cma_conj(float2 &acc, float2 a, float2 x) {   // acc += conj(a) x
  acc.x = fmaf(a.x, x.x, acc.x);
  acc.x = fmaf(a.y, x.y, acc.x);
  acc.y = fmaf(a.x, x.y, acc.y);
  acc.y = fmaf(-a.y, x.x, acc.y);
}
__device__ __forceinline__ void cma(float2 &acc, float2 a, float2 x) {        // acc += a x
  acc.x = fmaf(a.x, x.x, acc.x);
  acc.x = fmaf(-a.y, x.y, acc.x);
  acc.y = fmaf(a.x, x.y, acc.y);
  acc.y = fmaf(a.y, x.x, acc.y);
}
}  // namespace

constexpr size_t kBecpSmem = sizeof(float2) * 2 * (kBP + kBB) * kBPit;

__global__ void __launch_bounds__(128, 4)
k_becp_f32(const float2 *__restrict__ proj, const float2 *__restrict__ psi, int nb, int nG, int nproj, int nsplit,
           int gchunk, float2 *__restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  auto sA = reinterpret_cast<float2 (*)[kBP][kBPit]>(smem);                                        // [2][kBP][kBPit]
  auto sX = reinterpret_cast<float2 (*)[kBB][kBPit]>(smem + sizeof(float2) * 2 * kBP * kBPit);    // [2][kBB][kBPit]
  const int p0 = blockIdx.y * kBP, b0 = blockIdx.x * kBB;
  const int nkz = gridDim.z / nsplit;
  const int k = blockIdx.z / nsplit, sp = blockIdx.z - k * nsplit;
  const int ga = sp * gchunk, gb = min(nG, ga + gchunk);
  const float2 *Pk = proj + (size_t)k * nproj * nG;
  const float2 *Xk = psi + (size_t)k * nb * nG;
  const int tb = threadIdx.x & 15, tp = threadIdx.x >> 4;
  float2 acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[r][u] = make_float2(0.f, 0.f);
  auto issue = [&](int g0, int buf) {
    for (int t = threadIdx.x; t < (kBP + kBB) * kBG; t += 128) {
      const int row = t / kBG, c = t - row * kBG;
      const int g = g0 + c;
      if (row < kBP) {
        const bool ok = p0 + row < nproj && g < gb;
        cp_async_el(&sA[buf][row][c], ok ? Pk + (size_t)(p0 + row) * nG + g : Pk, ok);
      } else {
        const int rr = row - kBP;
        const bool ok = b0 + rr < nb && g < gb;
        cp_async_el(&sX[buf][rr][c], ok ? Xk + (size_t)(b0 + rr) * nG + g : Xk, ok);
      }
    }
    cp_async_commit();
  };
  int buf = 0;
  if (ga < gb) issue(ga, 0);
  for (int g0 = ga; g0 < gb; g0 += kBG) {
    if (g0 + kBG < gb) {
      issue(g0 + kBG, buf ^ 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
#pragma unroll 8
    for (int c = 0; c < kBG; ++c) {
      float2 a[4], x[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = sA[buf][tp + 8 * r][c];
#pragma unroll
      for (int u = 0; u < 4; ++u) x[u] = sX[buf][tb + 16 * u][c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int u = 0; u < 4; ++u) cma_conj(acc[r][u], a[r], x[u]);
    }
    __syncthreads();
    buf ^= 1;
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int p = p0 + tp + 8 * r;
    if (p >= nproj) continue;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int b = b0 + tb + 16 * u;
      if (b < nb) out[(((size_t)sp * nkz + k) * nproj + p) * nb + b] = acc[r][u];
    }
  }
}

template <bool ACCUM>
__global__ void __launch_bounds__(256, 3)
k_apply_f32(const float2 *__restrict__ X, int xs_j, int xs_i, size_t xs_k, const float2 *__restrict__ A,
            size_t as_k, int nj, int ni, int nG, float2 *__restrict__ out, size_t os_k) {
  extern __shared__ __align__(16) unsigned char smem[];
  auto sX = reinterpret_cast<float2 (*)[kAPit]>(smem);                                  // [kAJ][kAPit]: X[j][i]
  auto sA = reinterpret_cast<float2 (*)[kAPit]>(smem + sizeof(float2) * kAJ * kAPit);   // [kAJ][kAPit]: A[j][g]
  auto sO = reinterpret_cast<float2 (*)[kAPit]>(smem + 2 * sizeof(float2) * kAJ * kAPit);   // [kAI][kAPit]
  const int g0 = blockIdx.x * kAG, i0 = blockIdx.y * kAI, k = blockIdx.z;
  const float2 *Ak = A + (size_t)k * as_k;
  const float2 *Xk = X + (size_t)k * xs_k;
  float2 *ok_ = out + (size_t)k * os_k;
  const int tg = threadIdx.x & 15, ti = threadIdx.x >> 4;
  float2 acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[r][u] = make_float2(0.f, 0.f);
  if (ACCUM) {   // output tile prefetch, joined to the first step's copies
    for (int t = threadIdx.x; t < kAI * kAG; t += 256) {
      const int r = t / kAG, c = t - r * kAG;
      const bool ok = i0 + r < ni && g0 + c < nG;
      cp_async_el(&sO[r][c], ok ? ok_ + (size_t)(i0 + r) * nG + g0 + c : ok_, ok);
    }
  }
  for (int j0 = 0; j0 < nj; j0 += kAJ) {
    for (int t = threadIdx.x; t < kAJ * kAI; t += 256) {
      const int r = t / kAI, c = t - r * kAI;
      const bool ok = j0 + r < nj && i0 + c < ni;
      cp_async_el(&sX[r][c], ok ? Xk + (size_t)(j0 + r) * xs_j + (size_t)(i0 + c) * xs_i : Xk, ok);
    }
    for (int t = threadIdx.x; t < kAJ * kAG; t += 256) {
      const int r = t / kAG, c = t - r * kAG;
      const bool ok = j0 + r < nj && g0 + c < nG;
      cp_async_el(&sA[r][c], ok ? Ak + (size_t)(j0 + r) * nG + g0 + c : Ak, ok);
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
#pragma unroll 8
    for (int j = 0; j < kAJ; ++j) {
      float2 x[4], a[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) x[r] = sX[j][ti + 16 * r];
#pragma unroll
      for (int u = 0; u < 4; ++u) a[u] = sA[j][tg + 16 * u];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int u = 0; u < 4; ++u) cma(acc[r][u], x[r], a[u]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int i = i0 + ti + 16 * r;
    if (i >= ni) continue;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int g = g0 + tg + 16 * u;
      if (g >= nG) continue;
      float2 v = acc[r][u];
      if (ACCUM) {
        const float2 o = sO[ti + 16 * r][tg + 16 * u];
        v.x += o.x;
        v.y += o.y;
      }
      ok_[(size_t)i * nG + g] = v;
    }
  }
}

addft_status launch_becp_f32(int nk, int nb, int nG, int nproj, int nsplit, int gchunk, const float2 *proj,
                             const float2 *psi, float2 *out, cudaStream_t st) {
  ADDFT_TRY(smem_optin(k_becp_f32, kBecpSmem));
  dim3 grid((nb + kBB - 1) / kBB, (nproj + kBP - 1) / kBP, nk * nsplit);
  k_becp_f32<<<grid, 128, kBecpSmem, st>>>(proj, psi, nb, nG, nproj, nsplit, gchunk, out);
  return check_launch("k_becp_f32");
}

addft_status launch_apply_f32(bool accum, const float2 *X, int xs_j, int xs_i, size_t xs_k, const float2 *A,
                              size_t as_k, int nk, int nj, int ni, int nG, float2 *out, size_t os_k,
                              cudaStream_t st) {
  const size_t sm = sizeof(float2) * ((size_t)2 * kAJ * kAPit + (accum ? (size_t)kAI * kAPit : 0));
  ADDFT_TRY(smem_optin(accum ? k_apply_f32<true> : k_apply_f32<false>, sm));
  dim3 grid((nG + kAG - 1) / kAG, (ni + kAI - 1) / kAI, nk);
  if (accum)
    k_apply_f32<true><<<grid, 256, sm, st>>>(X, xs_j, xs_i, xs_k, A, as_k, nj, ni, nG, out, os_k);
  else
    k_apply_f32<false><<<grid, 256, sm, st>>>(X, xs_j, xs_i, xs_k, A, as_k, nj, ni, nG, out, os_k);
  return check_launch("k_apply_f32");
}

}  // namespace addft
