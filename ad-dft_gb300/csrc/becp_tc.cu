// becp = conj(beta) psi on the tensor cores (FP32 path).
//
// With complex numbers stored as interleaved float pairs, beta (P x nG) and psi
// (nb x nG) are real matrices with K = 2 nG contiguous, and
//   Re becp[p,b] = sum_k A[p,k] B[b,k],       A = beta, B = psi,
//   Im becp[p,b] = sum_k A[p,k] B'[b,k],      B'[b,2g] = Im psi, B'[b,2g+1] = -Re psi.
// Each product runs as split-precision TF32 on mma.sync m16n8k8 (x = hi + lo,
// a b ~ a_hi b_hi + a_hi b_lo + a_lo b_hi, FP32 accumulation), which keeps the
// FP32 accuracy of the SIMT kernel.  A CTA computes a 32 (projectors) x 64
// (bands) tile over one K chunk (split-K over G as k_becp, same partial layout
// for k_sum_splits); 8 warps, each a 16 x 16 block (2 m16n8 tiles, Re and Im).
// Operands are staged through shared memory by a 2-stage cp.async pipeline.
#include "common.cuh"

namespace addft {

constexpr int kTP = 32, kTB = 64;      // projector and band tile
constexpr int kTK = 32;                // real K per stage (16 complex G)
constexpr int kTKP = kTK + 4;          // padded row pitch (floats): conflict-free fragment loads

__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void split_tf32(float x, uint32_t &hi, uint32_t &lo) {
  hi = to_tf32(x);
  lo = to_tf32(x - __uint_as_float(hi));
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__global__ void __launch_bounds__(256)
k_becp_tc(const float2 *__restrict__ proj, const float2 *__restrict__ psi, int nb, int nG, int nproj, int nsplit,
          int gchunk, float2 *__restrict__ out) {
  __shared__ __align__(16) float sA[2][kTP][kTKP];
  __shared__ __align__(16) float sB[2][kTB][kTKP];
  const int p0 = blockIdx.y * kTP, b0 = blockIdx.x * kTB;
  const int nkz = gridDim.z / nsplit;
  const int k = blockIdx.z / nsplit, sp = blockIdx.z - k * nsplit;
  const int ga = sp * gchunk, gb = min(nG, ga + gchunk);
  const float2 *Pk = proj + (size_t)k * nproj * nG;
  const float2 *Xk = psi + (size_t)k * nb * nG;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = lane >> 2, tig = lane & 3;
  const int wm = (warp & 1) * 16;          // projector rows of this warp
  const int wn = (warp >> 1) * 16;         // band columns of this warp (2 n8 tiles)

  float re[2][4], im[2][4];
#pragma unroll
  for (int j = 0; j < 2; ++j)
#pragma unroll
    for (int q = 0; q < 4; ++q) re[j][q] = im[j][q] = 0.f;

  // stage: 16 complex G of kTP projector rows and kTB band rows, 8-byte cp.async per element
  auto issue = [&](int g0, int buf) {
    for (int i = threadIdx.x; i < (kTP + kTB) * (kTK / 2); i += 256) {
      const int r = i / (kTK / 2), c = i - r * (kTK / 2);
      const int g = g0 + c;
      if (r < kTP) {
        const bool ok = p0 + r < nproj && g < gb;
        cp_async_el((float2 *)&sA[buf][r][2 * c], ok ? Pk + (size_t)(p0 + r) * nG + g : Pk, ok);
      } else {
        const int rr = r - kTP;
        const bool ok = b0 + rr < nb && g < gb;
        cp_async_el((float2 *)&sB[buf][rr][2 * c], ok ? Xk + (size_t)(b0 + rr) * nG + g : Xk, ok);
      }
    }
    cp_async_commit();
  };

  int buf = 0;
  if (ga < gb) issue(ga, 0);
  for (int g0 = ga; g0 < gb; g0 += kTK / 2) {
    if (g0 + kTK / 2 < gb) {
      issue(g0 + kTK / 2, buf ^ 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kTK; kk += 8) {
      uint32_t ahi[4], alo[4];
      split_tf32(sA[buf][wm + grp][kk + tig], ahi[0], alo[0]);
      split_tf32(sA[buf][wm + grp + 8][kk + tig], ahi[1], alo[1]);
      split_tf32(sA[buf][wm + grp][kk + tig + 4], ahi[2], alo[2]);
      split_tf32(sA[buf][wm + grp + 8][kk + tig + 4], ahi[3], alo[3]);
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const float *row = sB[buf][wn + 8 * j + grp];
        // B fragment: k = tig (b0) and tig + 4 (b1); Im operand swaps each (re, im) pair and negates
        const float x0 = row[kk + tig], x1 = row[kk + tig + 4];
        const float y0 = (tig & 1) ? -row[kk + tig - 1] : row[kk + tig + 1];
        const float y1 = (tig & 1) ? -row[kk + tig + 3] : row[kk + tig + 5];
        uint32_t bh0, bl0, bh1, bl1, ch0, cl0, ch1, cl1;
        split_tf32(x0, bh0, bl0);
        split_tf32(x1, bh1, bl1);
        split_tf32(y0, ch0, cl0);
        split_tf32(y1, ch1, cl1);
        mma_tf32(re[j], ahi, bh0, bh1);
        mma_tf32(re[j], ahi, bl0, bl1);
        mma_tf32(re[j], alo, bh0, bh1);
        mma_tf32(im[j], ahi, ch0, ch1);
        mma_tf32(im[j], ahi, cl0, cl1);
        mma_tf32(im[j], alo, ch0, ch1);
      }
    }
    __syncthreads();
    buf ^= 1;
  }
  // D fragment: rows grp / grp + 8, columns 2 tig, 2 tig + 1 of each n8 tile
  float2 *dst = out + ((size_t)sp * nkz + k) * nproj * nb;
#pragma unroll
  for (int j = 0; j < 2; ++j)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int p = p0 + wm + grp + ((q & 2) ? 8 : 0);
      const int bb = b0 + wn + 8 * j + 2 * tig + (q & 1);
      if (p < nproj && bb < nb) dst[(size_t)p * nb + bb] = make_float2(re[j][q], im[j][q]);
    }
}

// Launches k_becp_tc with the grid of k_becp (same split-K partial layout).
addft_status launch_becp_tc(int nk, int nb, int nG, int nproj, int nsplit, int gchunk, const float2 *proj,
                            const float2 *psi, float2 *out, cudaStream_t st) {
  dim3 grid((nb + kTB - 1) / kTB, (nproj + kTP - 1) / kTP, nk * nsplit);
  k_becp_tc<<<grid, 256, 0, st>>>(proj, psi, nb, nG, nproj, nsplit, gchunk, out);
  return check_launch("k_becp_tc");
}

}  // namespace addft
