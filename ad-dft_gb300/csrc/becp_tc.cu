// becp = conj(beta) psi on the tensor cores (FP32 path).
//
// With complex numbers stored as interleaved float pairs, beta (P x nG) and psi
// (nb x nG) are real matrices with K = 2 nG contiguous, and
//   Re becp[p,b] = sum_k A[p,k] B[b,k],       A = beta, B = psi,
//   Im becp[p,b] = sum_k A[p,k] B'[b,k],      B'[b,2g] = Im psi, B'[b,2g+1] = -Re psi.
// Each product runs as split-precision TF32 on mma.sync m16n8k8 (x = hi + lo,
// a b ~ a_hi b_hi + a_hi b_lo + a_lo b_hi, FP32 accumulation), which keeps the
// FP32 accuracy of the SIMT kernel.  A CTA computes a 32 (projectors) x 64 (bands)
// tile over one K chunk (split-K over G as k_becp, same partial layout for
// k_sum_splits).  Operands are staged 32 complex G at a time by a 2-stage cp.async
// pipeline.  Each warp owns a 32 x 32 block (2 m16 x 4 n8 tiles, Re and Im), so a
// split A fragment feeds 4 n-tiles and a split B fragment 2 m-tiles; the 4 warp
// pairs take different 8-wide K steps of each stage and their partial tiles are
// summed through shared memory at the end.
#include "common.cuh"

namespace addft {

constexpr int kTP = 32, kTB = 64;      // projector and band tile
constexpr int kTK = 64;                // real K per stage (32 complex G)
constexpr int kTKP = kTK + 4;          // padded row pitch (floats): conflict-free fragment loads
constexpr int kRows = kTP + kTB;       // staged rows: projectors, then bands
constexpr int kRedP = kTB + 1;         // reduction row pitch (complex)
constexpr size_t kStageBytes = (size_t)kRows * kTKP * sizeof(float);
constexpr size_t kRedBytes = 4 * (size_t)kTP * kRedP * sizeof(float2);
constexpr size_t kBecpSmem = 2 * kStageBytes > kRedBytes ? 2 * kStageBytes : kRedBytes;

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

__global__ void __launch_bounds__(256, 2)
k_becp_tc(const float2 *__restrict__ proj, const float2 *__restrict__ psi, int nb, int nG, int nproj, int nsplit,
          int gchunk, float2 *__restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  auto stage = [&](int buf) { return reinterpret_cast<float (*)[kTKP]>(smem + buf * kStageBytes); };
  const int p0 = blockIdx.y * kTP, b0 = blockIdx.x * kTB;
  const int nkz = gridDim.z / nsplit;
  const int k = blockIdx.z / nsplit, sp = blockIdx.z - k * nsplit;
  const int ga = sp * gchunk, gb = min(nG, ga + gchunk);
  const float2 *Pk = proj + (size_t)k * nproj * nG;
  const float2 *Xk = psi + (size_t)k * nb * nG;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = lane >> 2, tig = lane & 3;
  const int wb = (warp & 1) * 32;          // band columns of this warp (4 n8 tiles)
  const int kg = warp >> 1;                // K steps 2 kg, 2 kg + 1 of each stage

  float re[2][4][4], im[2][4][4];
#pragma unroll
  for (int m = 0; m < 2; ++m)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) re[m][j][q] = im[m][j][q] = 0.f;

  // stage: 32 complex G of kTP projector rows and kTB band rows, 8-byte cp.async per element
  auto issue = [&](int g0, int buf) {
    float(*st)[kTKP] = stage(buf);
    for (int i = threadIdx.x; i < kRows * (kTK / 2); i += 256) {
      const int r = i / (kTK / 2), c = i - r * (kTK / 2);
      const int g = g0 + c;
      const bool ok = g < gb && (r < kTP ? p0 + r < nproj : b0 + r - kTP < nb);
      const float2 *src = r < kTP ? Pk + (size_t)(p0 + r) * nG + g : Xk + (size_t)(b0 + r - kTP) * nG + g;
      cp_async_el((float2 *)&st[r][2 * c], ok ? src : Pk, ok);
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
    const float(*sA)[kTKP] = stage(buf);
    const float(*sB)[kTKP] = stage(buf) + kTP;
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
      const int kk = (2 * kg + ks) * 8;
      uint32_t ahi[2][4], alo[2][4];
#pragma unroll
      for (int m = 0; m < 2; ++m) {
        split_tf32(sA[16 * m + grp][kk + tig], ahi[m][0], alo[m][0]);
        split_tf32(sA[16 * m + grp + 8][kk + tig], ahi[m][1], alo[m][1]);
        split_tf32(sA[16 * m + grp][kk + tig + 4], ahi[m][2], alo[m][2]);
        split_tf32(sA[16 * m + grp + 8][kk + tig + 4], ahi[m][3], alo[m][3]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float *row = sB[wb + 8 * j + grp];
        // B fragment: k = tig (b0) and tig + 4 (b1); Im operand swaps each (re, im) pair and negates
        const float x0 = row[kk + tig], x1 = row[kk + tig + 4];
        const float y0 = (tig & 1) ? -row[kk + tig - 1] : row[kk + tig + 1];
        const float y1 = (tig & 1) ? -row[kk + tig + 3] : row[kk + tig + 5];
        uint32_t bh0, bl0, bh1, bl1, ch0, cl0, ch1, cl1;
        split_tf32(x0, bh0, bl0);
        split_tf32(x1, bh1, bl1);
        split_tf32(y0, ch0, cl0);
        split_tf32(y1, ch1, cl1);
#pragma unroll
        for (int m = 0; m < 2; ++m) {
          mma_tf32(re[m][j], ahi[m], bh0, bh1);
          mma_tf32(re[m][j], ahi[m], bl0, bl1);
          mma_tf32(re[m][j], alo[m], bh0, bh1);
          mma_tf32(im[m][j], ahi[m], ch0, ch1);
          mma_tf32(im[m][j], ahi[m], cl0, cl1);
          mma_tf32(im[m][j], alo[m], ch0, ch1);
        }
      }
    }
    __syncthreads();
    buf ^= 1;
  }
  // partial tiles of the 4 K groups -> shared memory (D fragment: rows grp / grp + 8,
  // columns 2 tig, 2 tig + 1 of each n8 tile), then summed in a fixed order
  auto red = reinterpret_cast<float2 (*)[kTP][kRedP]>(smem);
#pragma unroll
  for (int m = 0; m < 2; ++m)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q)
        red[kg][16 * m + grp + ((q & 2) ? 8 : 0)][wb + 8 * j + 2 * tig + (q & 1)] = make_float2(re[m][j][q], im[m][j][q]);
  __syncthreads();
  float2 *dst = out + ((size_t)sp * nkz + k) * nproj * nb;
  for (int e = threadIdx.x; e < kTP * kTB; e += 256) {
    const int p = e / kTB, bb = e - p * kTB;
    if (p0 + p < nproj && b0 + bb < nb) {
      float2 v = red[0][p][bb];
#pragma unroll
      for (int g = 1; g < 4; ++g) v = make_float2(v.x + red[g][p][bb].x, v.y + red[g][p][bb].y);
      dst[(size_t)(p0 + p) * nb + b0 + bb] = v;
    }
  }
}

// Launches k_becp_tc with the grid of k_becp (same split-K partial layout).
addft_status launch_becp_tc(int nk, int nb, int nG, int nproj, int nsplit, int gchunk, const float2 *proj,
                            const float2 *psi, float2 *out, cudaStream_t st) {
  ADDFT_TRY(smem_optin(k_becp_tc, kBecpSmem));
  dim3 grid((nb + kTB - 1) / kTB, (nproj + kTP - 1) / kTP, nk * nsplit);
  k_becp_tc<<<grid, 256, kBecpSmem, st>>>(proj, psi, nb, nG, nproj, nsplit, gchunk, out);
  return check_launch("k_becp_tc");
}

}  // namespace addft
