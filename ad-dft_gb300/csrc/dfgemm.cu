// Complex FP64 GEMM in double-float arithmetic on the FP32 pipes.
//
//   C (M x N) = op(A) op(B),  op(A)[i][k] = A[i sAi + k sAk] (conjugated if conjA),
//                             op(B)[k][j] = B[k sBk + j sBj] (conjugated if conjB),
// complex128 in and out (interleaved), for the subspace products of the
// FP64-anchored refinement: projections X^H Y with K = nG (solver/davidson.py:48,
// :59-61) and rotations U [X, H X] with K = block size (davidson.py:51-52).
// GB300's FP64 rate is ~1/64 of FP32, so each operand element is split into an
// FP32 pair x = hi + lo (hi = the top 24 significand bits, lo = the next 24;
// formed with integer operations, so nothing runs on the FP64 pipe) and every
// real product a b is accumulated as
//   p = fl(ah bh), e = fma(ah, bh, -p) + ah bl + al bh   (the exact error of p plus the cross terms)
//   (s, c) <- TwoSum(s, p) with c += err + e
// with the additions written as non-contracting intrinsics.  The pair (s, c) is
// renormalised after every K step of a tile and written out as the double s + c.
// Relative error ~1e-14 (48-bit operands, exact products, compensated sums).
//
// Tiling: a CTA computes 32 x 64 outputs with 256 threads (2 x 4 outputs each),
// K staged 16 at a time through shared memory as float4 (re_hi, im_hi, re_lo,
// im_lo), k-major with padded rows (conflict-free stores and broadcast /
// contiguous fragment reads).  Long K is split over gridDim.z; the partial tiles
// are summed in a fixed order by a second kernel.
#include <algorithm>

#include "common.cuh"

namespace addft {

namespace {
constexpr int kDM = 32, kDN = 64, kDK = 16;

// x -> (hi, lo) with hi = x truncated to 24 significand bits and lo = the
// remainder rounded to 24 bits; values below the FP32 normal range flush to 0.
__device__ __forceinline__ void split_d(double x, float &hi, float &lo) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned sign = (unsigned)(u >> 63) << 31;
  const int e = (int)((u >> 52) & 0x7ff);
  const int fe = e - 1023 + 127;
  if (fe <= 0) {
    hi = 0.f;
    lo = 0.f;
    return;
  }
  if (fe >= 255) {   // beyond the FP32 range (inputs here are bounded): infinity
    hi = __uint_as_float(sign | 0x7f800000u);
    lo = 0.f;
    return;
  }
  const unsigned long long m = u & 0xFFFFFFFFFFFFFull;
  hi = __uint_as_float(sign | ((unsigned)fe << 23) | (unsigned)(m >> 29));
  const int se = e - 1075 + 127;   // 2^(e - 1075) as an FP32 scale
  const float r = __uint2float_rn((unsigned)(m & 0x1FFFFFFFull));
  const float l = se > 0 ? __fmul_rn(r, __uint_as_float((unsigned)se << 23)) : 0.f;
  lo = sign ? -l : l;
}

__device__ __forceinline__ float4 split_c(double2 v, bool conj) {
  float rh, rl, ih, il;
  split_d(v.x, rh, rl);
  split_d(conj ? -v.y : v.y, ih, il);
  return make_float4(rh, ih, rl, il);
}

// (s, c) += (ah + al)(bh + bl)
__device__ __forceinline__ void df_mac(float &s, float &c, float ah, float al, float bh, float bl) {
  const float p = __fmul_rn(ah, bh);
  float e = fmaf(ah, bh, -p);
  e = fmaf(ah, bl, e);
  e = fmaf(al, bh, e);
  const float t = __fadd_rn(s, p);
  const float z = __fsub_rn(t, s);
  const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
  s = t;
  c = __fadd_rn(c, __fadd_rn(err, e));
}

// acc = (re_s, re_c, im_s, im_c) += a b for double-float complex a, b (float4 layout)
__device__ __forceinline__ void df_cmac(float (&acc)[4], const float4 a, const float4 b) {
  df_mac(acc[0], acc[1], a.x, a.z, b.x, b.z);
  df_mac(acc[0], acc[1], -a.y, -a.w, b.y, b.w);
  df_mac(acc[2], acc[3], a.x, a.z, b.y, b.w);
  df_mac(acc[2], acc[3], a.y, a.w, b.x, b.z);
}

__device__ __forceinline__ void renorm(float &s, float &c) {
  const float t = __fadd_rn(s, c);
  c = __fsub_rn(c, __fsub_rn(t, s));
  s = t;
}
}  // namespace

// KA / KB: the operand's contiguous index is k (lanes step along k while staging)
template <bool KA, bool KB>
__global__ void __launch_bounds__(256)
k_zgemm_df(int M, int N, int K, const double2 *__restrict__ A, long sAi, long sAk, int conjA,
           const double2 *__restrict__ B, long sBk, long sBj, int conjB, int kchunk, double2 *__restrict__ C,
           long ldc, size_t split_stride) {
  __shared__ float4 sA[kDK][kDM + 1];
  __shared__ float4 sB[kDK][kDN + 1];
  const int j0 = blockIdx.x * kDN, i0 = blockIdx.y * kDM;
  const int ks = blockIdx.z * kchunk, ke = min(K, ks + kchunk);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float acc[2][4][4];
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[r][c][q] = 0.f;

  for (int k0 = ks; k0 < ke; k0 += kDK) {
    for (int e = threadIdx.x; e < kDM * kDK; e += 256) {
      const int k = KA ? e % kDK : e / kDM, i = KA ? e / kDK : e % kDM;
      const int gi = i0 + i, gk = k0 + k;
      const double2 v = gi < M && gk < ke ? A[gi * sAi + gk * sAk] : make_double2(0.0, 0.0);
      sA[k][i] = split_c(v, conjA != 0);
    }
    for (int e = threadIdx.x; e < kDN * kDK; e += 256) {
      const int k = KB ? e % kDK : e / kDN, j = KB ? e / kDK : e % kDN;
      const int gj = j0 + j, gk = k0 + k;
      const double2 v = gj < N && gk < ke ? B[gk * sBk + gj * sBj] : make_double2(0.0, 0.0);
      sB[k][j] = split_c(v, conjB != 0);
    }
    __syncthreads();
#pragma unroll 2
    for (int k = 0; k < kDK; ++k) {
      float4 a[2], b[4];
#pragma unroll
      for (int r = 0; r < 2; ++r) a[r] = sA[k][ty + 16 * r];
#pragma unroll
      for (int c = 0; c < 4; ++c) b[c] = sB[k][tx + 16 * c];
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) df_cmac(acc[r][c], a[r], b[c]);
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        renorm(acc[r][c][0], acc[r][c][1]);
        renorm(acc[r][c][2], acc[r][c][3]);
      }
  }
  double2 *Cz = C + blockIdx.z * split_stride;
#pragma unroll
  for (int r = 0; r < 2; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int i = i0 + ty + 16 * r, j = j0 + tx + 16 * c;
      if (i < M && j < N)
        Cz[(size_t)i * ldc + j] = make_double2((double)acc[r][c][0] + (double)acc[r][c][1],
                                               (double)acc[r][c][2] + (double)acc[r][c][3]);
    }
}

// C[i][j] = sum_s part[s][i][j] in split order (FP64)
__global__ void __launch_bounds__(256)
k_zgemm_df_splits(const double2 *__restrict__ part, int nsplit, int M, int N, double2 *__restrict__ C, long ldc) {
  const size_t n = (size_t)M * N;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    double2 s = part[t];
    for (int z = 1; z < nsplit; ++z) {
      const double2 v = part[(size_t)z * n + t];
      s.x += v.x;
      s.y += v.y;
    }
    C[(t / N) * ldc + t % N] = s;
  }
}

// split count: about 4 CTAs per SM of work, K chunks of at least 256
static int df_nsplit(int M, int N, int K) {
  const int tiles = ((M + kDM - 1) / kDM) * ((N + kDN - 1) / kDN);
  int ns = (4 * 152 + tiles - 1) / tiles;
  ns = std::min(ns, std::max(1, K / 256));
  return std::max(ns, 1);
}

}  // namespace addft

using namespace addft;

extern "C" size_t addft_zgemm_df_work_bytes(int M, int N, int K) {
  if (M <= 0 || N <= 0 || K <= 0) return 0;
  const int ns = df_nsplit(M, N, K);
  return ns > 1 ? (size_t)ns * M * N * sizeof(double2) : 0;
}

extern "C" addft_status addft_zgemm_df(int M, int N, int K, const void *A, long sAi, long sAk, int conjA,
                                       const void *B, long sBk, long sBj, int conjB, void *C, long ldc,
                                       void *work, size_t work_bytes, void *stream) {
  ADDFT_REQUIRE(M >= 0 && N >= 0 && K >= 0 && ldc >= N, ADDFT_INVALID_ARG, "zgemm_df: bad sizes");
  if (M == 0 || N == 0) return ADDFT_OK;
  ADDFT_REQUIRE(C, ADDFT_INVALID_ARG, "zgemm_df: null C");
  cudaStream_t st = as_stream(stream);
  if (K == 0) {
    ADDFT_REQUIRE(cudaMemset2DAsync(C, sizeof(double2) * ldc, 0, sizeof(double2) * N, M, st) == cudaSuccess,
                  ADDFT_CUDA_ERROR, "zgemm_df: clearing C failed");
    return ADDFT_OK;
  }
  ADDFT_REQUIRE(A && B, ADDFT_INVALID_ARG, "zgemm_df: null operand");
  int ns = df_nsplit(M, N, K);
  if (ns > 1 && (work == nullptr || work_bytes < (size_t)ns * M * N * sizeof(double2))) ns = 1;
  const int kchunk = ns > 1 ? ((K + ns - 1) / ns + kDK - 1) / kDK * kDK : K;
  ns = (K + kchunk - 1) / kchunk;
  dim3 grid((N + kDN - 1) / kDN, (M + kDM - 1) / kDM, ns);
  double2 *dst = ns > 1 ? (double2 *)work : (double2 *)C;
  const long ld = ns > 1 ? N : ldc;
  const size_t ss = ns > 1 ? (size_t)M * N : 0;
  const bool ka = sAk == 1, kb = sBk == 1;
  const double2 *a = (const double2 *)A, *b = (const double2 *)B;
  if (ka && kb)
    k_zgemm_df<true, true><<<grid, 256, 0, st>>>(M, N, K, a, sAi, sAk, conjA, b, sBk, sBj, conjB, kchunk, dst, ld, ss);
  else if (ka)
    k_zgemm_df<true, false><<<grid, 256, 0, st>>>(M, N, K, a, sAi, sAk, conjA, b, sBk, sBj, conjB, kchunk, dst, ld, ss);
  else if (kb)
    k_zgemm_df<false, true><<<grid, 256, 0, st>>>(M, N, K, a, sAi, sAk, conjA, b, sBk, sBj, conjB, kchunk, dst, ld, ss);
  else
    k_zgemm_df<false, false><<<grid, 256, 0, st>>>(M, N, K, a, sAi, sAk, conjA, b, sBk, sBj, conjB, kchunk, dst, ld, ss);
  ADDFT_TRY(check_launch("k_zgemm_df"));
  if (ns > 1) {
    const size_t n = (size_t)M * N;
    const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 4 * 152);
    k_zgemm_df_splits<<<blocks, 256, 0, st>>>((const double2 *)work, ns, M, N, (double2 *)C, ldc);
    ADDFT_TRY(check_launch("k_zgemm_df_splits"));
  }
  return ADDFT_OK;
}
