// H psi += beta (D becp) on the tensor cores (FP32 path of the V_NL apply).
//
// out[k][i][g] (+)= sum_j A[k][j][g] X[k][j][i]   (A = beta (nj x nG), X = D becp (nj x ni)).
// With complex numbers as interleaved float pairs and K = 2 nj real indices,
//   Re out = sum_k Ar[i][k] B[k][g],   Ar[i][2j] = Re X[j][i], Ar[i][2j+1] = -Im X[j][i]
//   Im out = sum_k Ai[i][k] B[k][g],   Ai[i][2j] = Im X[j][i], Ai[i][2j+1] =  Re X[j][i]
//   B[2j + c][g] = (Re, Im)_c A[j][g],
// each product as split-precision TF32 (hi hi + hi lo + lo hi) on mma.sync m16n8k8 with
// FP32 accumulation.  A CTA computes 64 rows (i) x 64 G over all j in stages of 16 j
// staged by cp.async; 8 warps, each 32 rows x 16 G (2 m16 x 2 n8 tiles, Re and Im).
// Shared-memory rows are padded to 72 complex (8 mod 16) so that fragment loads are
// bank-conflict-free.  The accumulate form prefetches its 64 x 64 output tile with the
// first stage, so that the whole tile has one memory latency; the result goes back
// through shared memory and is stored row-contiguous.
#include "common.cuh"

namespace addft {

namespace {
constexpr int kMI = 64, kNG = 64, kJS = 16;     // rows, G, projectors per stage
constexpr int kPit = 72;                        // padded row length (complex)
constexpr int kOPit = 65;                       // output tile row length (complex)
constexpr size_t kStageBytes = 2 * 2 * kJS * kPit * sizeof(float2);
constexpr size_t kSmemBytes = kStageBytes + (size_t)kMI * kOPit * sizeof(float2);

__device__ __forceinline__ uint32_t tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ void split(float x, uint32_t &hi, uint32_t &lo) {
  hi = tf32(x);
  lo = tf32(x - __uint_as_float(hi));
}
__device__ __forceinline__ void mma(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
}  // namespace

template <bool ACCUM>
__global__ void __launch_bounds__(256, 2)
k_apply_tc(const float2 *__restrict__ X, int xs_j, int xs_i, size_t xs_k, const float2 *__restrict__ A,
           size_t as_k, int nj, int ni, int nG, float2 *__restrict__ out, size_t os_k) {
  extern __shared__ __align__(16) unsigned char smem[];
  auto sX = reinterpret_cast<float2 (*)[kJS][kPit]>(smem);                           // X[j][i]
  auto sB = reinterpret_cast<float2 (*)[kJS][kPit]>(smem + kStageBytes / 2);         // A[j][g]
  auto sO = reinterpret_cast<float2 (*)[kOPit]>(smem + kStageBytes);                 // out[i][g]
  const int g0 = blockIdx.x * kNG, i0 = blockIdx.y * kMI, k = blockIdx.z;
  const float2 *Ak = A + (size_t)k * as_k;
  const float2 *Xk = X + (size_t)k * xs_k;
  float2 *ok_ = out + (size_t)k * os_k;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = lane >> 2, tig = lane & 3;
  const int wm = (warp & 1) * 32, wn = (warp >> 1) * 16;

  float re[2][2][4], im[2][2][4];
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b)
#pragma unroll
      for (int q = 0; q < 4; ++q) re[a][b][q] = im[a][b][q] = 0.f;

  auto issue = [&](int j0, int buf) {
    for (int t = threadIdx.x; t < kJS * kNG; t += 256) {
      const int r = t / kNG, c = t - r * kNG;
      const bool ok = j0 + r < nj && g0 + c < nG;
      cp_async_el(&sB[buf][r][c], ok ? Ak + (size_t)(j0 + r) * nG + g0 + c : Ak, ok);
    }
    for (int t = threadIdx.x; t < kJS * kMI; t += 256) {
      const int r = t / kMI, c = t - r * kMI;
      const bool ok = j0 + r < nj && i0 + c < ni;
      cp_async_el(&sX[buf][r][c], ok ? Xk + (size_t)(j0 + r) * xs_j + (size_t)(i0 + c) * xs_i : Xk, ok);
    }
    cp_async_commit();
  };

  if (ACCUM) {   // output tile joins the first cp.async group
    for (int t = threadIdx.x; t < kMI * kNG; t += 256) {
      const int r = t / kNG, c = t - r * kNG;
      const bool ok = i0 + r < ni && g0 + c < nG;
      cp_async_el(&sO[r][c], ok ? ok_ + (size_t)(i0 + r) * nG + g0 + c : ok_, ok);
    }
  }
  int buf = 0;
  issue(0, 0);
  for (int j0 = 0; j0 < nj; j0 += kJS) {
    if (j0 + kJS < nj) {
      issue(j0 + kJS, buf ^ 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const float *xs = reinterpret_cast<const float *>(&sX[buf][0][0]);
    const float *bs = reinterpret_cast<const float *>(&sB[buf][0][0]);
#pragma unroll
    for (int kk = 0; kk < 2 * kJS; kk += 8) {
      // real index kr = kk + t -> projector j = kr >> 1, component c = kr & 1
      const int ja = (kk + tig) >> 1, jb = (kk + tig + 4) >> 1, c = tig & 1;
      uint32_t arh[2][4], arl[2][4], aih[2][4], ail[2][4];
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        const int r0 = wm + 16 * mt + grp;
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          const int row = r0 + ((h & 1) ? 8 : 0);
          const int j = (h & 2) ? jb : ja;
          const float xr = xs[(j * kPit + row) * 2], xi = xs[(j * kPit + row) * 2 + 1];
          split(c == 0 ? xr : -xi, arh[mt][h], arl[mt][h]);
          split(c == 0 ? xi : xr, aih[mt][h], ail[mt][h]);
        }
      }
#pragma unroll
      for (int nt = 0; nt < 2; ++nt) {
        const int col = wn + 8 * nt + grp;
        uint32_t bh0, bl0, bh1, bl1;
        split(bs[(ja * kPit + col) * 2 + c], bh0, bl0);
        split(bs[(jb * kPit + col) * 2 + c], bh1, bl1);
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
          mma(re[mt][nt], arh[mt], bh0, bh1);
          mma(re[mt][nt], arh[mt], bl0, bl1);
          mma(re[mt][nt], arl[mt], bh0, bh1);
          mma(im[mt][nt], aih[mt], bh0, bh1);
          mma(im[mt][nt], aih[mt], bl0, bl1);
          mma(im[mt][nt], ail[mt], bh0, bh1);
        }
      }
    }
    __syncthreads();
    buf ^= 1;
  }
  // D fragment: rows grp / grp + 8, columns 2 tig, 2 tig + 1 of each n8 tile
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        float2 &o = sO[wm + 16 * mt + grp + ((q & 2) ? 8 : 0)][wn + 8 * nt + 2 * tig + (q & 1)];
        o = ACCUM ? make_float2(o.x + re[mt][nt][q], o.y + im[mt][nt][q]) : make_float2(re[mt][nt][q], im[mt][nt][q]);
      }
  __syncthreads();
  for (int t = threadIdx.x; t < kMI * kNG; t += 256) {
    const int r = t / kNG, c = t - r * kNG;
    if (i0 + r < ni && g0 + c < nG) ok_[(size_t)(i0 + r) * nG + g0 + c] = sO[r][c];
  }
}

addft_status launch_apply_tc(bool accum, const float2 *X, int xs_j, int xs_i, size_t xs_k, const float2 *A,
                             size_t as_k, int nk, int nj, int ni, int nG, float2 *out, size_t os_k,
                             cudaStream_t st) {
  ADDFT_TRY(smem_optin(accum ? k_apply_tc<true> : k_apply_tc<false>, kSmemBytes));
  dim3 grid((nG + kNG - 1) / kNG, (ni + kMI - 1) / kMI, nk);
  if (accum)
    k_apply_tc<true><<<grid, 256, kSmemBytes, st>>>(X, xs_j, xs_i, xs_k, A, as_k, nj, ni, nG, out, os_k);
  else
    k_apply_tc<false><<<grid, 256, kSmemBytes, st>>>(X, xs_j, xs_i, xs_k, A, as_k, nj, ni, nG, out, os_k);
  return check_launch("k_apply_tc");
}

}  // namespace addft
