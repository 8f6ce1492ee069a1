// FP32 projector contractions of V_NL psi on the 5th-generation tensor cores
// (tcgen05.mma kind::tf32, accumulators in tensor memory), split-precision TF32:
// every product a b is formed as hi(a) hi(b) + hi(a) lo(b) + lo(a) hi(b) with
// FP32 accumulation (hi = round-to-nearest TF32 of x, lo = TF32 of x - hi), about
// 1e-6 relative, like the warp-MMA kernels.
//
//   becp[k][p][b] = sum_G conj(proj[k][p][G]) psi[k][b][G]          (nonlocal_op.py:67-70)
//     D (128 x 32) = X (128 x K) P^T: rows of X are the 64 bands of a tile, then the
//     same bands with each (re, im) pair replaced by (im, -re); columns of P are 32
//     projectors; K runs over (G, re/im).  Row b of D is Re becp[.][b], row 64 + b
//     is Im becp[.][b].  Split-K over G across CTAs, deterministic partials.
//   out[k][b][G] (+)= sum_p beta[k][p][G] DB[k][p][b]                 (nonlocal_op.py:73-76)
//     D (128 x 128) = Bt (128 x K) Y^T: rows are 128 G of a tile, columns the real and
//     imaginary parts of 64 bands; K runs over (projector, re/im).
//
// Operands are written by the CTA's threads into shared memory in the canonical
// no-swizzle K-major layout (8-row x 16-byte core matrices; LBO = 128 B between the
// two core matrices of one K = 8 step, SBO = 256 B between 8-row groups), since the
// hi/lo split has to happen in registers on the way.  One thread issues the MMAs; a
// commit to an mbarrier tells the producers when the operand buffer is free again, and
// the next step's global loads are in flight (in registers) while the MMAs run.
// Every mbarrier wait has an iteration limit: on expiry the kernel records an error
// (read with addft_tc05_status), waits (bounded) for its own MMAs, frees its tensor
// memory and returns.
#include "common.cuh"

namespace addft {

namespace {

__device__ unsigned g_tc05_error = 0;   // bit 0: an mbarrier wait ran out

constexpr int kWaitLimit = 1 << 24;

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// tcgen05 shared-memory matrix descriptor: start address, LBO, SBO (bytes >> 4), the
// fixed 0b001 at bits 46-48, base offset 0, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | ((uint64_t)1 << 46);
}

// instruction descriptor, kind::tf32: F32 accumulator, TF32 A and B, both K-major, N and M.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
               : "memory");
}

__device__ __forceinline__ void bar_init(uint64_t *bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(bar)));
}

// Bounded wait for the completion of the mbarrier phase with this parity; false on timeout.
__device__ __forceinline__ bool bar_wait(uint64_t *bar, uint32_t parity) {
  for (int it = 0; it < kWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(saddr(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ uint32_t tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ void split4(const float (&x)[4], uint4 &hi, uint4 &lo) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    h[i] = tf32_rna(x[i]);
    l[i] = tf32_rna(x[i] - __uint_as_float(h[i]));
  }
  hi = make_uint4(h[0], h[1], h[2], h[3]);
  lo = make_uint4(l[0], l[1], l[2], l[3]);
}

__device__ __forceinline__ void sts128(uint32_t addr, uint4 v) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w)
               : "memory");
}

// byte offset of K-chunk kc (4 floats) of row r in a canonical tile of R rows, K = 8 per slice
__device__ __forceinline__ uint32_t coff(int R, int r, int k4) {
  const int slice = k4 >> 1, kc = k4 & 1;
  return (uint32_t)(slice * (R / 8) * 256 + (r >> 3) * 256 + kc * 128 + (r & 7) * 16);
}

__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(slot)), "r"(ncols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

#define TC05_LD32(taddr, r)                                                                                      \
  asm volatile(                                                                                                  \
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18," \
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"                                             \
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),          \
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),    \
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),  \
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])   \
      : "r"(taddr))

// ---------------------------------------------------------------------------
// becp
// ---------------------------------------------------------------------------
constexpr int kBB = 64;            // bands per tile (rows 0..63 and 64..127 of X)
constexpr int kBP = 32;            // projectors per tile (N)
constexpr int kBGs = 16;           // G per stage (K = 32 floats = 4 MMA steps)
constexpr int kXTile = 128 * 2 * kBGs * 4;   // bytes of one X tile (hi or lo): 16 KB
constexpr int kPTile = kBP * 2 * kBGs * 4;   // bytes of one P tile: 4 KB
constexpr int kStage = 2 * kXTile + 2 * kPTile;   // X hi, X lo, P hi, P lo
constexpr size_t kBecpSmem = 2 * (size_t)kStage + 1024;   // two stages in shared memory, one in registers

}  // namespace

__global__ void __launch_bounds__(128, 2)
k_becp_tc05(const float2 *__restrict__ proj, const float2 *__restrict__ psi, int nb, int nG, int nproj, int nsplit,
            int gchunk, float2 *__restrict__ out) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char *smem = smem_raw + ((1024 - (saddr(smem_raw) & 1023)) & 1023);
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int p0 = blockIdx.y * kBP, b0 = blockIdx.x * kBB;
  const int nkz = gridDim.z / nsplit;
  const int k = blockIdx.z / nsplit, sp = blockIdx.z - k * nsplit;
  const int ga = sp * gchunk, gb = min(nG, ga + gchunk);
  const float2 *Pk = proj + (size_t)k * nproj * nG;
  const float2 *Xk = psi + (size_t)k * nb * nG;
  if (tid == 0) {
    bar_init(&bars[0]);
    bar_init(&bars[1]);
  }
  if (warp == 0) tmem_alloc(&tslot, 32);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tslot;
  const uint32_t idesc = idesc_tf32(128, kBP);
  const int nst = (gb - ga + kBGs - 1) / kBGs;
  // producer mapping: lane -> row rl = lane % 8 of an 8-row group and G quarter gq = lane / 8.
  // A load instruction reads, per row, 4 consecutive G (32 B) from the 4 lanes rl, rl + 8,
  // rl + 16, rl + 24: 8 rows x one sector.  The lanes of a pair (gq, gq ^ 1) swap their
  // values, so both hold the two G of one 16-byte K chunk: the even lane writes the chunk,
  // the odd lane its (im, -re) rotation (X) or its lo part (P).  Each group of 8
  // consecutive lanes then writes 8 rows of one core matrix (128 contiguous bytes).
  // X: row groups warp and warp + 4 (bands), P: warp.
  const int rl = lane & 7, gq = lane >> 3, odd = gq & 1;
  int xr[2];
  bool xok[2];
  const float2 *xs[2];
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    xr[i] = 8 * (warp + 4 * i) + rl;
    xok[i] = b0 + xr[i] < nb;
    xs[i] = Xk + (size_t)(b0 + xr[i]) * nG;
  }
  const int pr = 8 * warp + rl;
  const bool pok = p0 + pr < nproj;
  const float2 *ps = Pk + (size_t)(p0 + pr) * nG;
  float2 xv[2][4], pv[4];
  auto load = [&](int s) {
    const int g0 = ga + s * kBGs + gq;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const bool gin = g0 + 4 * j < gb;
#pragma unroll
      for (int i = 0; i < 2; ++i) xv[i][j] = (xok[i] && gin) ? xs[i][g0 + 4 * j] : make_float2(0.f, 0.f);
      pv[j] = (pok && gin) ? ps[g0 + 4 * j] : make_float2(0.f, 0.f);
    }
  };
  // (even, odd) G of this lane's pair
  auto pair = [&](float2 v, float2 &e, float2 &o) {
    float2 w;
    w.x = __shfl_xor_sync(0xffffffffu, v.x, 8);
    w.y = __shfl_xor_sync(0xffffffffu, v.y, 8);
    e = odd ? w : v;
    o = odd ? v : w;
  };
  bool ok = true;
  if (nst > 0) load(0);
  for (int s = 0; s < nst && ok; ++s) {
    const int buf = s & 1;
    if (s >= 2) ok = __syncthreads_and(bar_wait(&bars[buf], ((s - 2) >> 1) & 1)) != 0;   // buffer free
    if (!ok) break;
    const uint32_t xhi = saddr(smem + buf * kStage), xlo = xhi + kXTile, phi = xhi + 2 * kXTile, plo = phi + kPTile;
#pragma unroll
    for (int j = 0; j < 4; ++j) {   // G 4 j .. 4 j + 3 of the stage: K chunks 2 j, 2 j + 1
      const int k4 = 2 * j + (gq >> 1);
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        float2 e, o;
        pair(xv[i][j], e, o);
        float a[4];
        if (odd) {   // (re, im) -> (im, -re), rows 64 + b
          a[0] = e.y; a[1] = -e.x; a[2] = o.y; a[3] = -o.x;
        } else {
          a[0] = e.x; a[1] = e.y; a[2] = o.x; a[3] = o.y;
        }
        uint4 hi, lo;
        split4(a, hi, lo);
        const uint32_t off = coff(128, xr[i] + 64 * odd, k4);
        sts128(xhi + off, hi);
        sts128(xlo + off, lo);
      }
      float2 e, o;
      pair(pv[j], e, o);
      float a[4] = {e.x, e.y, o.x, o.y};
      uint4 hi, lo;
      split4(a, hi, lo);
      sts128((odd ? plo : phi) + coff(kBP, pr, k4), odd ? lo : hi);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int kk = 0; kk < kBGs * 2 / 8; ++kk) {
        const uint64_t xh_ = sdesc(xhi + kk * (128 / 8) * 256, 128, 256);
        const uint64_t xl_ = sdesc(xlo + kk * (128 / 8) * 256, 128, 256);
        const uint64_t ph_ = sdesc(phi + kk * (kBP / 8) * 256, 128, 256);
        const uint64_t pl_ = sdesc(plo + kk * (kBP / 8) * 256, 128, 256);
        mma_tf32(tmem, xh_, ph_, idesc, (s > 0 || kk > 0) ? 1u : 0u);
        mma_tf32(tmem, xh_, pl_, idesc, 1u);
        mma_tf32(tmem, xl_, ph_, idesc, 1u);
      }
      commit(&bars[buf]);
    }
    if (s + 1 < nst) load(s + 1);   // next stage's operands in flight while the MMAs run
  }
  // the commit of the last stage covers every MMA this CTA issued
  bool fin = true;
  if (nst > 0) fin = __syncthreads_and(bar_wait(&bars[(nst - 1) & 1], ((nst - 1) >> 1) & 1)) != 0;
  const int row = 32 * warp + lane;
  const int b = b0 + (row & 63);
  float *o = reinterpret_cast<float *>(out + (((size_t)sp * nkz + k) * nproj + p0) * nb + b) + (row >> 6);
  if (!ok || !fin) {
    if (lane == 0) atomicOr(&g_tc05_error, 1u);
  } else if (nst > 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    uint32_t rr[32];
    TC05_LD32(tmem + ((uint32_t)(32 * warp) << 16), rr);
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    if (b < nb) {
#pragma unroll
      for (int j = 0; j < kBP; ++j)
        if (p0 + j < nproj) o[(size_t)j * nb * 2] = __uint_as_float(rr[j]);
    }
  } else if (b < nb) {
    for (int j = 0; j < kBP; ++j)
      if (p0 + j < nproj) o[(size_t)j * nb * 2] = 0.f;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) tmem_free(tmem, 32);
}

addft_status launch_becp_tc05(int nk, int nb, int nG, int nproj, int nsplit, int gchunk, const float2 *proj,
                              const float2 *psi, float2 *out, cudaStream_t st) {
  ADDFT_TRY(smem_optin(k_becp_tc05, kBecpSmem));
  dim3 grid((nb + kBB - 1) / kBB, (nproj + kBP - 1) / kBP, nk * nsplit);
  k_becp_tc05<<<grid, 128, kBecpSmem, st>>>(proj, psi, nb, nG, nproj, nsplit, gchunk, out);
  return check_launch("k_becp_tc05");
}

// ---------------------------------------------------------------------------
// V_NL apply: out[k][b][G] (+)= sum_j A[k][j][G] X[k][j][b]   (A = beta, X = D becp)
// ---------------------------------------------------------------------------
namespace {
constexpr int kAG = 128;   // G per tile (M)
constexpr int kAB = 64;    // bands per tile (N = 128: real parts, then imaginary parts)
constexpr int kAJ = 32;    // projectors per K chunk (K = 64 floats = 8 MMA steps)
constexpr int kATile = 128 * 2 * kAJ * 4;   // bytes of one 128-row operand tile: 32 KB
constexpr size_t kApplySmem = 4 * (size_t)kATile + 1024;   // A hi, A lo, B hi, B lo
}  // namespace

template <bool ACCUM>
__global__ void __launch_bounds__(256, 1)
k_apply_tc05(const float2 *__restrict__ X, int xs_j, int xs_i, size_t xs_k, const float2 *__restrict__ A,
             size_t as_k, int nj, int ni, int nG, float2 *__restrict__ out, size_t os_k) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char *smem = smem_raw + ((1024 - (saddr(smem_raw) & 1023)) & 1023);
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int b0 = blockIdx.y * kAB, k = blockIdx.z;
  const float2 *Ak = A + (size_t)k * as_k;
  const float2 *Xk = X + (size_t)k * xs_k;
  float2 *ok_ = out + (size_t)k * os_k;
  if (tid == 0) bar_init(&bar);
  if (warp == 0) tmem_alloc(&tslot, 128);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tslot;
  const uint32_t idesc = idesc_tf32(128, 128);
  const uint32_t ahi = saddr(smem), alo = ahi + kATile, bhi = alo + kATile, blo = bhi + kATile;
  const int nchunk = (nj + kAJ - 1) / kAJ;
  const int ntile = (nG + kAG - 1) / kAG;
  // operand rows: row r = tid % 128 of A (G) and B (band part), projector half ph = tid / 128
  const int r = tid & 127, ph = tid >> 7;
  constexpr int kH = kAJ / 2;   // projectors per thread and chunk
  // B row r: band b0 + (r & 63); r < 64: (Re X, -Im X) per projector, r >= 64: (Im X, Re X)
  const int bn = b0 + (r & 63);
  const bool bpart = r >= 64, bok = bn < ni;
  auto build_b = [&](int c) {
    float2 xv[kH];
#pragma unroll
    for (int jj = 0; jj < kH; ++jj) {
      const int j = c * kAJ + ph * kH + jj;
      xv[jj] = (bok && j < nj) ? Xk[(size_t)j * xs_j + (size_t)bn * xs_i] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int q = 0; q < kH / 2; ++q) {   // two projectors per 4-float K chunk
      float v[4];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float2 x = xv[2 * q + h];
        v[2 * h] = bpart ? x.y : x.x;
        v[2 * h + 1] = bpart ? x.x : -x.y;
      }
      uint4 hi, lo;
      split4(v, hi, lo);
      sts128(bhi + coff(128, r, ph * (kH / 2) + q), hi);
      sts128(blo + coff(128, r, ph * (kH / 2) + q), lo);
    }
  };
  float2 av[kH];   // this thread's A values of the next (tile, chunk), loaded ahead
  auto load_a = [&](int t, int c) {
    const int g = t * kAG + r;
#pragma unroll
    for (int jj = 0; jj < kH; ++jj) {
      const int j = c * kAJ + ph * kH + jj;
      av[jj] = (g < nG && j < nj) ? Ak[(size_t)j * nG + g] : make_float2(0.f, 0.f);
    }
  };
  bool ok = true;
  int ncommit = 0;
  if (nchunk == 1) build_b(0);
  if (blockIdx.x < ntile) load_a(blockIdx.x, 0);
  // epilogue mapping: warp w reads D lanes 32 (w % 4) .. (rows = G), band half bh = w / 4
  const int bh = warp >> 2;
  for (int t = blockIdx.x; t < ntile && ok; t += gridDim.x) {
    for (int c = 0; c < nchunk && ok; ++c) {
      if (ncommit > 0) ok = __syncthreads_and(bar_wait(&bar, (ncommit - 1) & 1)) != 0;   // operands free
      if (!ok) break;
      if (nchunk > 1) build_b(c);
#pragma unroll
      for (int q = 0; q < kH / 2; ++q) {
        float v[4] = {av[2 * q].x, av[2 * q].y, av[2 * q + 1].x, av[2 * q + 1].y};
        uint4 hi, lo;
        split4(v, hi, lo);
        sts128(ahi + coff(128, r, ph * (kH / 2) + q), hi);
        sts128(alo + coff(128, r, ph * (kH / 2) + q), lo);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
        for (int kk = 0; kk < kAJ * 2 / 8; ++kk) {
          const uint64_t ah = sdesc(ahi + kk * 16 * 256, 128, 256), al = sdesc(alo + kk * 16 * 256, 128, 256);
          const uint64_t bh_ = sdesc(bhi + kk * 16 * 256, 128, 256), bl = sdesc(blo + kk * 16 * 256, 128, 256);
          mma_tf32(tmem, ah, bh_, idesc, (c > 0 || kk > 0) ? 1u : 0u);
          mma_tf32(tmem, ah, bl, idesc, 1u);
          mma_tf32(tmem, al, bh_, idesc, 1u);
        }
        commit(&bar);
      }
      ++ncommit;
      // next operands in flight while the MMAs run
      if (c + 1 < nchunk) load_a(t, c + 1);
      else if (t + (int)gridDim.x < ntile) load_a(t + gridDim.x, 0);
    }
    if (!ok) break;
    const int row = t * kAG + 32 * (warp & 3) + lane;   // D row (G) of this thread
    float2 w[32];   // old values, read before the accumulator is waited for
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const int b = b0 + 32 * bh + j;
      w[j] = (ACCUM && b < ni && row < nG) ? ok_[(size_t)b * nG + row] : make_float2(0.f, 0.f);
    }
    ok = __syncthreads_and(bar_wait(&bar, (ncommit - 1) & 1)) != 0;   // accumulator complete
    if (!ok) break;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    uint32_t re[32], im[32];
    TC05_LD32(tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(32 * bh), re);
    TC05_LD32(tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(64 + 32 * bh), im);
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    if (row < nG) {
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int b = b0 + 32 * bh + j;
        if (b < ni)
          ok_[(size_t)b * nG + row] = make_float2(__uint_as_float(re[j]) + w[j].x, __uint_as_float(im[j]) + w[j].y);
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  if (!ok) {
    if (tid == 0 && ncommit > 0) commit(&bar);   // one more commit tracks every MMA issued
    bar_wait(&bar, ncommit & 1);
    if (lane == 0) atomicOr(&g_tc05_error, 1u);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) tmem_free(tmem, 128);
}

addft_status launch_apply_tc05(bool accum, const float2 *X, int xs_j, int xs_i, size_t xs_k, const float2 *A,
                               size_t as_k, int nk, int nj, int ni, int nG, float2 *out, size_t os_k,
                               cudaStream_t st) {
  ADDFT_TRY(smem_optin(accum ? k_apply_tc05<true> : k_apply_tc05<false>, kApplySmem));
  int dev = 0, nsm = 0;
  ADDFT_CUDA(cudaGetDevice(&dev));
  ADDFT_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int nbt = (ni + kAB - 1) / kAB, ntile = (nG + kAG - 1) / kAG;
  int gx = (nsm + nbt * nk - 1) / (nbt * nk);   // about one CTA per SM over the whole grid
  if (gx > ntile) gx = ntile;
  if (gx < 1) gx = 1;
  dim3 grid(gx, nbt, nk);
  if (accum)
    k_apply_tc05<true><<<grid, 256, kApplySmem, st>>>(X, xs_j, xs_i, xs_k, A, as_k, nj, ni, nG, out, os_k);
  else
    k_apply_tc05<false><<<grid, 256, kApplySmem, st>>>(X, xs_j, xs_i, xs_k, A, as_k, nj, ni, nG, out, os_k);
  return check_launch("k_apply_tc05");
}

// ---------------------------------------------------------------------------
// Peak rate of kind::tf32 MMAs: one CTA per SM, one thread issues `iters` MMAs of
// 128 x 256 x 8 on fixed shared-memory operands into one tensor-memory accumulator,
// then waits (bounded) for their completion.  Diagnostic for the compute roof.
// ---------------------------------------------------------------------------
namespace {
constexpr int kPeakN = 256;
}  // namespace

__global__ void __launch_bounds__(128, 1) k_peak_tc05(int iters) {
  __shared__ __align__(128) unsigned char a_s[128 * 32];
  __shared__ __align__(128) unsigned char b_s[kPeakN * 32];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int i = tid; i < (int)sizeof(a_s) / 4; i += blockDim.x) reinterpret_cast<float *>(a_s)[i] = 1e-3f;
  for (int i = tid; i < (int)sizeof(b_s) / 4; i += blockDim.x) reinterpret_cast<float *>(b_s)[i] = 1e-3f;
  if (tid == 0) bar_init(&bar);
  if (warp == 0) tmem_alloc(&tslot, kPeakN);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tslot;
  if (tid == 0) {
    const uint64_t ad = sdesc(saddr(a_s), 128, 256), bd = sdesc(saddr(b_s), 128, 256);
    const uint32_t idesc = idesc_tf32(128, kPeakN);
    for (int it = 0; it < iters; ++it) mma_tf32(tmem, ad, bd, idesc, it > 0 ? 1u : 0u);
    commit(&bar);
  }
  __syncthreads();   // the issuing loop is finite; only the MMAs still queued remain
  const bool ok = __syncthreads_and(bar_wait(&bar, 0)) != 0;
  if (!ok && tid == 0) atomicOr(&g_tc05_error, 1u);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) tmem_free(tmem, kPeakN);
}

// Launches k_peak_tc05 on every SM (warm-up, then a timed launch); *tflops and *ms of the
// timed launch.  Synchronises with the stream.
addft_status peak_tc05(int iters, double *tflops, float *ms, cudaStream_t st) {
  int dev = 0, nsm = 0;
  ADDFT_CUDA(cudaGetDevice(&dev));
  ADDFT_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  k_peak_tc05<<<nsm, 128, 0, st>>>(iters / 16 + 1);
  ADDFT_TRY(check_launch("k_peak_tc05 (warm-up)"));
  cudaEvent_t e0, e1;
  ADDFT_CUDA(cudaEventCreate(&e0));
  ADDFT_CUDA(cudaEventCreate(&e1));
  ADDFT_CUDA(cudaEventRecord(e0, st));
  k_peak_tc05<<<nsm, 128, 0, st>>>(iters);
  const addft_status s = check_launch("k_peak_tc05");
  ADDFT_CUDA(cudaEventRecord(e1, st));
  ADDFT_CUDA(cudaEventSynchronize(e1));
  float t = 0.f;
  ADDFT_CUDA(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ADDFT_TRY(s);
  *ms = t;
  *tflops = (double)nsm * iters * 2.0 * 128 * kPeakN * 8 / (t * 1e-3) / 1e12;
  return ADDFT_OK;
}

}  // namespace addft

extern "C" {

// Bit set of device-side errors of the tcgen05 kernels since the last call (bit 0: an
// mbarrier wait ran out); reading clears it.  Synchronises with the device.
unsigned addft_tc05_status(void) {
  unsigned v = 0, z = 0;
  if (cudaMemcpyFromSymbol(&v, addft::g_tc05_error, sizeof(v)) != cudaSuccess) return 0xffffffffu;
  cudaMemcpyToSymbol(addft::g_tc05_error, &z, sizeof(z));
  return v;
}

}  // extern "C"
