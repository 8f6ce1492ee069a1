// Shared definitions of the GB300 plane-wave kernels: complex helpers, the
// device-side plan descriptor, status / error plumbing.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "../../include/addft_gb300.h"

namespace addft {

// ----------------------------------------------------------------------------
// complex arithmetic on float2 / double2
// ----------------------------------------------------------------------------
template <typename R> struct Cx;
template <> struct Cx<float> { using T = float2; };
template <> struct Cx<double> { using T = double2; };

template <typename C> __host__ __device__ __forceinline__ C mk(double x, double y) {
  C c; c.x = (decltype(c.x))x; c.y = (decltype(c.y))y; return c;
}
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
__host__ __device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__host__ __device__ __forceinline__ double2 cmulc(double2 a, double2 b) {
  return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__host__ __device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
// multiply by -i  (x + iy)(-i) = y - ix
__host__ __device__ __forceinline__ float2 cmul_mi(float2 a) { return make_float2(a.y, -a.x); }
__host__ __device__ __forceinline__ double2 cmul_mi(double2 a) { return make_double2(a.y, -a.x); }
__host__ __device__ __forceinline__ float2 czero_f() { return make_float2(0.f, 0.f); }
template <typename C> __host__ __device__ __forceinline__ C czero() { C c; c.x = 0; c.y = 0; return c; }

// ----------------------------------------------------------------------------
// cp.async (global -> shared, bypassing registers) for 8- and 16-byte elements;
// an invalid element is zero-filled (source size 0, nothing is read).
// ----------------------------------------------------------------------------
template <typename C>
__device__ __forceinline__ void cp_async_el(C *smem_dst, const C *gmem_src, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  const int n = valid ? (int)sizeof(C) : 0;
  if constexpr (sizeof(C) == 16) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem_src), "r"(n));
  } else {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem_src), "r"(n));
  }
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

// ----------------------------------------------------------------------------
// FFT axis plan: length and its radix factorisation (radices 2, 3, 4, 5)
// ----------------------------------------------------------------------------
constexpr int kMaxStages = 12;
struct AxisPlan {
  int n;
  int nst;
  int rad[kMaxStages];
};

// Launch tunables of the FFT pipeline (host side): threads per CTA of the
// generic plane and x-line kernels, the shared-memory budget of a generic
// x-line tile, the slab bytes per band chunk, and whether the two-pass
// register kernels are used where they are instantiated.  Process defaults
// come from ADDFT_FFT_THREADS, ADDFT_FFT_THREADS_X, ADDFT_XTILE_KB,
// ADDFT_SLAB_MB, ADDFT_XLINE2, ADDFT_PLANE2, ADDFT_PLANE2_THREADS; each plan
// carries its own copy.
struct FftTuning {
  int threads_plane;
  int threads_x;
  int xtile_kb;
  size_t slab_chunk_bytes;
  int xline2;
  int plane2;
  int threads_plane2;  // threads per CTA of the two-pass plane kernels
  int colfft;          // 1: H psi through the column pipeline where instantiated
  int threads_xy;      // threads per CTA of the xy-plane kernel (0: default, 256)
  int xy_direct;       // 1: xy-plane kernel loads / stores columns directly where the shell allows
  int plane_split;     // 1: z / y plane stages as separate column-group and y-tile kernels on every box
                       // (0: only where the yz-plane tiles exceed a CTA's shared memory)
};

// Device view of a plan: sphere-aware layout of one G-shell in one FFT box.
//   planes p = 0..np-1 are the x-planes (fixed i1) that hold sphere points;
//   each plane owns a contiguous range [gptr[p], gptr[p+1]) of the
//   plane-sorted sphere list (sp_g = original G index, sp_pos = i2*n3 + i3)
//   and a range [rptr[p], rptr[p+1]) of active rows (row_i2 = i2).
struct PlanDev {
  int n1, n2, n3, nG, np, nrows;
  const int *sp_g;
  const int *sp_pos;
  const int *gptr;
  const int *plane_i1;
  const int *rptr;
  const int *row_i2;
  const int *plane_of_i1;  // n1 entries, -1 for empty planes
  const int *miller;       // nG*3 (original order), unwrapped integers
  // column pipeline: a column is an (i1, i2) pair holding sphere points; columns
  // are the rows above (row_i2, in plane order), ncols = nrows, padded to ncols_pad
  int ncols_pad;           // multiple of kColGroup
  const int *cgptr;        // ncols_pad / kColGroup + 1: first sorted point of each column group
  const int *pt_pos;       // nG: i3 * kColPitch + (column % kColGroup) of each sorted point
  const int *col_xy;       // ncols: i1 * (n2 | 1) + i2 of each column (xy tile position)
  // xy_direct = 1 when every active x-plane's columns are i2 = 0 .. nlo-1 and n2-nhi .. n2-1
  // (true for spheres around G = 0): row_lohi[p] = nlo | nhi << 16
  int xy_direct;
  const int *row_lohi;
  const void *tw_d;        // double2 twiddles: n1 | n2 | n3, e^{-2 pi i t/n}
  const void *tw_f;        // float2 twiddles, same layout
  AxisPlan ax[3];
  FftTuning tun;           // launch tunables (read on the host only)
};

constexpr int kColGroup = 32;   // columns per CTA of the z-column kernels
constexpr int kColPitch = 33;   // z-row pitch of their shared tiles (odd: z-strided scatter is conflict-free)

// ----------------------------------------------------------------------------
// status / error string
// ----------------------------------------------------------------------------
void set_error(const char *fmt, ...);
addft_status check_launch(const char *what);

#define ADDFT_REQUIRE(cond, code, ...)   \
  do {                                   \
    if (!(cond)) {                       \
      ::addft::set_error(__VA_ARGS__);   \
      return (code);                     \
    }                                    \
  } while (0)

#define ADDFT_CUDA(call)                                                         \
  do {                                                                           \
    cudaError_t _e = (call);                                                     \
    if (_e != cudaSuccess) {                                                     \
      ::addft::set_error("%s failed: %s", #call, cudaGetErrorString(_e));        \
      return ADDFT_CUDA_ERROR;                                                   \
    }                                                                            \
  } while (0)

#define ADDFT_TRY(expr)                  \
  do {                                   \
    addft_status _s = (expr);            \
    if (_s != ADDFT_OK) return _s;       \
  } while (0)

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Raises the dynamic shared-memory limit of a kernel on the current device (per launch).
template <typename K>
inline addft_status smem_optin(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return ADDFT_OK;
  int dev = 0, maxb = 0;
  ADDFT_CUDA(cudaGetDevice(&dev));
  ADDFT_CUDA(cudaDeviceGetAttribute(&maxb, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  ADDFT_REQUIRE((size_t)maxb >= bytes, ADDFT_UNSUPPORTED,
                "kernel needs %zu B shared memory, device allows %d B", bytes, maxb);
  ADDFT_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return ADDFT_OK;
}

// Deterministic two-pass reductions: blocks write partial sums, one block adds them.
constexpr int kRedBlocks = 304;   // 2 x 152 SMs
constexpr int kRedThreads = 256;

template <int NV>
__device__ __forceinline__ void block_reduce_store(double (&v)[NV], double *partial) {
  // partial layout: [NV][gridDim.x]
  __shared__ double red[32][NV];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double x = v[j];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][j] = x;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double x = lane < nw ? red[lane][j] : 0.0;
      for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
      if (lane == 0) partial[(size_t)j * gridDim.x + blockIdx.x] = x;
    }
  }
}

// Sums partial[NV][nblk] into out[j] (accumulate if acc, else overwrite).  One block.
__global__ void k_finalize_sums(const double *partial, int nv, int nblk, double *out, int acc);

addft_status finalize_sums(const double *partial, int nv, int nblk, double *out, bool acc,
                           cudaStream_t st);

}  // namespace addft

struct addft_plan_s {
  addft::PlanDev dev;
  int ncols;
  void *blob;   // single device allocation holding all tables
  int device;
};
