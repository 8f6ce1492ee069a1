// Entry points with the argument meaning of the reference's XLA FFI handlers, so a
// maintainer can bind each handler to one call of this library with no glue beyond
// unpacking the FFI buffers:
//
//   XcLdaHandler        native/xc_lda.cu:56-75   -> addft_ffi_xc_lda
//   ScatterC128Handler  native/pack.cu:43-66     -> addft_ffi_scatter (ADDFT_F64)
//   GatherC128Handler   native/pack.cu:68-87     -> addft_ffi_gather  (ADDFT_F64)
//   Scatter/GatherC64   native/pack.cu:101-189   -> the same with ADDFT_F32
//   EighLowestHandler   native/eigh.cu:55-160    -> addft_ffi_eigh_lowest
//
// Differences from the handlers, all in how memory is obtained: scratch comes from the
// caller (the *_work_bytes functions size it) instead of cudaMallocAsync, and the XC
// energy sum is reduced deterministically (block partials summed in a fixed order)
// instead of by atomicAdd.  cuSOLVER is opened with dlopen on the first eigensolver
// call, so the library itself has no link-time dependency on it.
#include <dlfcn.h>

#include <mutex>

#include <cusolverDn.h>

#include "xc.cuh"

namespace addft {
namespace {

// v_xc and sum n (eps_x + eps_c) at the clamped density max(rho, 1e-14), as the
// native handler computes them (xc_lda.cu:28-45).
__global__ void __launch_bounds__(kRedThreads)
k_ffi_xc(int n, const double *__restrict__ rho, double *__restrict__ vxc, double *__restrict__ partial) {
  double acc[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const XcPoint x = pz81(rho[i]);
    vxc[i] = x.vn;
    acc[0] += fmax(rho[i], 1e-14) * (x.ex + x.ec);
  }
  block_reduce_store<1>(acc, partial);
}

template <typename C>
__global__ void k_ffi_scatter(const C *__restrict__ coeffs, const int *__restrict__ idx, C *__restrict__ out,
                              int batch, int nG, int nfft) {
  const long total = (long)batch * nG;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const int b = (int)(t / nG), i = (int)(t - (long)b * nG);
    const int j = idx[i];
    if ((unsigned)j < (unsigned)nfft) out[(size_t)b * nfft + j] = coeffs[t];   // out-of-range: skipped
  }
}

template <typename C>
__global__ void k_ffi_gather(const C *__restrict__ grid, const int *__restrict__ idx, C *__restrict__ out,
                             int batch, int nG, int nfft) {
  const long total = (long)batch * nG;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const int b = (int)(t / nG), i = (int)(t - (long)b * nG);
    const int j = idx[i];
    C v;
    v.x = 0;
    v.y = 0;
    if ((unsigned)j < (unsigned)nfft) v = grid[(size_t)b * nfft + j];   // out-of-range: zero
    out[t] = v;
  }
}

// Flags every index outside [0, nfft) (one int, 0 = all in range).
__global__ void k_ffi_check_idx(const int *__restrict__ idx, int nG, int nfft, int *__restrict__ bad) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nG; i += gridDim.x * blockDim.x)
    if (idx[i] < 0 || idx[i] >= nfft) *bad = 1;
}

// The lowest nband eigenpairs of every k from cuSOLVER's column-major output.  The
// solver saw the row-major input as its transpose conj(H), whose eigenvectors are the
// conjugates of H's, so the extraction conjugates them back.
__global__ void k_ffi_extract(const double2 *__restrict__ A, const double *__restrict__ W, double *__restrict__ eig,
                              double2 *__restrict__ vec, int n, int nband, int nk) {
  const long total = (long)nk * nband * n;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    const int k = (int)(t / ((long)nband * n));
    const long rem = t - (long)k * nband * n;
    const int i = (int)(rem / n), j = (int)(rem - (long)i * n);
    const double2 a = A[(size_t)k * n * n + (size_t)i * n + j];
    vec[t] = make_double2(a.x, -a.y);
    if (j == 0) eig[(size_t)k * nband + i] = W[(size_t)k * n + i];
  }
}

inline int grid_for(long total) { return (int)std::min<long>((total + 255) / 256, 8 * 152); }
inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

// cuSOLVER, opened on first use.
struct Solver {
  using create_t = cusolverStatus_t (*)(cusolverDnHandle_t *);
  using stream_t = cusolverStatus_t (*)(cusolverDnHandle_t, cudaStream_t);
  using bufsize_t = cusolverStatus_t (*)(cusolverDnHandle_t, cusolverEigMode_t, cublasFillMode_t, int,
                                         const cuDoubleComplex *, int, const double *, int *);
  using heevd_t = cusolverStatus_t (*)(cusolverDnHandle_t, cusolverEigMode_t, cublasFillMode_t, int,
                                       cuDoubleComplex *, int, double *, cuDoubleComplex *, int, int *);
  void *lib = nullptr;
  create_t create = nullptr;
  stream_t set_stream = nullptr;
  bufsize_t bufsize = nullptr;
  heevd_t heevd = nullptr;
  char err[256] = {0};
};

Solver &solver() {
  static Solver s;
  static std::once_flag once;
  std::call_once(once, [] {
    const char *names[] = {"libcusolver.so.12", "libcusolver.so", "/usr/local/cuda/lib64/libcusolver.so.12"};
    for (const char *nm : names) {
      s.lib = dlopen(nm, RTLD_NOW | RTLD_LOCAL);
      if (s.lib) break;
    }
    if (!s.lib) {
      snprintf(s.err, sizeof(s.err), "cannot open libcusolver: %s", dlerror());
      return;
    }
    s.create = (Solver::create_t)dlsym(s.lib, "cusolverDnCreate");
    s.set_stream = (Solver::stream_t)dlsym(s.lib, "cusolverDnSetStream");
    s.bufsize = (Solver::bufsize_t)dlsym(s.lib, "cusolverDnZheevd_bufferSize");
    s.heevd = (Solver::heevd_t)dlsym(s.lib, "cusolverDnZheevd");
    if (!s.create || !s.set_stream || !s.bufsize || !s.heevd)
      snprintf(s.err, sizeof(s.err), "libcusolver lacks a cusolverDn Zheevd symbol");
  });
  return s;
}

// One cuSOLVER handle per (host thread, device), created on first use and kept.
addft_status solver_handle(cusolverDnHandle_t *out) {
  Solver &s = solver();
  ADDFT_REQUIRE(s.err[0] == 0, ADDFT_UNSUPPORTED, "ffi_eigh_lowest: %s", s.err);
  constexpr int kDev = 64;
  static thread_local cusolverDnHandle_t h[kDev] = {};
  int dev = 0;
  ADDFT_CUDA(cudaGetDevice(&dev));
  ADDFT_REQUIRE(dev >= 0 && dev < kDev, ADDFT_UNSUPPORTED, "ffi_eigh_lowest: device index %d >= %d", dev, kDev);
  if (!h[dev]) {
    const cusolverStatus_t e = s.create(&h[dev]);
    ADDFT_REQUIRE(e == CUSOLVER_STATUS_SUCCESS, ADDFT_CUDA_ERROR, "cusolverDnCreate failed (%d)", (int)e);
  }
  *out = h[dev];
  return ADDFT_OK;
}

}  // namespace
}  // namespace addft

using namespace addft;

extern "C" {

size_t addft_ffi_xc_lda_work_bytes(void) { return kRedBlocks * sizeof(double); }

addft_status addft_ffi_xc_lda(int n, const double *rho, double *vxc, double *exc, void *work, size_t work_bytes,
                              void *stream) {
  ADDFT_REQUIRE(n >= 0 && exc && (n == 0 || (rho && vxc)), ADDFT_INVALID_ARG, "ffi_xc_lda: bad arguments");
  ADDFT_REQUIRE(work && work_bytes >= addft_ffi_xc_lda_work_bytes(), ADDFT_INVALID_ARG,
                "ffi_xc_lda: work needs %zu B", addft_ffi_xc_lda_work_bytes());
  cudaStream_t st = as_stream(stream);
  double *part = (double *)work;
  k_ffi_xc<<<kRedBlocks, kRedThreads, 0, st>>>(n, rho, vxc, part);
  ADDFT_TRY(check_launch("k_ffi_xc"));
  return finalize_sums(part, 1, kRedBlocks, exc, false, st);
}

addft_status addft_ffi_scatter(addft_dtype dt, int batch, int nG, int nfft, const void *coeffs, const int *idx,
                               void *out, void *stream) {
  ADDFT_REQUIRE(batch >= 0 && nG >= 0 && nfft >= 1, ADDFT_INVALID_ARG, "ffi_scatter: bad sizes");
  ADDFT_REQUIRE((long)batch * nfft < (1L << 31) && (long)batch * nG < (1L << 31), ADDFT_UNSUPPORTED,
                "ffi_scatter: batch x nfft must stay below 2^31 elements");
  if (batch == 0) return ADDFT_OK;
  ADDFT_REQUIRE(out && (nG == 0 || (coeffs && idx)), ADDFT_INVALID_ARG, "ffi_scatter: null pointer");
  cudaStream_t st = as_stream(stream);
  const size_t csz = dt == ADDFT_F64 ? 16 : 8;
  ADDFT_CUDA(cudaMemsetAsync(out, 0, (size_t)batch * nfft * csz, st));
  if (nG == 0) return ADDFT_OK;
  const int g = grid_for((long)batch * nG);
  if (dt == ADDFT_F64)
    k_ffi_scatter<double2><<<g, 256, 0, st>>>((const double2 *)coeffs, idx, (double2 *)out, batch, nG, nfft);
  else
    k_ffi_scatter<float2><<<g, 256, 0, st>>>((const float2 *)coeffs, idx, (float2 *)out, batch, nG, nfft);
  return check_launch("k_ffi_scatter");
}

addft_status addft_ffi_gather(addft_dtype dt, int batch, int nG, int nfft, const void *grid, const int *idx,
                              void *out, void *stream) {
  ADDFT_REQUIRE(batch >= 0 && nG >= 0 && nfft >= 1, ADDFT_INVALID_ARG, "ffi_gather: bad sizes");
  ADDFT_REQUIRE((long)batch * nfft < (1L << 31) && (long)batch * nG < (1L << 31), ADDFT_UNSUPPORTED,
                "ffi_gather: batch x nfft must stay below 2^31 elements");
  if (batch == 0 || nG == 0) return ADDFT_OK;
  ADDFT_REQUIRE(grid && idx && out, ADDFT_INVALID_ARG, "ffi_gather: null pointer");
  cudaStream_t st = as_stream(stream);
  const int g = grid_for((long)batch * nG);
  if (dt == ADDFT_F64)
    k_ffi_gather<double2><<<g, 256, 0, st>>>((const double2 *)grid, idx, (double2 *)out, batch, nG, nfft);
  else
    k_ffi_gather<float2><<<g, 256, 0, st>>>((const float2 *)grid, idx, (float2 *)out, batch, nG, nfft);
  return check_launch("k_ffi_gather");
}

addft_status addft_ffi_check_index(int nG, int nfft, const int *idx, int *bad, void *stream) {
  ADDFT_REQUIRE(nG >= 0 && nfft >= 1 && bad && (nG == 0 || idx), ADDFT_INVALID_ARG,
                "ffi_check_index: bad arguments");
  cudaStream_t st = as_stream(stream);
  ADDFT_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), st));
  if (nG == 0) return ADDFT_OK;
  k_ffi_check_idx<<<grid_for(nG), 256, 0, st>>>(idx, nG, nfft, bad);
  return check_launch("k_ffi_check_idx");
}

size_t addft_ffi_eigh_lowest_work_bytes(int nk, int n) {
  if (nk < 1 || n < 1) return 0;
  cusolverDnHandle_t h = nullptr;
  if (solver_handle(&h) != ADDFT_OK) return 0;
  int lwork = 0;
  if (solver().bufsize(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, nullptr, n, nullptr, &lwork) !=
      CUSOLVER_STATUS_SUCCESS)
    return 0;
  return al256((size_t)nk * n * n * sizeof(double2)) + al256((size_t)nk * n * sizeof(double)) +
         al256((size_t)nk * sizeof(int)) + al256((size_t)lwork * sizeof(double2));
}

addft_status addft_ffi_eigh_lowest(int nk, int n, int nband, const void *H, double *eig, void *vec, void *work,
                                   size_t work_bytes, void *stream) {
  ADDFT_REQUIRE(nk >= 0 && n >= 1 && nband >= 0, ADDFT_INVALID_ARG, "ffi_eigh_lowest: bad sizes");
  ADDFT_REQUIRE(nband <= n, ADDFT_INVALID_ARG, "ffi_eigh_lowest: nband (%d) > n (%d)", nband, n);
  if (nk == 0 || nband == 0) return ADDFT_OK;
  ADDFT_REQUIRE(H && eig && vec && work, ADDFT_INVALID_ARG, "ffi_eigh_lowest: null pointer");
  cusolverDnHandle_t h = nullptr;
  ADDFT_TRY(solver_handle(&h));
  Solver &s = solver();
  cudaStream_t st = as_stream(stream);
  int lwork = 0;
  cusolverStatus_t e =
      s.bufsize(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, nullptr, n, nullptr, &lwork);
  ADDFT_REQUIRE(e == CUSOLVER_STATUS_SUCCESS, ADDFT_CUDA_ERROR, "zheevd_bufferSize failed (%d)", (int)e);
  const size_t o_w = al256((size_t)nk * n * n * sizeof(double2));
  const size_t o_info = o_w + al256((size_t)nk * n * sizeof(double));
  const size_t o_lw = o_info + al256((size_t)nk * sizeof(int));
  const size_t need = o_lw + al256((size_t)lwork * sizeof(double2));
  ADDFT_REQUIRE(work_bytes >= need, ADDFT_INVALID_ARG, "ffi_eigh_lowest: work needs %zu B, got %zu B", need,
                work_bytes);
  char *w = (char *)work;
  double2 *A = (double2 *)w;
  double *W = (double *)(w + o_w);
  int *info = (int *)(w + o_info);
  cuDoubleComplex *lw = (cuDoubleComplex *)(w + o_lw);
  ADDFT_CUDA(cudaMemcpyAsync(A, H, (size_t)nk * n * n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  e = s.set_stream(h, st);
  ADDFT_REQUIRE(e == CUSOLVER_STATUS_SUCCESS, ADDFT_CUDA_ERROR, "cusolverDnSetStream failed (%d)", (int)e);
  for (int k = 0; k < nk; ++k) {
    e = s.heevd(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, (cuDoubleComplex *)(A + (size_t)k * n * n),
                n, W + (size_t)k * n, lw, lwork, info + k);
    ADDFT_REQUIRE(e == CUSOLVER_STATUS_SUCCESS, ADDFT_CUDA_ERROR, "zheevd failed at k = %d (%d)", k, (int)e);
  }
  k_ffi_extract<<<grid_for((long)nk * nband * n), 256, 0, st>>>(A, W, eig, (double2 *)vec, n, nband, nk);
  return check_launch("k_ffi_extract");
}

}  // extern "C"
