// Arithmetic peaks of this GPU, measured by kernels that do nothing else: the
// denominators of the compute roofline of the FFT (FP32 FMA) and projector
// (tensor-core) kernels.  No counterpart in the reference.
//
//   fp32 FMA:  every thread runs 8 independent FFMA chains (no memory traffic),
//   fp64 FMA:  the same with DFMA,
//   tf32 mma:  every warp runs 4 independent mma.sync.m16n8k8 TF32 chains (the
//              warp MMA of the split-TF32 becp kernel),
//   tf32 tcgen05: one thread per SM issues tcgen05.mma kind::tf32 128 x 256 x 8 into
//              tensor memory (the MMA of the V_NL apply kernel; tc05.cu).
// Grids are 8 CTAs of 256 threads per SM.  The result stays live through a
// data-dependent store so the loops are not removed.
#include "common.cuh"

namespace addft {

addft_status peak_tc05(int iters, double *tflops, float *ms, cudaStream_t st);   // tc05.cu


__global__ void __launch_bounds__(256) k_peak_fp32(int iters, float seed, float *sink) {
  float a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = seed + (float)(threadIdx.x + j);
  const float m = 0.999999f, c = 1e-7f;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < 16; ++u)
#pragma unroll
      for (int j = 0; j < 8; ++j) a[j] = fmaf(a[j], m, c);
  }
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += a[j];
  if (s == 12345.678f) sink[threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) k_peak_fp64(int iters, double seed, double *sink) {
  double a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = seed + (double)(threadIdx.x + j);
  const double m = 0.999999999, c = 1e-12;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < 16; ++u)
#pragma unroll
      for (int j = 0; j < 8; ++j) a[j] = fma(a[j], m, c);
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += a[j];
  if (s == 12345.678) sink[threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) k_peak_tf32_mma(int iters, float seed, float *sink) {
  float d[4][4];
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int e = 0; e < 4; ++e) d[j][e] = 0.f;
  uint32_t a[4], b[2];
#pragma unroll
  for (int e = 0; e < 4; ++e) a[e] = __float_as_uint(seed + 0.001f * (float)(threadIdx.x + e));
  b[0] = __float_as_uint(seed * 0.5f);
  b[1] = __float_as_uint(seed * 0.25f + 1e-3f * (float)threadIdx.x);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int j = 0; j < 4; ++j)
        asm volatile(
            "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
            "{%0,%1,%2,%3};\n"
            : "+f"(d[j][0]), "+f"(d[j][1]), "+f"(d[j][2]), "+f"(d[j][3])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
  }
  float s = 0.f;
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int e = 0; e < 4; ++e) s += d[j][e];
  if (s == 12345.678f) sink[threadIdx.x] = s;
}

}  // namespace addft

using namespace addft;

extern "C" {

addft_status addft_peak_flops(int which, int iters, double *tflops, float *ms, void *sink, void *stream) {
  ADDFT_REQUIRE(tflops && ms && sink && iters > 0 && which >= 0 && which <= 3, ADDFT_INVALID_ARG,
                "peak_flops: bad arguments");
  cudaStream_t st = as_stream(stream);
  if (which == 3) return peak_tc05(iters, tflops, ms, st);
  int dev = 0, nsm = 0;
  ADDFT_CUDA(cudaGetDevice(&dev));
  ADDFT_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = 8 * nsm, threads = 256;
  auto launch = [&](int n) {
    if (which == 0) k_peak_fp32<<<blocks, threads, 0, st>>>(n, 1.0f, (float *)sink);
    else if (which == 1) k_peak_fp64<<<blocks, threads, 0, st>>>(n, 1.0, (double *)sink);
    else k_peak_tf32_mma<<<blocks, threads, 0, st>>>(n, 1.0f, (float *)sink);
  };
  launch(iters / 16 + 1);   // warm-up
  ADDFT_TRY(check_launch("k_peak (warm-up)"));
  cudaEvent_t e0, e1;
  ADDFT_CUDA(cudaEventCreate(&e0));
  ADDFT_CUDA(cudaEventCreate(&e1));
  ADDFT_CUDA(cudaEventRecord(e0, st));
  launch(iters);
  addft_status s = check_launch("k_peak");
  ADDFT_CUDA(cudaEventRecord(e1, st));
  ADDFT_CUDA(cudaEventSynchronize(e1));
  float t = 0.f;
  ADDFT_CUDA(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ADDFT_TRY(s);
  const double threads_total = (double)blocks * threads;
  double flops;
  if (which == 2)   // per warp: 16 mma of m16n8k8 per iteration, 2 * 16 * 8 * 8 flops each
    flops = threads_total / 32.0 * iters * 16.0 * 2.0 * 16 * 8 * 8;
  else              // per thread: 128 FMA per iteration
    flops = threads_total * iters * 128.0 * 2.0;
  *ms = t;
  *tflops = flops / (t * 1e-3) / 1e12;
  return ADDFT_OK;
}

}  // extern "C"
