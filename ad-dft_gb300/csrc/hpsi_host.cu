// H psi of bands that live in host memory, with the copies overlapped with the compute.
//
// A caller that keeps its wavefunctions on the host (the reference's CPU path hands
// NumPy arrays to the kernels) pays for the host -> device copy of psi and the device
// -> host copy of H psi on every application.  addft_hpsi_host streams the bands
// through the GPU in chunks: chunk c is copied in on an upload stream, transformed on
// the caller's stream by addft_hpsi (whose projector chain forks onto its own
// stream), and copied out on a download stream, so the upload of chunk c + 1, the H
// psi of chunk c and the download of chunk c - 1 run at the same time (the first chunk
// is half a chunk, so the pipeline fills and drains sooner).  Two device
// slots for inputs and two for outputs alternate between chunks; events order slot
// reuse.  The caller's stream is joined with the last download, so synchronising it
// means the host result is complete.
//
// Bands are independent in H psi, so chunking changes only the order of the becp
// split sums (results agree with one addft_hpsi call to FP32 / FP64 rounding).
#include <vector>

#include "common.cuh"

namespace addft {
namespace {

inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

// The calling thread's upload (0) and download (1) streams on the current device.
addft_status copy_stream(int which, cudaStream_t *out) {
  constexpr int kDev = 64;
  static thread_local cudaStream_t s[2][kDev] = {};
  int dev = 0;
  ADDFT_CUDA(cudaGetDevice(&dev));
  ADDFT_REQUIRE(dev >= 0 && dev < kDev, ADDFT_UNSUPPORTED, "hpsi_host: device index %d >= %d", dev, kDev);
  if (s[which][dev] == nullptr) ADDFT_CUDA(cudaStreamCreateWithFlags(&s[which][dev], cudaStreamNonBlocking));
  *out = s[which][dev];
  return ADDFT_OK;
}

struct Chunk {
  int k, b0, nb;
};

}  // namespace
}  // namespace addft

using namespace addft;

extern "C" {

size_t addft_hpsi_host_work_bytes(addft_plan plan, addft_dtype dt, int nk, int nb, int nproj, int chunk_bands) {
  if (!plan || nk < 1 || nb < 1) return 0;
  int nG = 0, np = 0, nc = 0;
  if (addft_plan_info(plan, &np, &nc, &nG) != ADDFT_OK) return 0;
  const int cb = chunk_bands < 1 || chunk_bands > nb ? nb : chunk_bands;
  const size_t csz = dt == ADDFT_F64 ? 16 : 8;
  const size_t slot = al256((size_t)cb * nG * csz);
  return 4 * slot + addft_hpsi_work_bytes(plan, dt, 1, cb, nproj, cb);
}

addft_status addft_hpsi_host(addft_plan plan, addft_dtype dt, int nk, int nb, const void *psi_host, const void *kin,
                             const void *v_r, int nproj, const void *proj, const void *dion, void *hpsi_host,
                             int chunk_bands, void *work, size_t work_bytes, void *stream) {
  ADDFT_REQUIRE(plan && nk >= 1 && nb >= 0 && nproj >= 0, ADDFT_INVALID_ARG, "hpsi_host: bad arguments");
  if (nb == 0) return ADDFT_OK;   // no bands: the data pointers may be NULL
  ADDFT_REQUIRE(psi_host && hpsi_host && kin && v_r, ADDFT_INVALID_ARG, "hpsi_host: null pointer");
  ADDFT_REQUIRE(nproj == 0 || (proj && dion), ADDFT_INVALID_ARG, "hpsi_host: null projector tables");
  ADDFT_REQUIRE(psi_host != hpsi_host, ADDFT_INVALID_ARG, "hpsi_host: output aliases input");
  int nG = 0, np = 0, nc = 0;
  ADDFT_TRY(addft_plan_info(plan, &np, &nc, &nG));
  const int cb = chunk_bands < 1 || chunk_bands > nb ? nb : chunk_bands;
  const size_t csz = dt == ADDFT_F64 ? 16 : 8;
  const size_t rsz = csz / 2;
  const size_t slot = al256((size_t)cb * nG * csz);
  const size_t need = addft_hpsi_host_work_bytes(plan, dt, nk, nb, nproj, cb);
  ADDFT_REQUIRE(work && work_bytes >= need, ADDFT_INVALID_ARG, "hpsi_host: work needs %zu B, got %zu B", need,
                work_bytes);
  char *w = (char *)work;
  char *in[2] = {w, w + slot}, *out[2] = {w + 2 * slot, w + 3 * slot};
  char *hw = w + 4 * slot;
  const size_t hw_bytes = work_bytes - 4 * slot;

  cudaStream_t st = as_stream(stream), up = nullptr, down = nullptr;
  ADDFT_TRY(copy_stream(0, &up));
  ADDFT_TRY(copy_stream(1, &down));
  // the first chunk of the call is half a chunk, so the first H psi starts after half the
  // upload and the last download (the remainder) is short: the pipeline fills and drains sooner
  std::vector<Chunk> chunks;
  for (int k = 0; k < nk; ++k)
    for (int b0 = 0; b0 < nb;) {
      const int first = k == 0 && b0 == 0 && cb < nb ? (cb + 1) / 2 : cb;
      const int n1 = std::min(first, nb - b0);
      chunks.push_back({k, b0, n1});
      b0 += n1;
    }
  const int n = (int)chunks.size();
  // per chunk: upload done, compute done, download done; plus the caller's stream at entry
  std::vector<cudaEvent_t> ev(3 * (size_t)n + 1, nullptr);
  struct Release {
    std::vector<cudaEvent_t> &e;
    ~Release() {
      for (cudaEvent_t x : e)
        if (x) cudaEventDestroy(x);
    }
  } release{ev};
  for (auto &e : ev) ADDFT_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  cudaEvent_t *ev_up = ev.data(), *ev_comp = ev.data() + n, *ev_down = ev.data() + 2 * n, ev_entry = ev[3 * n];
  // the copies may not start before the work the caller queued ahead of this call
  ADDFT_CUDA(cudaEventRecord(ev_entry, st));
  ADDFT_CUDA(cudaStreamWaitEvent(up, ev_entry, 0));
  ADDFT_CUDA(cudaStreamWaitEvent(down, ev_entry, 0));
  addft_status status = ADDFT_OK;
  int issued = 0;
  for (int c = 0; c < n && status == ADDFT_OK; ++c) {
    const Chunk &ch = chunks[c];
    const int s = c & 1;
    const size_t off = ((size_t)ch.k * nb + ch.b0) * nG * csz;
    const size_t bytes = (size_t)ch.nb * nG * csz;
    // upload: the slot's previous chunk (c - 2) must have been consumed by its H psi
    if (c >= 2) ADDFT_CUDA(cudaStreamWaitEvent(up, ev_comp[c - 2], 0));
    ADDFT_CUDA(cudaMemcpyAsync(in[s], (const char *)psi_host + off, bytes, cudaMemcpyHostToDevice, up));
    ADDFT_CUDA(cudaEventRecord(ev_up[c], up));
    // H psi on the caller's stream: input uploaded, output slot downloaded (chunk c - 2)
    ADDFT_CUDA(cudaStreamWaitEvent(st, ev_up[c], 0));
    if (c >= 2) ADDFT_CUDA(cudaStreamWaitEvent(st, ev_down[c - 2], 0));
    status = addft_hpsi(plan, dt, 1, ch.nb, in[s], (const char *)kin + (size_t)ch.k * nG * rsz, v_r, nproj,
                        nproj ? (const char *)proj + (size_t)ch.k * nproj * nG * csz : nullptr, dion, out[s], hw,
                        hw_bytes, st);
    ADDFT_CUDA(cudaEventRecord(ev_comp[c], st));
    // download
    ADDFT_CUDA(cudaStreamWaitEvent(down, ev_comp[c], 0));
    ADDFT_CUDA(cudaMemcpyAsync((char *)hpsi_host + off, out[s], bytes, cudaMemcpyDeviceToHost, down));
    ADDFT_CUDA(cudaEventRecord(ev_down[c], down));
    issued = c + 1;
  }
  // join: the caller's stream completes after every download issued
  if (issued > 0) ADDFT_CUDA(cudaStreamWaitEvent(st, ev_down[issued - 1], 0));
  return status;
}

}  // extern "C"
