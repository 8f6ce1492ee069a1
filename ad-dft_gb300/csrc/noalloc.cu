// H psi without any device allocation, for callers that cannot allocate.
//
// Some callers of this library may not call cudaMalloc (or any allocating
// routine) at the point where they need H psi: an XLA FFI custom call inside a
// JAX program runs while XLA owns a pre-reserved pool of most of the device
// memory, so an allocation from inside the handler can fail and would hold
// memory the framework does not track; a host application under a fixed
// device-memory budget is in the same position.  addft_hpsi_noalloc gives
// them the matrix-free H psi with its scratch taken from a statically sized
// __device__ array in this file instead of a caller-supplied work buffer.
//
// Properties a caller must know:
//   * The array is kNoAllocScratchBytes (8 MiB) per device.  Every GPU that
//     loads this library holds it until the process exits.
//   * Host code cannot use the array's name as a device address; the first
//     call on each device resolves the address with cudaGetSymbolAddress
//     (with that device current) and caches it.  Make that first call
//     outside any CUDA stream capture.
//   * All calls share the one array and it keeps the previous call's data.
//     Nothing in it has to start at zero: every byte H psi reads from the
//     scratch is written earlier in the same call.  Two calls that overlap on
//     the GPU (different streams, or host threads without ordering) race on
//     the array; serialise them.
//   * Problems whose minimum scratch (one band of FFT scratch for the box plus
//     the becp and D becp arrays) exceeds the array are rejected with
//     ADDFT_UNSUPPORTED and a message; use addft_hpsi with a caller buffer.
//     Room beyond the minimum goes to split-K partials of becp, as many
//     splits as fit.
//   * The cached address belongs to the device's primary context.  After a
//     cudaDeviceReset every plan and this address are stale; the library
//     does not support a reset while it is in use.
//   * The call allocates and frees nothing and creates no CUDA objects: it runs
//     the addft_hpsi kernels on the static scratch and on the caller's stream
//     only (addft_hpsi itself may fork its projector chain onto a second
//     stream), processing as many bands per chunk as fit.
#include <atomic>

#include "common.cuh"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::atomic<void *> g_scratch_addr[kMaxDevices];

addft_status scratch_address(void **out) {
  int dev = 0;
  ADDFT_CUDA(cudaGetDevice(&dev));
  ADDFT_REQUIRE(dev >= 0 && dev < kMaxDevices, ADDFT_UNSUPPORTED, "hpsi_noalloc: device index %d >= %d", dev,
                kMaxDevices);
  void *p = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (p == nullptr) {
    // Resolve the device address of the static array on the current device.
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      ::addft::set_error("hpsi_noalloc: cudaGetSymbolAddress of the static scratch failed on device %d: %s", dev,
                         cudaGetErrorString(e));
      return ADDFT_CUDA_ERROR;
    }
    g_scratch_addr[dev].store(p, std::memory_order_release);
  }
  *out = p;
  return ADDFT_OK;
}

}  // namespace

namespace addft {
addft_status hpsi_one_stream(addft_plan plan, addft_dtype dt, int nk, int nb, const void *psi, const void *kin,
                             const void *v_r, int nproj, const void *proj, const void *dion, void *hpsi, void *work,
                             size_t work_bytes, void *stream);   // nonlocal.cu
}  // namespace addft

extern "C" {

size_t addft_hpsi_noalloc_max_scratch_bytes(void) { return kNoAllocScratchBytes; }

addft_status addft_hpsi_noalloc(addft_plan plan, addft_dtype dt, int nk, int nb, const void *psi, const void *kin,
                                const void *v_r, int nproj, const void *proj, const void *dion, void *hpsi,
                                void *stream) {
  ADDFT_REQUIRE(plan != nullptr && nk >= 1 && nb >= 0 && nproj >= 0, ADDFT_INVALID_ARG,
                "hpsi_noalloc: bad arguments");
  // the least addft_hpsi runs with: becp and D becp, one band of FFT scratch (no split-K
  // partials: with less room becp uses fewer splits, down to one)
  const size_t csz = dt == ADDFT_F64 ? 16 : 8;
  const size_t arrays = nproj > 0 ? ((2 * (size_t)nk * nproj * nb * csz + 255) & ~size_t(255)) : 0;
  const size_t need = arrays + addft_work_bytes(plan, 1, dt);
  ADDFT_REQUIRE(need <= kNoAllocScratchBytes, ADDFT_UNSUPPORTED,
                "hpsi_noalloc: this problem needs at least %zu B of scratch but the static scratch holds %zu B "
                "(use addft_hpsi with a caller work buffer)",
                need, kNoAllocScratchBytes);
  void *scratch = nullptr;
  ADDFT_TRY(scratch_address(&scratch));
  return ::addft::hpsi_one_stream(plan, dt, nk, nb, psi, kin, v_r, nproj, proj, dion, hpsi, scratch,
                                   kNoAllocScratchBytes, stream);
}

}  // extern "C"
