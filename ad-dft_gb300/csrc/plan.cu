// Plans (sphere-aware FFT layout), library status plumbing and shared helpers.
#include <stdarg.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "transforms.cuh"

namespace addft {

static thread_local char g_last_error[512] = "";
static unsigned long long g_launches = 0;   // kernels launched through this library

void set_error(const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

addft_status check_launch(const char *what) {
  __atomic_add_fetch(&g_launches, 1ull, __ATOMIC_RELAXED);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("launch of %s failed: %s", what, cudaGetErrorString(e));
    return ADDFT_CUDA_ERROR;
  }
  return ADDFT_OK;
}

__global__ void k_finalize_sums(const double *partial, int nv, int nblk, double *out, int acc) {
  __shared__ double red[32];
  for (int j = 0; j < nv; ++j) {
    double x = 0.0;
    for (int i = threadIdx.x; i < nblk; i += blockDim.x) x += partial[(size_t)j * nblk + i];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
      const int nw = (blockDim.x + 31) >> 5;
      double y = threadIdx.x < nw ? red[threadIdx.x] : 0.0;
      for (int o = 16; o > 0; o >>= 1) y += __shfl_down_sync(0xffffffffu, y, o);
      if (threadIdx.x == 0) out[j] = acc ? out[j] + y : y;
    }
    __syncthreads();
  }
}

addft_status finalize_sums(const double *partial, int nv, int nblk, double *out, bool acc,
                           cudaStream_t st) {
  k_finalize_sums<<<1, 256, 0, st>>>(partial, nv, nblk, out, acc ? 1 : 0);
  return check_launch("finalize_sums");
}

// Factor n into the fewest radices from {16, 15, 12, 10, 9, 8, 6, 5, 4, 3, 2}
// (each a register-resident DFT), preferring balanced factors (72 = 8 x 9).
static void best_factor(int n, int depth, std::vector<int> &cur, std::vector<int> &best, int &best_min) {
  static const int rad[] = {16, 15, 12, 10, 9, 8, 6, 5, 4, 3, 2};
  if (n == 1) {
    int mn = 1 << 30;
    for (int r : cur) mn = std::min(mn, r);
    if (best.empty() || cur.size() < best.size() || (cur.size() == best.size() && mn > best_min)) {
      best = cur;
      best_min = mn;
    }
    return;
  }
  if (depth >= kMaxStages) return;
  if (!best.empty() && cur.size() + 1 > best.size()) return;
  for (int r : rad) {
    if (n % r) continue;
    cur.push_back(r);
    best_factor(n / r, depth + 1, cur, best, best_min);
    cur.pop_back();
  }
}

static bool factorize(int n, AxisPlan &ap) {
  ap.n = n;
  ap.nst = 0;
  std::vector<int> cur, best;
  int best_min = 0;
  best_factor(n, 0, cur, best, best_min);
  if (best.empty() && n != 1) return false;
  // larger radix first
  std::sort(best.begin(), best.end(), [](int a, int b) { return a > b; });
  for (int r : best) ap.rad[ap.nst++] = r;
  if (n == 1) { ap.rad[0] = 1; ap.nst = 0; }
  return true;
}

}  // namespace addft

using namespace addft;

extern "C" {

const char *addft_status_string(addft_status s) {
  switch (s) {
    case ADDFT_OK: return "ok";
    case ADDFT_INVALID_ARG: return "invalid argument";
    case ADDFT_CUDA_ERROR: return "cuda error";
    case ADDFT_NOT_CONVERGED: return "not converged";
    case ADDFT_TIMEOUT: return "timeout";
    case ADDFT_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

const char *addft_last_error(void) { return g_last_error; }

int addft_version(void) { return 1; }

unsigned long long addft_launch_count(void) { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

addft_status addft_plan_create(addft_plan *plan, int n1, int n2, int n3, int nG,
                               const int32_t *miller) {
  ADDFT_REQUIRE(plan != nullptr && miller != nullptr, ADDFT_INVALID_ARG, "null plan or miller");
  ADDFT_REQUIRE(n1 > 0 && n2 > 0 && n3 > 0 && nG > 0, ADDFT_INVALID_ARG,
                "bad box %d x %d x %d or nG %d", n1, n2, n3, nG);
  *plan = nullptr;
  AxisPlan ax[3];
  const int ns[3] = {n1, n2, n3};
  for (int a = 0; a < 3; ++a)
    ADDFT_REQUIRE(factorize(ns[a], ax[a]), ADDFT_UNSUPPORTED,
                  "box dimension %d is not 2,3,5-smooth", ns[a]);
  const long N = (long)n1 * n2 * n3;
  // wrap and check uniqueness
  std::vector<int> i1(nG), i2(nG), i3(nG);
  std::vector<char> seen(N, 0);
  for (int g = 0; g < nG; ++g) {
    auto wrap = [](int m, int n) { int r = m % n; return r < 0 ? r + n : r; };
    i1[g] = wrap(miller[3 * g + 0], n1);
    i2[g] = wrap(miller[3 * g + 1], n2);
    i3[g] = wrap(miller[3 * g + 2], n3);
    const long f = ((long)i1[g] * n2 + i2[g]) * n3 + i3[g];
    ADDFT_REQUIRE(!seen[f], ADDFT_INVALID_ARG,
                  "G index %d aliases another G in the %dx%dx%d box", g, n1, n2, n3);
    seen[f] = 1;
  }
  // sort sphere points by (i1, i2, i3)
  std::vector<int> order(nG);
  for (int g = 0; g < nG; ++g) order[g] = g;
  std::sort(order.begin(), order.end(), [&](int a, int b) {
    if (i1[a] != i1[b]) return i1[a] < i1[b];
    if (i2[a] != i2[b]) return i2[a] < i2[b];
    return i3[a] < i3[b];
  });
  std::vector<int> sp_g(nG), sp_pos(nG), gptr, plane_i1, rptr, row_i2;
  std::vector<int> plane_of_i1(n1, -1);
  for (int k = 0; k < nG; ++k) {
    const int g = order[k];
    sp_g[k] = g;
    sp_pos[k] = i2[g] * (n3 | 1) + i3[g];   // shared-memory tile position (odd row pitch)
    if (k == 0 || i1[g] != i1[order[k - 1]]) {
      plane_of_i1[i1[g]] = (int)plane_i1.size();
      plane_i1.push_back(i1[g]);
      gptr.push_back(k);
      rptr.push_back((int)row_i2.size());
    }
    if (k == 0 || i1[g] != i1[order[k - 1]] || i2[g] != i2[order[k - 1]]) row_i2.push_back(i2[g]);
  }
  gptr.push_back(nG);
  rptr.push_back((int)row_i2.size());
  const int np = (int)plane_i1.size();
  const int nrows = (int)row_i2.size();
  // per active x-plane: its columns as a low run i2 = 0 .. nlo-1 and a high run n2-nhi .. n2-1
  std::vector<int> row_lohi(np, 0);
  bool xy_direct = n2 < (1 << 15);
  for (int p = 0; p < np && xy_direct; ++p) {
    int nlo = 0, nhi = 0;
    for (int r = rptr[p]; r < rptr[p + 1]; ++r) (row_i2[r] <= n2 / 2 ? nlo : nhi)++;
    for (int r = rptr[p]; r < rptr[p + 1]; ++r) {
      const int t = r - rptr[p];
      const int want = t < nlo ? t : n2 - nhi + (t - nlo);
      if (row_i2[r] != want) xy_direct = false;
    }
    row_lohi[p] = nlo | (nhi << 16);
  }
  // column pipeline tables: column c = c-th (i1, i2) row in sorted order
  const int ncols_pad = (nrows + kColGroup - 1) / kColGroup * kColGroup;
  std::vector<int> cgptr(ncols_pad / kColGroup + 1, nG), pt_pos(nG), col_xy(nrows);
  {
    int c = -1;
    for (int k = 0; k < nG; ++k) {
      const int g = order[k];
      if (k == 0 || i1[g] != i1[order[k - 1]] || i2[g] != i2[order[k - 1]]) {
        ++c;
        col_xy[c] = i1[g] * (n2 | 1) + i2[g];
        if (c % kColGroup == 0) cgptr[c / kColGroup] = k;
      }
      pt_pos[k] = i3[g] * kColPitch + c % kColGroup;
    }
  }

  // twiddles e^{-2 pi i t / n}
  const int ntw = n1 + n2 + n3;
  std::vector<double> twd(2 * ntw);
  std::vector<float> twf(2 * ntw);
  {
    int off = 0;
    for (int a = 0; a < 3; ++a) {
      for (int t = 0; t < ns[a]; ++t) {
        const double ang = -2.0 * M_PI * (double)t / (double)ns[a];
        twd[2 * (off + t)] = std::cos(ang);
        twd[2 * (off + t) + 1] = std::sin(ang);
        twf[2 * (off + t)] = (float)std::cos(ang);
        twf[2 * (off + t) + 1] = (float)std::sin(ang);
      }
      off += ns[a];
    }
  }

  // one device blob: [twd | twf | ints...], each section 256-byte aligned
  auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
  size_t off_twd = 0;
  size_t off_twf = align(off_twd + sizeof(double) * 2 * ntw);
  size_t off_int = align(off_twf + sizeof(float) * 2 * ntw);
  std::vector<int> ints;
  auto push = [&](const std::vector<int> &v) {
    size_t at = ints.size();
    ints.insert(ints.end(), v.begin(), v.end());
    while (ints.size() % 64) ints.push_back(0);
    return at;
  };
  std::vector<int> mil(miller, miller + 3 * (size_t)nG);
  const size_t o_spg = push(sp_g), o_spp = push(sp_pos), o_gptr = push(gptr),
               o_pi1 = push(plane_i1), o_rptr = push(rptr), o_row = push(row_i2),
               o_poi = push(plane_of_i1), o_mil = push(mil), o_cgp = push(cgptr), o_ptp = push(pt_pos),
               o_cxy = push(col_xy), o_rlh = push(row_lohi);
  const size_t total = off_int + sizeof(int) * ints.size();

  auto *p = new addft_plan_s();
  if (cudaGetDevice(&p->device) != cudaSuccess) { delete p; set_error("cudaGetDevice failed"); return ADDFT_CUDA_ERROR; }
  cudaError_t e = cudaMalloc(&p->blob, total);
  if (e != cudaSuccess) {
    delete p;
    set_error("plan allocation of %zu B failed: %s", total, cudaGetErrorString(e));
    return ADDFT_CUDA_ERROR;
  }
  std::vector<char> host(total, 0);
  memcpy(host.data() + off_twd, twd.data(), sizeof(double) * twd.size());
  memcpy(host.data() + off_twf, twf.data(), sizeof(float) * twf.size());
  memcpy(host.data() + off_int, ints.data(), sizeof(int) * ints.size());
  e = cudaMemcpy(p->blob, host.data(), total, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(p->blob);
    delete p;
    set_error("plan upload failed: %s", cudaGetErrorString(e));
    return ADDFT_CUDA_ERROR;
  }
  char *b = (char *)p->blob;
  const int *ib = (const int *)(b + off_int);
  PlanDev &d = p->dev;
  d.n1 = n1; d.n2 = n2; d.n3 = n3; d.nG = nG; d.np = np; d.nrows = nrows;
  d.sp_g = ib + o_spg; d.sp_pos = ib + o_spp; d.gptr = ib + o_gptr; d.plane_i1 = ib + o_pi1;
  d.rptr = ib + o_rptr; d.row_i2 = ib + o_row; d.plane_of_i1 = ib + o_poi; d.miller = ib + o_mil;
  d.ncols_pad = ncols_pad; d.cgptr = ib + o_cgp; d.pt_pos = ib + o_ptp; d.col_xy = ib + o_cxy;
  d.xy_direct = xy_direct ? 1 : 0; d.row_lohi = ib + o_rlh;
  d.tw_d = b + off_twd;
  d.tw_f = b + off_twf;
  for (int a = 0; a < 3; ++a) d.ax[a] = ax[a];
  d.tun = fft_tuning();
  p->ncols = nrows;
  *plan = p;
  return ADDFT_OK;
}

addft_status addft_plan_destroy(addft_plan plan) {
  if (!plan) return ADDFT_OK;
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != plan->device) cudaSetDevice(plan->device);
  cudaError_t e = cudaFree(plan->blob);
  if (cur != plan->device) cudaSetDevice(cur);
  delete plan;
  if (e != cudaSuccess) {
    set_error("plan free failed: %s", cudaGetErrorString(e));
    return ADDFT_CUDA_ERROR;
  }
  return ADDFT_OK;
}

addft_status addft_plan_info(addft_plan plan, int *nplanes, int *ncols, int *nG) {
  ADDFT_REQUIRE(plan != nullptr, ADDFT_INVALID_ARG, "null plan");
  if (nplanes) *nplanes = plan->dev.np;
  if (ncols) *ncols = plan->ncols;
  if (nG) *nG = plan->dev.nG;
  return ADDFT_OK;
}

addft_status addft_plan_set_tuning(addft_plan plan, const char *key, long value) {
  ADDFT_REQUIRE(plan != nullptr && key != nullptr, ADDFT_INVALID_ARG, "plan_set_tuning: null argument");
  FftTuning &t = plan->dev.tun;
  const bool threads = value >= 64 && value <= kFftMaxThreads && value % 32 == 0;
  if (!strcmp(key, "threads_plane")) {
    ADDFT_REQUIRE(threads, ADDFT_INVALID_ARG, "threads_plane must be a multiple of 32 in [64, %d]", kFftMaxThreads);
    t.threads_plane = (int)value;
  } else if (!strcmp(key, "threads_x")) {
    ADDFT_REQUIRE(threads, ADDFT_INVALID_ARG, "threads_x must be a multiple of 32 in [64, %d]", kFftMaxThreads);
    t.threads_x = (int)value;
  } else if (!strcmp(key, "xtile_kb")) {
    ADDFT_REQUIRE(value >= 8 && value <= 200, ADDFT_INVALID_ARG, "xtile_kb must be in [8, 200]");
    t.xtile_kb = (int)value;
  } else if (!strcmp(key, "slab_mb")) {
    ADDFT_REQUIRE(value >= 1 && value <= (1L << 20), ADDFT_INVALID_ARG, "slab_mb must be in [1, 2^20]");
    t.slab_chunk_bytes = (size_t)value << 20;
  } else if (!strcmp(key, "threads_plane2")) {
    ADDFT_REQUIRE(threads, ADDFT_INVALID_ARG, "threads_plane2 must be a multiple of 32 in [64, %d]", kFftMaxThreads);
    t.threads_plane2 = (int)value;
  } else if (!strcmp(key, "xline2")) {
    ADDFT_REQUIRE(value == 0 || value == 1, ADDFT_INVALID_ARG, "xline2 must be 0 or 1");
    t.xline2 = (int)value;
  } else if (!strcmp(key, "plane2")) {
    ADDFT_REQUIRE(value == 0 || value == 1, ADDFT_INVALID_ARG, "plane2 must be 0 or 1");
    t.plane2 = (int)value;
  } else if (!strcmp(key, "colfft")) {
    ADDFT_REQUIRE(value >= 0 && value <= 2, ADDFT_INVALID_ARG, "colfft must be 0, 1 or 2");
    t.colfft = (int)value;
  } else if (!strcmp(key, "xy_direct")) {
    ADDFT_REQUIRE(value == 0 || value == 1, ADDFT_INVALID_ARG, "xy_direct must be 0 or 1");
    t.xy_direct = (int)value;
  } else if (!strcmp(key, "plane_split")) {
    ADDFT_REQUIRE(value == 0 || value == 1, ADDFT_INVALID_ARG, "plane_split must be 0 or 1");
    t.plane_split = (int)value;
  } else if (!strcmp(key, "threads_xy")) {
    ADDFT_REQUIRE(value == 0 || (value >= 64 && value <= kXYMaxThreads && value % 32 == 0), ADDFT_INVALID_ARG,
                  "threads_xy must be 0 or a multiple of 32 in [64, %d]", kXYMaxThreads);
    t.threads_xy = (int)value;
  } else {
    ADDFT_REQUIRE(false, ADDFT_INVALID_ARG, "unknown tuning key '%s'", key);
  }
  return ADDFT_OK;
}

addft_status addft_plan_get_tuning(addft_plan plan, const char *key, long *value) {
  ADDFT_REQUIRE(plan != nullptr && key != nullptr && value != nullptr, ADDFT_INVALID_ARG,
                "plan_get_tuning: null argument");
  const FftTuning &t = plan->dev.tun;
  if (!strcmp(key, "threads_plane")) *value = t.threads_plane;
  else if (!strcmp(key, "threads_x")) *value = t.threads_x;
  else if (!strcmp(key, "xtile_kb")) *value = t.xtile_kb;
  else if (!strcmp(key, "slab_mb")) *value = (long)(t.slab_chunk_bytes >> 20);
  else if (!strcmp(key, "xline2")) *value = t.xline2;
  else if (!strcmp(key, "plane2")) *value = t.plane2;
  else if (!strcmp(key, "threads_plane2")) *value = t.threads_plane2;
  else if (!strcmp(key, "colfft")) *value = t.colfft;
  else if (!strcmp(key, "threads_xy")) *value = t.threads_xy;
  else if (!strcmp(key, "xy_direct")) *value = t.xy_direct;
  else if (!strcmp(key, "plane_split")) *value = t.plane_split;
  else ADDFT_REQUIRE(false, ADDFT_INVALID_ARG, "unknown tuning key '%s'", key);
  return ADDFT_OK;
}

size_t addft_work_bytes(addft_plan plan, int nbatch, addft_dtype dt) {
  if (!plan || nbatch < 1) return 0;
  const size_t csz = dt == ADDFT_F64 ? 16 : 8;
  const PlanDev &d = plan->dev;
  // reduction partials (1 MB) + the potential in xy-plane order (column pipeline, N reals)
  // + nbatch bands of the larger of the slab (np x n2 x n3) and the column pipeline's per-band
  // buffers (n3 x ncols_pad columns + nG kinetic terms)
  const size_t slab = (size_t)d.np * d.n2 * d.n3 * csz;
  // (the kinetic diagonals of up to one k point per band in flight, nG reals each, included)
  const size_t colb = (((size_t)d.n3 * d.ncols_pad * csz + 255) & ~size_t(255)) +
                      (((size_t)d.nG * csz + 255) & ~size_t(255)) + (((size_t)d.nG * (csz / 2) + 255) & ~size_t(255));
  const size_t vt = ((size_t)d.n1 * d.n2 * d.n3 * (csz / 2) + 255) & ~size_t(255);
  return (size_t)nbatch * (slab > colb ? slab : colb) + (size_t(1) << 20) + vt;
}

}  // extern "C"
