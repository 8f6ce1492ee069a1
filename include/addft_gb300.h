/*
 * addft_gb300.h -- C ABI of the GB300 (sm_103a) plane-wave hot path.
 *
 * This library replaces the native seam of ad-dft: the XLA FFI handlers
 * (XcLdaHandler, ScatterC128/GatherC128 and their C64 twins, EighLowestHandler;
 * native/xc_lda.cu:70-75, native/pack.cu:88-100,177-189, native/eigh.cu:155-160)
 * and the JAX code that those handlers sit under (src/addft/ops/hpsi.py,
 * physics/{density,hartree,xc,local,nonlocal_op,ewald}.py, the envelope
 * backward of api.py:106-113).
 *
 * Conventions (all identical to the reference):
 *   - psi is (nk, nb, nG) complex, row-major, G in the frozen Miller order of
 *     src/addft/geometry/basis.py:89-121;
 *   - real-space fields are (N,) with flat index (i1*n2 + i2)*n3 + i3
 *     (basis.py:196-202), N = n1*n2*n3;
 *   - psi(r) = ifftn * N/sqrt(Omega), c_G = fftn * sqrt(Omega)/N
 *     (basis.py:237-254); n(G) = fftn(rho)/N on the wavefunction shell
 *     (basis.py:257-262);
 *   - complex numbers are interleaved (re, im): float2 for ADDFT_F32,
 *     double2 for ADDFT_F64.
 *
 * Ownership: every data pointer is a DEVICE pointer owned by the caller
 * (inputs, outputs and the scratch "work" buffer), except where a comment says
 * "host".  Calls are asynchronous on the given CUDA stream (a cudaStream_t
 * passed as void*, NULL = legacy default stream).  Device-side results that
 * are scalars (energies, gradients) are written to device memory.
 * Only addft_plan_create / addft_plan_destroy allocate or free device memory
 * (and, once per host thread and device, cuSOLVER's handle in
 * addft_ffi_eigh_lowest).  addft_hpsi may run its projector contractions on a
 * second stream of the calling thread (created on first use), forked from and
 * joined back into the caller's stream with events; ADDFT_HPSI_OVERLAP=0 keeps
 * everything on the caller's stream.
 *
 * Errors: every entry point returns an addft_status.  A non-OK status leaves
 * a one-line message readable through addft_last_error() (thread-local).
 *
 * Empty inputs: a call whose band, batch or point count is zero does no work and
 * returns ADDFT_OK (a reduction into a scalar writes 0); the data pointers that
 * count sizes may then be NULL, as an empty array's are.  The plan and the
 * other sizes are still checked.
 */
#ifndef ADDFT_GB300_H
#define ADDFT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int addft_status;
#define ADDFT_OK 0
#define ADDFT_INVALID_ARG 1   /* shape / size / pointer mismatch (ffi::Error::InvalidArgument) */
#define ADDFT_CUDA_ERROR 2    /* a CUDA runtime call or launch failed (ffi::Error::Internal)   */
#define ADDFT_NOT_CONVERGED 3
#define ADDFT_TIMEOUT 4
#define ADDFT_UNSUPPORTED 5   /* valid input outside what the library supports (box too large) */

typedef enum { ADDFT_F32 = 0, ADDFT_F64 = 1 } addft_dtype;

typedef struct addft_plan_s *addft_plan;

/* Norm-conserving KB pseudopotential of one species (geometry/psp.py:19-138).
 * kind 0 (analytic, the reference's synthetic()):
 *   beta_i(q) = w_i q^l_i exp(-(q b_i)^2/2), v~_loc(q) = -vloc_amp exp(-(q vloc_sigma)^2/2)
 *   (psp.py:92-95,122-128,141-164);
 * kind 1 (from a UPF file, psp.py:102-119,130-138): radial functions tabulated on
 *   the uniform grid q_i = i dq, i < nq, in the device array tab (f64,
 *   layout [f][2][nq]: value, d/dq): f = 0..nrad-1 are beta_i(q) =
 *   4 pi int r beta_i(r) r j_l(q r) dr, f = nrad is the smooth part of the local
 *   potential 4 pi int (r v(r) + zval erf(r)) sin(q r)/q dr; the kernels add
 *   -4 pi zval exp(-q^2/4)/q^2 and use vloc_g0 at q = 0.  Values between nodes
 *   are cubic Hermite interpolants.
 * Y_lm order as ylm.py:8-26 (m = 0, +1, -1, +2, -2); l <= 2. */
typedef struct {
  int nrad;          /* radial projectors, <= 4 */
  int l[4];          /* angular momentum of each radial projector, <= 2 */
  double w[4];       /* kind 0 */
  double b[4];       /* kind 0 */
  double vloc_amp;   /* kind 0 */
  double vloc_sigma; /* kind 0 */
  int kind;          /* 0 analytic, 1 tabulated */
  int nq;            /* kind 1: table points */
  double dq;         /* kind 1: grid step (1/Bohr) */
  const double *tab; /* kind 1: device table, (nrad + 1) x 2 x nq */
  double vloc_g0;    /* kind 1: v~_loc(0) (Ha Bohr^3) */
  double zval;       /* kind 1: valence charge of the Coulomb tail */
} addft_psp;

/* ---- library --------------------------------------------------------- */
const char *addft_status_string(addft_status s);
const char *addft_last_error(void);
int addft_version(void);
/* Number of kernels this library has launched in the process (diagnostic). */
unsigned long long addft_launch_count(void);

/* ---- plans ------------------------------------------------------------
 * A plan binds an FFT box (n1, n2, n3; each a 2,3,5-smooth integer) to a
 * frozen G-sphere given as host Miller indices (nG x 3, int32, any integers;
 * they are wrapped mod n).  It builds the sphere-aware FFT layout and uploads
 * it to the current device.  Replaces the index arithmetic of
 * basis.py:196-230 and the packing of native/pack.cu:16-38.
 * Returns ADDFT_INVALID_ARG if two G map to the same box point. */
addft_status addft_plan_create(addft_plan *plan, int n1, int n2, int n3, int nG,
                               const int32_t *miller_host);
addft_status addft_plan_destroy(addft_plan plan);
/* Query: number of active x-planes, of active (x,y) columns, and nG. */
addft_status addft_plan_info(addft_plan plan, int *nplanes, int *ncols, int *nG);
/* Launch tunables of one plan (every transform, H psi and density call on it);
 * no counterpart in the reference (XLA picks cuFFT plans itself).  Keys:
 *   "threads_plane", "threads_x"  threads per CTA of the generic plane / x-line
 *                                 kernels (multiple of 32 in [64, 512]);
 *   "xtile_kb"                    shared memory of a generic x-line tile [8, 200];
 *   "slab_mb"                     slab bytes per band chunk (bands in flight);
 *   "xline2", "plane2"            1: two-pass register kernels where instantiated;
 *   "threads_plane2"              threads per CTA of the two-pass plane kernels;
 *   "colfft"                      1: H psi through the column pipeline (z-column FFTs,
 *                                 fused xy-plane FFT with V(r)) where instantiated;
 *                                 2: the same pipeline as one persistent kernel whose
 *                                 CTAs take work items (z-column groups, xy-planes)
 *                                 band by band (FP32, cubic boxes; else as 1);
 *   "threads_xy"                  threads per CTA of its xy-plane kernel (0: 256);
 *   "xy_direct"                   1: that kernel loads / stores the columns directly
 *                                 where every x-plane's columns are two wrapped runs;
 *   "plane_split"                 1: the z and y stages of the generic pipeline as
 *                                 z-column-group and y-tile kernels on every box; 0: only
 *                                 where a yz-plane's two tiles exceed a CTA's shared
 *                                 memory (n2 (n3 | 1) above ~7,200 in FP64, ~14,400 in
 *                                 FP32).  The split stages need n3 <= 216 (FP64) or
 *                                 432 (FP32); beyond that a call returns
 *                                 ADDFT_UNSUPPORTED.
 * A plan starts from the process defaults (ADDFT_FFT_THREADS, ADDFT_FFT_THREADS_X,
 * ADDFT_XTILE_KB, ADDFT_SLAB_MB, ADDFT_XLINE2, ADDFT_PLANE2, ADDFT_PLANE2_THREADS,
 * ADDFT_COLFFT, ADDFT_XY_THREADS, ADDFT_XY_DIRECT, ADDFT_PLANE_SPLIT).  Not thread-safe against concurrent
 * calls on the same plan. */
addft_status addft_plan_set_tuning(addft_plan plan, const char *key, long value);
addft_status addft_plan_get_tuning(addft_plan plan, const char *key, long *value);

/* Scratch bytes that lets one call process `nbatch` bands at once.  Every
 * transform entry point accepts any work size >= addft_work_bytes(plan, 1,
 * dtype) and loops over band chunks that fit. */
size_t addft_work_bytes(addft_plan plan, int nbatch, addft_dtype dtype);

/* ---- a5/a4: G-sphere <-> box transforms (basis.py:237-254) ---------- */
/* psi_r[b, :] = ifftn(scatter(psi[b, :])) * N/sqrt(omega); psi_r complex (nbatch, N). */
addft_status addft_psi_to_real(addft_plan plan, addft_dtype dt, int nbatch, double omega,
                               const void *psi, void *psi_r, void *work, size_t work_bytes,
                               void *stream);
/* psi[b, :] = gather(fftn(psi_r[b, :])) * sqrt(omega)/N. */
addft_status addft_real_to_psi(addft_plan plan, addft_dtype dt, int nbatch, double omega,
                               const void *psi_r, void *psi, void *work, size_t work_bytes,
                               void *stream);

/* ---- a2/a6: kinetic diagonal 1/2 |k+G|^2 (hpsi.py:18-26, scf.py:49-51) --
 * bvec: host 9 doubles, reciprocal rows b1,b2,b3 (2 pi inv(L)^T).
 * kpts: host nk*3 doubles (Cartesian).  kin: device (nk, nG) real of dtype dt. */
addft_status addft_kinetic(addft_plan plan, addft_dtype dt, const double *bvec_host, int nk,
                           const double *kpts_host, void *kin, void *stream);

/* ---- a1/a3: matrix-free H psi (ops/hpsi.py:35-50) --------------------
 * hpsi = kin*psi + real_to_psi(psi_to_real(psi) * v_r) + proj^T D conj(proj) psi
 * psi, hpsi: (nk, nb, nG) complex; kin: (nk, nG) real; v_r: (N,) real;
 * proj: (nk, nproj, nG) complex or NULL when nproj == 0; dion: (nproj, nproj) real.
 * All arrays in precision dt.  hpsi must not alias psi. */
addft_status addft_hpsi(addft_plan plan, addft_dtype dt, int nk, int nb, const void *psi,
                        const void *kin, const void *v_r, int nproj, const void *proj,
                        const void *dion, void *hpsi, void *work, size_t work_bytes,
                        void *stream);

/* ---- a9: nonlocal projector contractions (nonlocal_op.py:67-82) ------
 * becp[k, p, b] = sum_G conj(proj[k, p, G]) psi[k, b, G]   (nk, nproj, nb) complex. */
addft_status addft_becp(addft_dtype dt, int nk, int nb, int nG, int nproj, const void *proj,
                        const void *psi, void *becp, void *work, size_t work_bytes,
                        void *stream);
/* hpsi[k, b, G] += sum_p proj[k, p, G] (sum_q dion[p, q] becp[k, q, b]). */
addft_status addft_vnl_apply(addft_dtype dt, int nk, int nb, int nG, int nproj,
                             const void *proj, const void *dion, const void *becp, void *hpsi,
                             void *work, size_t work_bytes, void *stream);
/* e_out[0] (device f64) = sum_k sum_b wocc[k, b] Re(becp^H D becp) ; wocc (nk, nb) f64
 * already holds w_k f_kb g_s. */
addft_status addft_nonlocal_energy(addft_dtype dt, int nk, int nb, int nproj, const void *becp,
                                   const void *dion, const double *wocc, double *e_out, void *work,
                                   size_t work_bytes, void *stream);

/* ---- a7: projector tables (nonlocal_op.py:45-64) ---------------------
 * proj[k, (i,lm), G] = beta(|k+G|) Y_lm(k+G) e^{-i(k+G).R_i} / sqrt(omega)
 * pos_host: nat*3 Cartesian positions (host); proj: (nk, nat*nh, nG) complex of dt. */
addft_status addft_projectors(addft_plan plan, addft_dtype dt, const double *bvec_host,
                              double omega, int nk, const double *kpts_host, int nat,
                              const double *pos_host, const addft_psp *psp, void *proj,
                              void *stream);

/* ---- a10: band density (physics/density.py:18-23) --------------------
 * rho[r] = sum_{k,b} wocc[k, b] |psi_kb(r)|^2 with psi(r) as in addft_psi_to_real.
 * wocc: device (nk*nb) f64 = w_k f_kb g_s;  rho: device (N,) f64 (overwritten). */
addft_status addft_density(addft_plan plan, addft_dtype dt, int nk, int nb, double omega,
                           const void *psi, const double *wocc, double *rho, void *work,
                           size_t work_bytes, void *stream);

/* ---- a12: LDA PZ81 (physics/xc.py:51-73,152-191; native/xc_lda.cu) ---
 * v_xc[i] = d(n eps_xc)/dn at rho[i] (0 below the 1e-14 clamp);
 * sums (device f64[3]) = { sum n eps_x, sum n eps_c, sum v_xc * rho_dc }
 * where rho_dc = rho when rho_dc_or_null is NULL.  Multiply by omega/N for
 * energies.  v_loc / v_h may be NULL; if v_eff is non-NULL it receives
 * v_loc + v_h + v_xc (effective_potential, solver/scf.py:81-92). */
addft_status addft_xc_lda(int n, const double *rho, const double *rho_dc_or_null,
                          const double *v_loc, const double *v_h, double *v_xc, double *v_eff,
                          double *sums, void *work, size_t work_bytes, void *stream);
/* VJP of v_xc: out[i] = f_xc(rho[i]) * g[i]  (xc.py:195-212 custom_vjp). */
addft_status addft_xc_lda_vjp(int n, const double *rho, const double *g, double *out,
                              void *stream);

/* ---- a11: Hartree in G space on the wavefunction shell (hartree.py) ---
 * v_h = Re(N ifftn(scatter(4 pi n_G / G^2))), n_G = fftn(rho)/N on the plan's
 * shell, G = 0 dropped.  e_h (device f64[1]) = omega/2 sum Re(n V*).
 * f64 throughout; work >= addft_work_bytes(plan, 1, ADDFT_F64). */
addft_status addft_hartree(addft_plan plan, const double *bvec_host, double omega,
                           const double *rho, double *v_h, double *e_h, void *work,
                           size_t work_bytes, void *stream);

/* ---- a13: local pseudopotential (physics/local.py:21-39) --------------
 * rho_plan: plan built on the density shell miller_rho.
 * v_loc = Re(N ifftn(scatter(V_loc(G)))), V_loc(G) = (1/omega) sum_i v~(|G|) e^{-iG.R_i}. */
addft_status addft_local_potential(addft_plan rho_plan, const double *bvec_host, double omega,
                                   int nat, const double *pos_host, const addft_psp *psp,
                                   double *v_loc, void *work, size_t work_bytes, void *stream);

/* ---- a20: occupations (physics/occupation.py:25-49) ------------------
 * Fermi-Dirac f = sigmoid((mu - eig)/sigma) with mu from `iters` bisection steps so
 * that spin_deg * sum_k kweights[k] sum_b f = nelec.  All pointers device f64:
 * eig, occ (nk*nb), kweights (nk), mu (1).  sigma must be > 0 (the reference's
 * integer-filling branch for sigma < 1e-6 is handled by the host driver). */
addft_status addft_occupations(int nk, int nb, const double *eig, const double *kweights,
                               double nelec, double sigma, double spin_deg, int iters,
                               double *occ, double *mu, void *stream);

/* ---- a21: Kerker preconditioner of the SCF density mixing (solver/scf.py:202-223)
 * out = alpha * Re(N ifftn(q^2/(q^2 + gg0) fftn(in)/N)), q = 0 dropped; full_plan must hold
 * every point of the box with Miller indices folded to [-n/2, n/2) (scf.py:202-212). */
addft_status addft_kerker(addft_plan full_plan, const double *bvec_host, const double *in, double alpha,
                          double gg0, double *out, void *work, size_t work_bytes, void *stream);
size_t addft_kerker_work_bytes(addft_plan full_plan);

/* ---- a15: FP64 subspace products of the eigensolver (solver/davidson.py:48, :51-52, :59-61:
 * the projections q^H hq and the rotations q u, hq u), computed in double-float arithmetic on the
 * FP32 pipes (~1e-14 relative; operands split into FP32 hi/lo pairs, exact products,
 * compensated sums).  C (M x N, row stride ldc) = op(A) op(B) with
 *   op(A)[i][k] = A[i*sAi + k*sAk], conjugated when conjA != 0,
 *   op(B)[k][j] = B[k*sBk + j*sBj], conjugated when conjB != 0;
 * all complex128, strides in elements.  K is split across CTAs when work holds
 * addft_zgemm_df_work_bytes(M, N, K) bytes (else one pass); the splits are summed in a fixed order. */
addft_status addft_zgemm_df(int M, int N, int K, const void *A, long sAi, long sAk, int conjA,
                            const void *B, long sBk, long sBj, int conjB, void *C, long ldc,
                            void *work, size_t work_bytes, void *stream);
size_t addft_zgemm_df_work_bytes(int M, int N, int K);

/* ---- a24: Ewald (physics/ewald.py:34-77), f64 on the device -----------
 * out (device f64): [0] energy, [1 .. 3*nat] dE/dR, [1+3*nat .. 9+3*nat] dE/deps (row-major). */
addft_status addft_ewald(const double *lattice_host, int nat, const double *pos_host,
                         const double *charges_host, double eta, int nmax, double *out,
                         void *work, size_t work_bytes, void *stream);

/* ---- a25: envelope gradients (api.py:106-113 VJP, hand-derived) -------
 * Kinetic strain term: deps[a][b] += -sum_{k,b,G} wocc |psi|^2 (k+G)_a G_b.
 * out9: device f64[9] (accumulated into: caller zeroes). */
addft_status addft_kinetic_stress(addft_plan plan, addft_dtype dt, const double *bvec_host,
                                  int nk, const double *kpts_host, int nb, const void *psi,
                                  const double *wocc, double *out9, void *work,
                                  size_t work_bytes, void *stream);
/* Density terms with rho = rho(psi) (f64): n(G) on both shells, then
 * out (device f64[5 + 3*nat + 18]): [0] E_loc, [1] E_H, [2..4] reserved,
 * [5 .. 5+3nat) dE_loc/dR, then dE_H/deps (9), dE_loc/deps (9). */
addft_status addft_density_gradients(addft_plan wfc_plan, addft_plan rho_plan,
                                     const double *bvec_host, double omega, int nat,
                                     const double *pos_host, const addft_psp *psp,
                                     const double *rho, double *out, void *work,
                                     size_t work_bytes, void *stream);
/* Nonlocal terms: Y[p, G] = sum_b (wocc_b (D becp)[p, b]) conj(psi_b(G)), then
 * dE_NL/dR and dE_NL/deps from beta, d beta/dq and d Ylm built on the fly.
 * out (device f64[1 + 3*nat + 9]): [0] E_NL, dE/dR (nat*3), dE/deps (9). */
addft_status addft_nonlocal_gradients(addft_plan plan, addft_dtype dt, const double *bvec_host,
                                      double omega, int nk, const double *kpts_host, int nb,
                                      int nat, const double *pos_host, const addft_psp *psp,
                                      const void *psi, const double *wocc, const void *dion,
                                      double *out, void *work, size_t work_bytes, void *stream);

/* ---- scratch sizes of the entry points that need more than a plan slab ---- */
size_t addft_hpsi_work_bytes(addft_plan plan, addft_dtype dt, int nk, int nb, int nproj,
                             int nbatch_chunk);
size_t addft_hartree_work_bytes(addft_plan plan);
size_t addft_local_potential_work_bytes(addft_plan rho_plan);
size_t addft_density_gradients_work_bytes(addft_plan wfc_plan, addft_plan rho_plan, int nat);
size_t addft_nonlocal_gradients_work_bytes(addft_dtype dt, int nk, int nb, int nG, int nat, int nh);
size_t addft_ewald_work_bytes(int nat);

/* ---- arithmetic peaks of this GPU (diagnostic; no counterpart in the reference) ----
 * Runs a kernel that does only `which` = 0: FP32 FMA, 1: FP64 FMA, 2: TF32 mma.sync
 * (m16n8k8, the warp MMA of the split-TF32 becp kernel), 8 CTAs of 256 threads per SM,
 * `iters` loop iterations; 3: tcgen05.mma kind::tf32 128 x 256 x 8 (the MMA of the
 * V_NL apply kernel), one CTA per SM issuing `iters` MMAs into tensor memory; on
 * `stream`, and returns its rate (host *tflops) and CUDA-event time (host *ms).
 * sink: device scratch of >= 2 KB (never read).  Synchronises with the stream. */
addft_status addft_peak_flops(int which, int iters, double *tflops, float *ms, void *sink, void *stream);
/* Device-side error bits of the tcgen05 projector kernels since the last call (bit 0: a
 * bounded wait for tensor-core completion ran out; the kernel then returned without
 * results), cleared by the read; synchronises with the device.  Diagnostic, no
 * counterpart in the reference. */
unsigned addft_tc05_status(void);
/* Device-side error bits of the fused H psi kernel (tuning "colfft" = 2) since the last
 * call (bit 0: a bounded wait for another CTA's work item ran out; that call's H psi is
 * not valid), cleared by the read; synchronises with the device.  Diagnostic, no
 * counterpart in the reference. */
unsigned addft_hpsi_fused_status(void);

/* ---- H psi of host-resident bands (copies overlapped with the compute) ----
 * Same result as addft_hpsi for psi_host / hpsi_host in HOST memory (nk, nb, nG),
 * page-locked for the copies to overlap (pageable memory works, serialised): the
 * bands go through the GPU in chunks of chunk_bands (<= 0: all bands of a k point; the
 * first chunk of the call is half that size, which shortens pipeline fill and drain);
 * chunk c's upload, chunk c - 1's H psi and chunk c - 2's download run at once on
 * an upload stream, the caller's stream and a download stream of the calling thread
 * (created on first use).  kin, v_r, proj, dion and work are device memory as for
 * addft_hpsi; work >= addft_hpsi_host_work_bytes(...) holds two input and two output
 * slots of a chunk and the H psi scratch.  The caller's stream is joined with the
 * last download: synchronising it means hpsi_host is complete.  Counterpart of the
 * reference's host-array call path (ops/hpsi.py:35-50 on NumPy inputs). */
addft_status addft_hpsi_host(addft_plan plan, addft_dtype dt, int nk, int nb, const void *psi_host,
                             const void *kin, const void *v_r, int nproj, const void *proj,
                             const void *dion, void *hpsi_host, int chunk_bands, void *work,
                             size_t work_bytes, void *stream);
size_t addft_hpsi_host_work_bytes(addft_plan plan, addft_dtype dt, int nk, int nb, int nproj,
                                  int chunk_bands);

/* ---- the reference's XLA FFI handlers, argument for argument -----------
 * One call per handler, with the handler's buffers as plain pointers and sizes.
 * Scratch is the caller's (sized by the *_work_bytes functions) where the handler
 * used cudaMallocAsync.  All asynchronous on `stream`. */

/* XcLdaHandler (native/xc_lda.cu:56-75): vxc[i] = d(n eps_xc)/dn and
 * exc (device f64[1]) = sum_i n_i (eps_x + eps_c)(n_i), both at the clamped density
 * n_i = max(rho[i], 1e-14) as the handler computes them (no omega/N factor).  The
 * sum is deterministic (fixed-order block partials) where the handler used atomicAdd. */
addft_status addft_ffi_xc_lda(int n, const double *rho, double *vxc, double *exc, void *work,
                              size_t work_bytes, void *stream);
size_t addft_ffi_xc_lda_work_bytes(void);
/* ScatterC128Handler / ScatterC64Handler (native/pack.cu:43-66,101-125):
 * out (batch, nfft) = 0, then out[b][idx[i]] = coeffs[b][i] for i < nG.
 * dt = ADDFT_F64: complex128, ADDFT_F32: complex64.  Indices outside [0, nfft) are
 * skipped (the handler writes out of bounds); addft_ffi_check_index reports them. */
addft_status addft_ffi_scatter(addft_dtype dt, int batch, int nG, int nfft, const void *coeffs,
                               const int *idx, void *out, void *stream);
/* GatherC128Handler / GatherC64Handler (native/pack.cu:68-87,127-150):
 * out[b][i] = grid[b][idx[i]] (0 for an index outside [0, nfft)). */
addft_status addft_ffi_gather(addft_dtype dt, int batch, int nG, int nfft, const void *grid,
                              const int *idx, void *out, void *stream);
/* *bad (device int) = 1 if any idx[i] lies outside [0, nfft), else 0 (the handlers'
 * "idx length != nG" check is the caller's, since plain pointers carry no length). */
addft_status addft_ffi_check_index(int nG, int nfft, const int *idx, int *bad, void *stream);
/* EighLowestHandler (native/eigh.cu:55-160): for every k of H (nk, n, n) complex128
 * Hermitian, row-major, the nband lowest eigenvalues eig (nk, nband) ascending and
 * eigenvectors vec (nk, nband, n) (row i = eigenvector i, H v = e v).  cuSOLVER
 * zheevd per k (the handler: zheevdx with an index range), opened by dlopen on first
 * use; ADDFT_UNSUPPORTED if libcusolver cannot be opened.  H is not modified.
 * work >= addft_ffi_eigh_lowest_work_bytes(nk, n) (0 if cuSOLVER is unavailable). */
addft_status addft_ffi_eigh_lowest(int nk, int n, int nband, const void *H, double *eig, void *vec,
                                   void *work, size_t work_bytes, void *stream);
size_t addft_ffi_eigh_lowest_work_bytes(int nk, int n);

/* ---- H psi with no device allocation -----------------------------------
 * No counterpart in the reference.  Same inputs, outputs and result as
 * addft_hpsi, but the scratch comes from a static 8 MiB __device__ array
 * inside the library instead of a caller buffer, for callers that may not
 * allocate device memory (an XLA FFI handler inside a JAX program, whose
 * framework pre-reserves most of the device memory; an application under a
 * fixed device-memory budget).  The first call on a device resolves the
 * array's address (make it outside stream capture).  All calls share the
 * array: calls that overlap on the GPU race and must be serialised.
 * Problems whose minimum scratch (becp arrays plus one band of FFT scratch)
 * exceeds the array return ADDFT_UNSUPPORTED.  The array's address is cached
 * per device: a cudaDeviceReset (which also invalidates every plan) is not
 * supported while the library is in use. */
addft_status addft_hpsi_noalloc(addft_plan plan, addft_dtype dt, int nk, int nb, const void *psi,
                                const void *kin, const void *v_r, int nproj, const void *proj,
                                const void *dion, void *hpsi, void *stream);
/* Size in bytes of the static scratch used by addft_hpsi_noalloc. */
size_t addft_hpsi_noalloc_max_scratch_bytes(void);

#ifdef __cplusplus
}
#endif
#endif /* ADDFT_GB300_H */
