// Shared-memory batched line FFT for 2,3,5-smooth lengths.
//
// A CTA transforms L lines of length n that live in shared memory.  Line l
// starts at base(l) = (list ? list[l] : l) * base_mul and strides by
// `istride` elements.  The algorithm is the Stockham autosort formulation
// (out-of-place, natural order in and out): stage s with radix R and span Ns
// reads x[j + r n/R], twiddles by W_{Ns R}^{r (j mod Ns)}, does an R-point
// DFT in registers and writes y[(j div Ns) Ns R + (j mod Ns) + r Ns].
// Radices go up to 16; composite radices (6, 8, 9, 10, 12, 15, 16) run as
// nested DFTs in registers, so a 72-point line takes 2 shared-memory passes
// (8 x 9) and a 75-point line 2 passes (5 x 15).
//
// Thread mapping: consecutive threads take the same butterfly of
// consecutive lines.  Callers lay rows out with an odd pitch (in 8/16-byte
// elements), so every pass is free of shared-memory bank conflicts in both
// the row and the column direction, and the twiddle reads of a warp hit one
// address (broadcast).  Index arithmetic uses multiply-shift division.
#pragma once
#include "common.cuh"
#include "fft_consts.cuh"

namespace addft {

// x / d for 0 <= x < 2^31 by multiply-high and shift (round-up magic number).
struct FastDiv {
  unsigned d, m, s;
  __host__ __device__ __forceinline__ FastDiv() : d(1), m(1), s(0) {}
  __host__ __device__ __forceinline__ explicit FastDiv(unsigned dd) : d(dd) {
    s = 0;
    while ((1u << s) < d) ++s;
    m = (unsigned)((((unsigned long long)1 << 32) * (((unsigned long long)1 << s) - d)) / d + 1);
  }
  __device__ __forceinline__ int div(int x) const {
    return (int)((__umulhi((unsigned)x, m) + (unsigned)x) >> s);
  }
};

// constants of the radix-3 and radix-5 DFTs
#define ADDFT_S60 0.86602540378443864676
#define ADDFT_C1_5 0.30901699437494742410
#define ADDFT_C2_5 (-0.80901699437494742410)
#define ADDFT_S1_5 0.95105651629515357212
#define ADDFT_S2_5 0.58778525229247312917

template <int R> struct Split { static constexpr int P = 1, Q = R; };
template <> struct Split<6> { static constexpr int P = 2, Q = 3; };
template <> struct Split<8> { static constexpr int P = 2, Q = 4; };
template <> struct Split<9> { static constexpr int P = 3, Q = 3; };
template <> struct Split<10> { static constexpr int P = 2, Q = 5; };
template <> struct Split<12> { static constexpr int P = 3, Q = 4; };
template <> struct Split<15> { static constexpr int P = 3, Q = 5; };
template <> struct Split<16> { static constexpr int P = 4, Q = 4; };

// x * W_R^e, W_R = e^{-2 pi i / R} (forward) or its conjugate (inverse); e compile-time.
template <int R, int E, bool INV, typename C>
__device__ __forceinline__ C twmul(C x) {
  using Re = decltype(x.x);
  constexpr int e = E % R;
  if constexpr (e == 0) {
    return x;
  } else if constexpr (4 * e == R) {          // W = -i (forward) / +i (inverse)
    return INV ? cconj(cmul_mi(cconj(x))) : cmul_mi(x);
  } else if constexpr (2 * e == R) {
    C y; y.x = -x.x; y.y = -x.y; return y;
  } else if constexpr (4 * e == 3 * R) {      // W = +i (forward) / -i (inverse)
    return INV ? cmul_mi(x) : cconj(cmul_mi(cconj(x)));
  } else {
    const Re c = (Re)TwTab<R>::c[e];
    const Re s = (Re)(INV ? -TwTab<R>::s[e] : TwTab<R>::s[e]);
    // x * (c - i s)
    C y;
    y.x = x.x * c + x.y * s;
    y.y = x.y * c - x.x * s;
    return y;
  }
}

// In-register DFT of size R (INV = false: e^{-2 pi i jk/R}; true: e^{+...}).
template <int R, bool INV, typename C>
__device__ __forceinline__ void dft_reg(C (&v)[R]);

template <int R, bool INV, typename C>
__device__ __forceinline__ void dft_base(C (&v)[R]) {
  using Re = decltype(v[0].x);
  if constexpr (R == 1) {
  } else if constexpr (R == 2) {
    C a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if constexpr (R == 4) {
    C a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
    C b0 = cadd(v[1], v[3]), b1 = csub(v[1], v[3]);
    C ib1 = INV ? cconj(cmul_mi(cconj(b1))) : cmul_mi(b1);   // -/+ i b1
    v[0] = cadd(a0, b0);
    v[2] = csub(a0, b0);
    v[1] = cadd(a1, ib1);
    v[3] = csub(a1, ib1);
  } else if constexpr (R == 3) {
    const Re s = (Re)(INV ? -ADDFT_S60 : ADDFT_S60);
    C t1 = cadd(v[1], v[2]);
    C t2 = csub(v[0], cscale(t1, (Re)0.5));
    C t3 = cscale(cmul_mi(csub(v[1], v[2])), s);
    v[0] = cadd(v[0], t1);
    v[1] = cadd(t2, t3);
    v[2] = csub(t2, t3);
  } else if constexpr (R == 5) {
    const Re c1 = (Re)ADDFT_C1_5, c2 = (Re)ADDFT_C2_5;
    const Re s1 = (Re)(INV ? -ADDFT_S1_5 : ADDFT_S1_5);
    const Re s2 = (Re)(INV ? -ADDFT_S2_5 : ADDFT_S2_5);
    C a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]);
    C a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
    C x0 = v[0];
    C p1 = cadd(x0, cadd(cscale(a1, c1), cscale(a2, c2)));
    C p2 = cadd(x0, cadd(cscale(a1, c2), cscale(a2, c1)));
    C q1 = cmul_mi(cadd(cscale(b1, s1), cscale(b2, s2)));
    C q2 = cmul_mi(csub(cscale(b1, s2), cscale(b2, s1)));
    v[0] = cadd(x0, cadd(a1, a2));
    v[1] = cadd(p1, q1);
    v[4] = csub(p1, q1);
    v[2] = cadd(p2, q2);
    v[3] = csub(p2, q2);
  }
}

// R = P Q in registers: X[k1 + P k2] = sum_q W_Q^{q k2} W_R^{q k1} DFT_P(v[. Q + q])[k1]
template <int R, bool INV, int P, int Q, int K1, typename C>
__device__ __forceinline__ void dft_col(C (&a)[Q][P], C (&v)[R]) {
  if constexpr (K1 < P) {
    C b[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) b[q] = a[q][K1];
    dft_reg<Q, INV>(b);
#pragma unroll
    for (int k2 = 0; k2 < Q; ++k2) v[K1 + P * k2] = b[k2];
    dft_col<R, INV, P, Q, K1 + 1>(a, v);
  }
}

template <int R, bool INV, int P, int Q, int QI, int K1, typename C>
__device__ __forceinline__ void tw_apply(C (&a)[Q][P]) {
  if constexpr (QI < Q) {
    if constexpr (K1 < P) {
      a[QI][K1] = twmul<R, QI * K1, INV>(a[QI][K1]);
      tw_apply<R, INV, P, Q, QI, K1 + 1>(a);
    } else {
      tw_apply<R, INV, P, Q, QI + 1, 0>(a);
    }
  }
}

template <int R, bool INV, typename C>
__device__ __forceinline__ void dft_reg(C (&v)[R]) {
  constexpr int P = Split<R>::P, Q = Split<R>::Q;
  if constexpr (P == 1) {
    dft_base<R, INV>(v);
  } else {
    C a[Q][P];
#pragma unroll
    for (int q = 0; q < Q; ++q)
#pragma unroll
      for (int p = 0; p < P; ++p) a[q][p] = v[p * Q + q];
#pragma unroll
    for (int q = 0; q < Q; ++q) dft_reg<P, INV>(a[q]);
    tw_apply<R, INV, P, Q, 0, 0>(a);
    dft_col<R, INV, P, Q, 0>(a, v);
  }
}

// Identity epilogue of the last stage.
struct NoEpi {
  template <typename C>
  __device__ __forceinline__ C operator()(C v, int line, int pos) const { (void)line; (void)pos; return v; }
};

template <int R, bool INV, bool LAST, typename C, typename Epi>
__device__ __forceinline__ void fft_stage(const C *__restrict__ in, C *__restrict__ out, int n, int Ns,
                                          const FastDiv &dNs, const C *__restrict__ tw, int L,
                                          const FastDiv &dL, const int *__restrict__ list, int base_mul,
                                          int istride, const Epi &epi) {
  const int nr = n / R;
  const int total = L * nr;
  const int twstep = n / (Ns * R);
  // id -> (line l = id mod L, butterfly j = id div L), advanced incrementally
  int j = dL.div((int)threadIdx.x);
  int l = (int)threadIdx.x - j * L;
  const int dj = dL.div((int)blockDim.x);
  const int dl = (int)blockDim.x - dj * L;
  for (int id = threadIdx.x; id < total; id += blockDim.x) {
    const int base = (list ? list[l] : l) * base_mul;
    const int jd = dNs.div(j);
    const int k = j - jd * Ns;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = in[base + (j + r * nr) * istride];
    if (Ns > 1) {
      const int t1 = k * twstep;
#pragma unroll
      for (int r = 1; r < R; ++r) {
        const C w = tw[t1 * r];
        v[r] = INV ? cmulc(v[r], w) : cmul(v[r], w);
      }
    }
    dft_reg<R, INV>(v);
    const int d = jd * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int pos = d + r * Ns;
      out[base + pos * istride] = LAST ? epi(v[r], l, pos) : v[r];
    }
    l += dl;
    j += dj;
    if (l >= L) { l -= L; ++j; }
  }
}

template <int R, bool INV, typename C, typename Epi>
__device__ __forceinline__ void stage_dispatch(bool last, const C *in, C *out, int n, int Ns, const FastDiv &dNs,
                                               const C *tw, int L, const FastDiv &dL, const int *list,
                                               int base_mul, int istride, const Epi &epi) {
  if (last)
    fft_stage<R, INV, true>(in, out, n, Ns, dNs, tw, L, dL, list, base_mul, istride, epi);
  else
    fft_stage<R, INV, false>(in, out, n, Ns, dNs, tw, L, dL, list, base_mul, istride, epi);
}

// Transforms L lines; data starts in A; returns the buffer that holds the result.
// The caller must __syncthreads() before (data ready); every stage ends with one.
// epi(value, line, position) is applied to every output of the last stage.
template <bool INV, typename C, typename Epi = NoEpi>
__device__ C *fft_lines(C *A, C *B, const AxisPlan &ap, const C *tw, int L, const int *list, int base_mul,
                        int istride, const Epi &epi = Epi()) {
  C *in = A, *out = B;
  int Ns = 1;
  const FastDiv dL((unsigned)L);
  for (int s = 0; s < ap.nst; ++s) {
    const int R = ap.rad[s];
    const bool last = s == ap.nst - 1;
    const FastDiv dNs((unsigned)Ns);
    switch (R) {
      case 2: stage_dispatch<2, INV>(last, in, out, ap.n, Ns, dNs, tw, L, dL, list, base_mul, istride, epi); break;
      case 3: stage_dispatch<3, INV>(last, in, out, ap.n, Ns, dNs, tw, L, dL, list, base_mul, istride, epi); break;
      case 4: stage_dispatch<4, INV>(last, in, out, ap.n, Ns, dNs, tw, L, dL, list, base_mul, istride, epi); break;
      case 5: stage_dispatch<5, INV>(last, in, out, ap.n, Ns, dNs, tw, L, dL, list, base_mul, istride, epi); break;
      case 6: stage_dispatch<6, INV>(last, in, out, ap.n, Ns, dNs, tw, L, dL, list, base_mul, istride, epi); break;
      case 8: stage_dispatch<8, INV>(last, in, out, ap.n, Ns, dNs, tw, L, dL, list, base_mul, istride, epi); break;
      case 9: stage_dispatch<9, INV>(last, in, out, ap.n, Ns, dNs, tw, L, dL, list, base_mul, istride, epi); break;
      case 10: stage_dispatch<10, INV>(last, in, out, ap.n, Ns, dNs, tw, L, dL, list, base_mul, istride, epi); break;
      case 12: stage_dispatch<12, INV>(last, in, out, ap.n, Ns, dNs, tw, L, dL, list, base_mul, istride, epi); break;
      case 15: stage_dispatch<15, INV>(last, in, out, ap.n, Ns, dNs, tw, L, dL, list, base_mul, istride, epi); break;
      default: stage_dispatch<16, INV>(last, in, out, ap.n, Ns, dNs, tw, L, dL, list, base_mul, istride, epi); break;
    }
    __syncthreads();
    C *t = in; in = out; out = t;
    Ns *= R;
  }
  return in;
}

template <typename R>
__device__ __forceinline__ const typename Cx<R>::T *twiddles(const PlanDev &pd, int axis) {
  using C = typename Cx<R>::T;
  const C *base = (const C *)(sizeof(R) == 8 ? pd.tw_d : pd.tw_f);
  const int off = axis == 0 ? 0 : (axis == 1 ? pd.n1 : pd.n1 + pd.n2);
  return base + off;
}

// odd pitch (in elements) so that consecutive rows fall on distinct bank pairs
__host__ __device__ __forceinline__ int odd_pitch(int n) { return n | 1; }

}  // namespace addft
