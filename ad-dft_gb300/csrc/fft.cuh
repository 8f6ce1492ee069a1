// Shared-memory batched line FFT for 2,3,5-smooth lengths.
//
// A CTA transforms L lines of length n that live in shared memory.  Each line
// l starts at base(l) = (list ? list[l] : l) * base_mul and strides by
// `istride` elements.  The algorithm is the Stockham autosort formulation
// (out-of-place, natural order in and out) with mixed radix 2/3/4/5 stages:
// stage s with radix R and span Ns reads x[j + r n/R], twiddles by
// W_{Ns R}^{r (j mod Ns)}, does a radix-R DFT and writes
// y[(j div Ns) Ns R + (j mod Ns) + r Ns].  Between stages the two shared
// buffers swap roles; the function returns the buffer holding the result.
//
// Thread mapping: when the line is contiguous (istride == 1) consecutive
// threads take consecutive butterflies of one line; when lines are strided
// consecutive threads take the same butterfly of consecutive lines, so both
// cases keep shared-memory accesses on consecutive words.
#pragma once
#include "common.cuh"

namespace addft {

// constants of the radix-3 and radix-5 DFTs
#define ADDFT_S60 0.86602540378443864676
#define ADDFT_C1_5 0.30901699437494742410
#define ADDFT_C2_5 (-0.80901699437494742410)
#define ADDFT_S1_5 0.95105651629515357212
#define ADDFT_S2_5 0.58778525229247312917

// In-register DFT of size R.  INV = false: e^{-2 pi i jk/R}; true: e^{+...}.
template <int R, bool INV, typename C>
__device__ __forceinline__ void dft_small(C (&v)[R]) {
  using Re = decltype(v[0].x);
  if constexpr (R == 2) {
    C a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if constexpr (R == 4) {
    C a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
    C b0 = cadd(v[1], v[3]), b1 = csub(v[1], v[3]);
    // forward: y1 = a1 - i b1, y3 = a1 + i b1
    C ib1 = cmul_mi(b1);  // -i b1
    if (INV) ib1 = cconj(cmul_mi(cconj(b1)));  // +i b1
    v[0] = cadd(a0, b0);
    v[2] = csub(a0, b0);
    v[1] = cadd(a1, ib1);
    v[3] = csub(a1, ib1);
  } else if constexpr (R == 3) {
    const Re s = (Re)(INV ? -ADDFT_S60 : ADDFT_S60);
    C t1 = cadd(v[1], v[2]);
    C t2 = csub(v[0], cscale(t1, (Re)0.5));
    C d = csub(v[1], v[2]);
    // -i s d
    C t3 = cscale(cmul_mi(d), s);
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
    // q1 = -i (s1 b1 + s2 b2), q2 = -i (s2 b1 - s1 b2)
    C q1 = cmul_mi(cadd(cscale(b1, s1), cscale(b2, s2)));
    C q2 = cmul_mi(csub(cscale(b1, s2), cscale(b2, s1)));
    v[0] = cadd(x0, cadd(a1, a2));
    v[1] = cadd(p1, q1);
    v[4] = csub(p1, q1);
    v[2] = cadd(p2, q2);
    v[3] = csub(p2, q2);
  }
}

template <int R, bool INV, typename C>
__device__ __forceinline__ void fft_stage(const C *__restrict__ in, C *__restrict__ out, int n,
                                          int Ns, const C *__restrict__ tw, int L,
                                          const int *__restrict__ list, int base_mul,
                                          int istride) {
  const int nr = n / R;
  const int total = L * nr;
  const int twstep = n / (Ns * R);
  const bool jfast = (istride == 1);
  for (int id = threadIdx.x; id < total; id += blockDim.x) {
    int j, l;
    if (jfast) {
      l = id / nr;
      j = id - l * nr;
    } else {
      j = id / L;
      l = id - j * L;
    }
    const int base = (list ? list[l] : l) * base_mul;
    const int k = j % Ns;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = in[base + (j + r * nr) * istride];
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        const C w = tw[(k * r * twstep)];
        v[r] = INV ? cmulc(v[r], w) : cmul(v[r], w);
      }
    }
    dft_small<R, INV>(v);
    const int d = (j / Ns) * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) out[base + (d + r * Ns) * istride] = v[r];
  }
}

// Transforms L lines; data starts in A; returns pointer to the buffer with the result.
// Caller must __syncthreads() before (data ready) — this function syncs after every stage.
template <bool INV, typename C>
__device__ C *fft_lines(C *A, C *B, const AxisPlan &ap, const C *tw, int L, const int *list,
                        int base_mul, int istride) {
  C *in = A, *out = B;
  int Ns = 1;
  for (int s = 0; s < ap.nst; ++s) {
    const int R = ap.rad[s];
    switch (R) {
      case 2: fft_stage<2, INV>(in, out, ap.n, Ns, tw, L, list, base_mul, istride); break;
      case 3: fft_stage<3, INV>(in, out, ap.n, Ns, tw, L, list, base_mul, istride); break;
      case 4: fft_stage<4, INV>(in, out, ap.n, Ns, tw, L, list, base_mul, istride); break;
      default: fft_stage<5, INV>(in, out, ap.n, Ns, tw, L, list, base_mul, istride); break;
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

}  // namespace addft
