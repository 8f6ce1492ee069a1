// Tabulated radial functions of a pseudopotential (UPF path).
//
// A table holds, for every radial function f on a uniform grid q_i = i dq,
// i < nq, the values f(q_i) and derivatives f'(q_i) (layout [f][2][nq]);
// f(q) between nodes is the cubic Hermite interpolant, whose derivative is
// used for the strain and force terms.  With exact node derivatives the
// interpolation error is below dq^4 max|f''''| / 384.
#pragma once
#include "common.cuh"

namespace addft {

struct RadialTab {
  const double *tab;   // device [nfun][2][nq]
  int nq;
  double dq;
};

__device__ __forceinline__ void radial_eval(const RadialTab &t, int f, double q, double &v, double &dv) {
  const double x = q / t.dq;
  int i = (int)x;
  if (i > t.nq - 2) i = t.nq - 2;
  if (i < 0) i = 0;
  const double s = x - i, s2 = s * s, s3 = s2 * s;
  const double *y = t.tab + (size_t)f * 2 * t.nq;
  const double *m = y + t.nq;
  const double y0 = y[i], y1 = y[i + 1], m0 = m[i] * t.dq, m1 = m[i + 1] * t.dq;
  v = (2 * s3 - 3 * s2 + 1) * y0 + (s3 - 2 * s2 + s) * m0 + (-2 * s3 + 3 * s2) * y1 + (s3 - s2) * m1;
  dv = ((6 * s2 - 6 * s) * y0 + (3 * s2 - 4 * s + 1) * m0 + (-6 * s2 + 6 * s) * y1 + (3 * s2 - 2 * s) * m1) / t.dq;
}

}  // namespace addft
