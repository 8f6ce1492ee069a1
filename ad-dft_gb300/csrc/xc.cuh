// PZ81 local-density exchange-correlation at one density point (Hartree units),
// shared by the XC kernels of potentials.cu and the reference-shaped XC entry point.
// Published Perdew-Zunger 1981 parametrisation of the Ceperley-Alder correlation
// energy; reference: src/addft/physics/xc.py:51-73, native/xc_lda.cu:8-26.
#pragma once
#include "common.cuh"

namespace addft {

// ---------------------------------------------------------------------------
// PZ81 (Ha): eps_x, eps_c and derivatives, rho clamped at 1e-14
// ---------------------------------------------------------------------------
struct XcPoint {
  double ex, ec;   // energy densities per particle
  double v;        // d(n eps)/dn  (0 below the clamp)
  double vn;       // d(n eps)/dn at the clamped density (also below the clamp)
  double f;        // d^2(n eps)/dn^2 (0 below the clamp)
};

__device__ __forceinline__ XcPoint pz81(double rho) {
  constexpr double A = 0.0311, Bc = -0.048, Cc = 0.0020, Dc = -0.0116;
  constexpr double Gm = -0.1423, B1 = 1.0529, B2 = 0.3334;
  constexpr double PI = 3.14159265358979323846;
  const double n = fmax(rho, 1e-14);
  const double rs = cbrt(3.0 / (4.0 * PI * n));
  XcPoint o;
  o.ex = -0.75 * cbrt(3.0 * n / PI);
  double d1, d2;
  if (rs < 1.0) {
    const double lr = log(rs);
    o.ec = A * lr + Bc + Cc * rs * lr + Dc * rs;
    d1 = A / rs + Cc * (lr + 1.0) + Dc;
    d2 = -A / (rs * rs) + Cc / rs;
  } else {
    const double sr = sqrt(rs);
    const double den = 1.0 + B1 * sr + B2 * rs;
    const double dp = 0.5 * B1 / sr + B2;
    const double dpp = -0.25 * B1 / (rs * sr);
    o.ec = Gm / den;
    d1 = -Gm * dp / (den * den);
    d2 = -Gm * dpp / (den * den) + 2.0 * Gm * dp * dp / (den * den * den);
  }
  const bool act = rho > 1e-14;
  const double vx = (4.0 / 3.0) * o.ex;
  const double vc = o.ec - (rs / 3.0) * d1;
  const double fx = (4.0 / 9.0) * o.ex / n;
  const double fc = ((2.0 / 3.0) * d1 - (rs / 3.0) * d2) * (-rs / (3.0 * n));
  o.vn = vx + vc;
  o.v = act ? o.vn : 0.0;
  o.f = act ? fx + fc : 0.0;
  return o;
}

}  // namespace addft
