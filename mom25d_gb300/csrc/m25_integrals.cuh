// Closed-form integrals of 1/R over a flat triangle (Wilton et al., IEEE
// T-AP 32(3), 1984), the singular part of the MPIE kernels.
#pragma once

#include "m25_common.cuh"

namespace m25 {

// Dunavant degree-5 7-point rule and the 3-point rule (barycentric, weights
// summing to 1), the rules mom25d uses (integrals.py:5-16).
__host__ __device__ inline double tri7_bary(int k, int v) {
  const double a1 = 0.059715871789770, b1 = 0.470142064105115;
  const double a2 = 0.797426985353087, b2 = 0.101286507323456;
  if (k == 0) return 1.0 / 3.0;
  if (k <= 3) return (v == k - 1) ? a1 : b1;
  return (v == k - 4) ? a2 : b2;
}
__host__ __device__ inline double tri7_w(int k) {
  return k == 0 ? 0.225 : (k <= 3 ? 0.132394152788506 : 0.125939180544827);
}
__host__ __device__ inline double tri3_bary(int k, int v) { return v == k ? 2.0 / 3.0 : 1.0 / 6.0; }

// I0 = Int_T 1/R dS', I1 = Int_T (r' - r)/R dS' (in-plane part), with
// R = sqrt(|r - r'|^2 + d^2), for a counter-clockwise triangle v and an
// observer (rx, ry) at height d above its plane. Coordinates may be taken
// relative to any common origin. Edge-by-edge sum of the log term (and for
// d != 0 the arctan "solid angle" term); the observer on an edge's line
// makes that edge's log term vanish.
__device__ inline void potential_integrals(const double v[3][2], double rx, double ry, double d, double& I0,
                                           double& I1x, double& I1y) {
  d = fabs(d);
  const double d2 = d * d;
  I0 = 0.0;
  I1x = 0.0;
  I1y = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const double ax = v[(i + 1) % 3][0], ay = v[(i + 1) % 3][1];
    const double bx = v[(i + 2) % 3][0], by = v[(i + 2) % 3][1];
    const double ex = bx - ax, ey = by - ay;
    const double le = sqrt(ex * ex + ey * ey);
    const double tx = ex / le, ty = ey / le;
    const double nx = ty, ny = -tx;  // outward normal of a CCW edge
    const double dax = ax - rx, day = ay - ry, dbx = bx - rx, dby = by - ry;
    const double sa = dax * tx + day * ty;
    const double sb = dbx * tx + dby * ty;
    const double p = dax * nx + day * ny;
    const double Ra = sqrt(dax * dax + day * day + d2);
    const double Rb = sqrt(dbx * dbx + dby * dby + d2);
    const double q2 = p * p + d2;
    double lg = 0.0;
    if (!(sqrt(q2) <= 1e-12 * le)) {
      // R + s, stable for s < 0 as q^2 / (R - s)
      const double fb = sb >= 0 ? Rb + sb : q2 / (Rb - sb);
      const double fa = sa >= 0 ? Ra + sa : q2 / (Ra - sa);
      lg = log(fb / fa);
    }
    I0 += p * lg;
    if (d != 0.0) I0 -= d * (atan2(p * sb, q2 + d * Rb) - atan2(p * sa, q2 + d * Ra));
    const double g = 0.5 * (q2 * lg + sb * Rb - sa * Ra);
    I1x += nx * g;
    I1y += ny * g;
  }
}

}  // namespace m25
