// Port de-embedding on the device (Engine/mom25d/solver.py:1276-1325):
// triangle charges (1076-1091), line voltages at the feed sample points
// (1101-1125), cut currents and voltages (PortModel, 604-610), the wave fit
// (fit_waves, 618-670: Nelder-Mead on gamma with per-dataset 2x2 least
// squares) and S with reciprocity-fitted reference impedances (1316-1325,
// 1357-1427).
#include <cmath>
#include <vector>

#include "m25_integrals.cuh"
#include "m25_internal.h"

namespace m25 {

constexpr int kMaxPorts = 8;
constexpr int kMaxSamples = 64;   // fit-window cuts per port
constexpr int kMaxDatasets = 16;  // (port, excitation) datasets of one port group

// charge density per triangle, q = -div J / (jw)
__global__ void charges_kernel(int nt, int nb, int P, const TriData<double>* __restrict__ td,
                               const int32_t* __restrict__ tri_basis, const zd* __restrict__ x, double omega,
                               zd* __restrict__ q) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  const zd jw(0.0, omega);
  for (int e = 0; e < P; ++e) {
    zd div(0.0);
    for (int i = 0; i < 3; ++i) {
      int b = tri_basis[3 * t + i];
      if (b >= 0) div += x[(int64_t)b * P + e] * td[t].cV[i];
    }
    q[(int64_t)t * P + e] = -div / jw;
  }
}

// via segments drain their upper triangles and feed their lower ones
__global__ void via_charges_kernel(int nv, int nb, int P, const int32_t* __restrict__ seg_pad_off,
                                   const int32_t* __restrict__ seg_pad, const double* __restrict__ seg_pad_w,
                                   const int32_t* __restrict__ pad_tris, const zd* __restrict__ x, double omega,
                                   zd* __restrict__ q) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nv) return;
  const zd jw(0.0, omega);
  for (int e = seg_pad_off[k]; e < seg_pad_off[k + 1]; ++e) {
    int t = pad_tris[seg_pad[e]];
    for (int c = 0; c < P; ++c) {
      zd v = -(x[(int64_t)(nb + k) * P + c] * seg_pad_w[e]) / jw;
      atomicAdd(&q[(int64_t)t * P + c].re, v.re);
      atomicAdd(&q[(int64_t)t * P + c].im, v.im);
    }
  }
}

__device__ inline zd spline_w(const double* __restrict__ rho, int n, const zd* __restrict__ coef, int pair, double r) {
  int i;
  if (r < rho[1]) i = 0;
  else if (r >= rho[n - 2]) i = n - 2;
  else {
    int lo = 1, hi = n - 2;
    while (hi - lo > 1) {
      int mid = (lo + hi) >> 1;
      if (r < rho[mid]) hi = mid; else lo = mid;
    }
    i = lo;
  }
  double dx = r - rho[i];
  const zd* c = coef + ((size_t)pair * (n - 1) + i) * 12;
  double z = dx, z2 = dx * dx, z3 = z2 * dx;
  return c[3 * 3 + 2] + c[2 * 3 + 2] * z + c[1 * 3 + 2] * z2 + c[0 * 3 + 2] * z3;
}

// sum_k w_k S_W(|p - r_k|) + c_W I0(t, p) / 4pi of one triangle in fp64
// (Engine/mom25d/solver.py line voltages: 7-point smooth part plus the
// closed-form 1/R integral)
__device__ inline zd lv_tri64(const TriData<double>& T, double ox, double oy, double dz, int nrho,
                              const double* __restrict__ rho, const zd* __restrict__ coef, int pair, zd cw) {
  zd k0w(0.0);
  for (int k = 0; k < 7; ++k) {
    double dx = ox - T.q7[k][0], dy = oy - T.q7[k][1];
    k0w += spline_w(rho, nrho, coef, pair, sqrt(dx * dx + dy * dy)) * T.w7[k];
  }
  if (cw.re != 0.0 || cw.im != 0.0) {
    double I0, I1x, I1y;
    potential_integrals(T.v, ox, oy, dz, I0, I1x, I1y);
    k0w += cw * (I0 / (4.0 * kPi));
  }
  return k0w;
}

// sum of the per-port accumulators over the CTA, times 1/eps0, into phi[m]
__device__ inline void lv_reduce(int P, zd* acc, zd* __restrict__ phi_m) {
  __shared__ double red[32][2];
  const double ie0 = 1.0 / eps0();
  for (int e = 0; e < P; ++e) {
    double a = acc[e].re, b = acc[e].im;
    for (int o = 16; o; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if ((threadIdx.x & 31) == 0) {
      red[threadIdx.x >> 5][0] = a;
      red[threadIdx.x >> 5][1] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double sa = 0, sb = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        sa += red[w][0];
        sb += red[w][1];
      }
      phi_m[e] = zd(sa, sb) * ie0;
    }
    __syncthreads();
  }
}

// phi[m][e] = (1/eps0) sum_t [sum_k w_k S_W(|p_m - r_k|) + c_W I0(t, p_m) / 4pi] q[t][e]
__global__ void line_voltage_kernel(int nt, int P, int L, const double* __restrict__ pts,
                                    const int32_t* __restrict__ pt_level, const double* __restrict__ cen,
                                    const TriData<double>* __restrict__ td, const int32_t* __restrict__ tri_layer,
                                    const double* __restrict__ level_z, int nrho, const double* __restrict__ rho,
                                    const zd* __restrict__ coef, const zd* __restrict__ cW, const zd* __restrict__ q,
                                    zd* __restrict__ phi) {
  int m = blockIdx.x;
  int li = pt_level[m];
  double px = pts[2 * m], py = pts[2 * m + 1];
  zd acc[kMaxPorts];
  for (int t = threadIdx.x; t < nt; t += blockDim.x) {
    int ls = tri_layer[t];
    int pair = li * L + ls;
    zd k0w = lv_tri64(td[t], px - cen[2 * t], py - cen[2 * t + 1], fabs(level_z[li] - level_z[ls]), nrho, rho, coef,
                      pair, cW[pair]);
    for (int e = 0; e < P; ++e) acc[e] += k0w * q[(int64_t)t * P + e];
  }
  lv_reduce(P, acc, phi + (int64_t)m * P);
}

// Mixed precision: a (point, triangle) pair at least kLvFarEdges longest
// edges apart is summed in fp32 from the fp32 tables, with the 1/R part of
// the W kernel integrated by the same 7-point rule instead of in closed form
// (relative error of the rule below 1e-7 at that distance, under the fp32
// rounding of the rest); nearer pairs as line_voltage_kernel. The products
// with the charges and the sums over triangles stay in fp64.
constexpr float kLvFarEdges = 5.0f;

__host__ __device__ inline size_t lv_mixed_smem(int L, int nrho) {
  return sizeof(float) * (((size_t)nrho + 3) / 4 * 4 + (size_t)L * (nrho - 1) * 8);
}

__global__ void __launch_bounds__(256) line_voltage_mixed_kernel(
    int nt, int P, int L, const double* __restrict__ pts, const int32_t* __restrict__ pt_level,
    const double* __restrict__ cen, const TriData<double>* __restrict__ td, const TriData<float>* __restrict__ td32,
    const int32_t* __restrict__ tri_layer, const double* __restrict__ level_z, int nrho, const double* __restrict__ rho,
    const float* __restrict__ rho32, const zd* __restrict__ coef, const zf* __restrict__ coef32,
    const zd* __restrict__ cW, const zd* __restrict__ q, zd* __restrict__ phi) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float* xf = reinterpret_cast<float*>(smem_raw);
  float* tab = xf + (nrho + 3) / 4 * 4;  // [ls][interval][power 0..3][re, im] of S_W
  const int m = blockIdx.x;
  const int li = pt_level[m];
  const int ni = nrho - 1;
  for (int i = threadIdx.x; i < nrho; i += blockDim.x) xf[i] = rho32[i];
  for (int e = threadIdx.x; e < L * ni * 4; e += blockDim.x) {
    const int ls = e / (ni * 4), r = e - ls * ni * 4, iv = r >> 2, pw = r & 3;
    const zf v = coef32[(((size_t)(li * L + ls) * ni + iv) * 4 + pw) * 3 + 2];
    tab[(size_t)e * 2] = v.re;
    tab[(size_t)e * 2 + 1] = v.im;
  }
  __syncthreads();
  const double px = pts[2 * m], py = pts[2 * m + 1];
  zd acc[kMaxPorts];
  for (int t = threadIdx.x; t < nt; t += blockDim.x) {
    const int ls = tri_layer[t];
    const int pair = li * L + ls;
    const double ox = px - cen[2 * t], oy = py - cen[2 * t + 1];
    const double dz = fabs(level_z[li] - level_z[ls]);
    const zd cw = cW[pair];
    const TriData<float>& T = td32[t];
    const float ox32 = (float)ox, oy32 = (float)oy, far = kLvFarEdges * T.size;
    zd k0w;
    if (ox32 * ox32 + oy32 * oy32 >= far * far) {
      const float* tb = tab + (size_t)ls * ni * 8;
      const float dz2 = (float)(dz * dz);
      const float cr = (float)(cw.re * (1.0 / (4.0 * kPi))), ci = (float)(cw.im * (1.0 / (4.0 * kPi)));
      float sr = 0.f, si = 0.f;
#pragma unroll
      for (int k = 0; k < 7; ++k) {
        const float dx = ox32 - T.q7[k][0], dy = oy32 - T.q7[k][1];
        const float r2 = dx * dx + dy * dy;
        const float r = sqrtf(r2);
        int i;
        if (r < xf[1]) i = 0;
        else if (r >= xf[nrho - 2]) i = nrho - 2;
        else {
          int lo = 1, hi = nrho - 2;
          while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (r < xf[mid]) hi = mid; else lo = mid;
          }
          i = lo;
        }
        const float z = r - xf[i];
        const float4 c01 = *reinterpret_cast<const float4*>(tb + (size_t)i * 8);
        const float4 c23 = *reinterpret_cast<const float4*>(tb + (size_t)i * 8 + 4);
        // powers stored from z^3 down to z^0
        float vr = fmaf(fmaf(fmaf(c01.x, z, c01.z), z, c23.x), z, c23.z);
        float vi = fmaf(fmaf(fmaf(c01.y, z, c01.w), z, c23.y), z, c23.w);
        const float ir = rsqrtf(r2 + dz2);
        vr = fmaf(cr, ir, vr);
        vi = fmaf(ci, ir, vi);
        sr = fmaf(vr, T.w7[k], sr);
        si = fmaf(vi, T.w7[k], si);
      }
      k0w = zd(sr, si);
    } else {
      k0w = lv_tri64(td[t], ox, oy, dz, nrho, rho, coef, pair, cw);
    }
    for (int e = 0; e < P; ++e) acc[e] += k0w * q[(int64_t)t * P + e];
  }
  lv_reduce(P, acc, phi + (int64_t)m * P);
}

// cut currents I[c][e] = sum sign len x and cut voltages V[c][e] = mean of phi over its 8 points
__global__ void cuts_kernel(int ncut, int P, const int32_t* __restrict__ cut_off, const int32_t* __restrict__ cut_edge,
                            const double* __restrict__ cut_w, const zd* __restrict__ x, const zd* __restrict__ phi,
                            int nper, zd* __restrict__ I, zd* __restrict__ V) {
  int gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= ncut * P) return;
  int c = gid / P, e = gid % P;
  zd s(0.0);
  for (int k = cut_off[c]; k < cut_off[c + 1]; ++k) s += x[(int64_t)cut_edge[k] * P + e] * cut_w[k];
  I[gid] = s;
  zd v(0.0);
  for (int k = 0; k < nper; ++k) v += phi[((int64_t)c * nper + k) * P + e];
  V[gid] = v / double(nper);
}

// ------------------------------------------------------------------ fit
struct FitArgs {
  int P, ngroup;
  int E;                    // excitation columns of x (P feeds, then internal ports)
  int group_of[kMaxPorts];
  int ns[kMaxPorts];
  int s_off[kMaxPorts];     // offset of port p's cuts in s / I / V rows
  double beta0[kMaxPorts];  // per group
  double v_weight;
  const double* s;          // concatenated cut positions
  const zd* I;              // (sum ns, P)
  const zd* V;              // (sum ns, P)
  zd* A;                    // (P, P) incident amplitudes
  zd* B;                    // (P, P)
  zd* gamma;                // (P)
  zd* zline;                // (P)
  double* resid;            // (P)
  int* iters;               // (ngroup) iterations of the fit; lossless: minus them when beta ended at a bound
  int lossless;             // 1: gamma = j beta, bounded Brent search over beta / |beta0|
  double lo[kMaxPorts], hi[kMaxPorts];  // per group: the search interval of beta / |beta0|
  zd* S;                    // (P, P)
  double* z0;               // (P)
};

__device__ inline double warp_sum(double v) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ inline zd warp_sum(zd v) { return zd(warp_sum(v.re), warp_sum(v.im)); }

// Residual of the wave model at gamma for the datasets of one group (all lanes
// of the warp return the same value); optionally stores coefficients, z0.
__device__ double wave_objective(const FitArgs& a, int grp, zd g, double Inrm, double Vnrm, bool store) {
  const int lane = threadIdx.x & 31;
  double res = 0.0;
  zd UV(0.0);
  double UU = 0.0;
  constexpr int kPer = kMaxSamples / 32;
  zd U[kMaxDatasets][kPer];
  int nd = 0;
  for (int p = 0; p < a.P; ++p) {
    if (a.group_of[p] != grp) continue;
    const int ns = a.ns[p], off = a.s_off[p];
    // e^{+-g s} and the QR of [e^{gs}, e^{-gs}] depend on the port only:
    // shared by its P excitations
    zd ep[kPer], em[kPer], q1[kPer], q2[kPer];
    double n11 = 0;
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      int i = lane + 32 * u;
      if (i < ns) {
        double sv = a.s[off + i];
        ep[u] = cexp(g * sv);
        // e^{-g s} = 1 / e^{g s}: one reciprocal instead of a second exp and sincos
        const double m2 = norm2(ep[u]);
        em[u] = zd(ep[u].re / m2, -ep[u].im / m2);
        n11 += m2;
      } else {
        ep[u] = em[u] = zd(0.0);
      }
    }
    // two-column least squares by modified Gram-Schmidt with one re-orthogonalisation
    const double r11 = sqrt(warp_sum(n11));
    zd r12(0.0);
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      q1[u] = ep[u] / r11;
      r12 += conj(q1[u]) * em[u];
    }
    r12 = warp_sum(r12);
    zd r12b(0.0);
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      q2[u] = em[u] - r12 * q1[u];
      r12b += conj(q1[u]) * q2[u];
    }
    r12b = warp_sum(r12b);
    double n22 = 0;
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      q2[u] -= r12b * q1[u];
      n22 += norm2(q2[u]);
    }
    r12 += r12b;
    const double r22 = sqrt(warp_sum(n22));
#pragma unroll
    for (int u = 0; u < kPer; ++u) q2[u] = q2[u] / r22;
    for (int e = 0; e < a.E; ++e, ++nd) {
      zd Iv[kPer];
      zd b1(0.0), b2(0.0);
#pragma unroll
      for (int u = 0; u < kPer; ++u) {
        int i = lane + 32 * u;
        Iv[u] = i < ns ? a.I[(int64_t)(off + i) * a.E + e] : zd(0.0);
        b1 += conj(q1[u]) * Iv[u];
        b2 += conj(q2[u]) * Iv[u];
      }
      b1 = warp_sum(b1);
      b2 = warp_sum(b2);
      const zd c1 = b2 / zd(r22);
      const zd c0 = (b1 - r12 * c1) / zd(r11);
      double rr = 0;
#pragma unroll
      for (int u = 0; u < kPer; ++u) {
        zd d = c0 * ep[u] + c1 * em[u] - Iv[u];
        rr += norm2(d);
        U[nd][u] = c0 * ep[u] - c1 * em[u];
        if (lane + 32 * u < ns) {
          zd Vv = a.V[(int64_t)(off + lane + 32 * u) * a.E + e];
          UV += conj(U[nd][u]) * Vv;
          UU += norm2(U[nd][u]);
        }
      }
      res += warp_sum(rr) / Inrm;
      if (store && lane == 0) {
        a.A[p * a.E + e] = c0;
        a.B[p * a.E + e] = c1;
      }
    }
  }
  zd z0 = warp_sum(UV) / zd(warp_sum(UU));
  double rv = 0;
  nd = 0;
  for (int p = 0; p < a.P; ++p) {
    if (a.group_of[p] != grp) continue;
    const int ns = a.ns[p], off = a.s_off[p];
    for (int e = 0; e < a.E; ++e, ++nd) {
#pragma unroll
      for (int u = 0; u < kPer; ++u)
        if (lane + 32 * u < ns) {
          zd Vv = a.V[(int64_t)(off + lane + 32 * u) * a.E + e];
          rv += norm2(Vv - z0 * U[nd][u]);
        }
    }
  }
  res += a.v_weight * warp_sum(rv) / Vnrm;
  if (store && lane == 0)
    for (int p = 0; p < a.P; ++p)
      if (a.group_of[p] == grp) a.zline[p] = z0;
  return res;
}

// Minimum of f on [lo, hi] by Brent's method (R. P. Brent, "Algorithms for
// Minimization without Derivatives", 1973, ch. 5, procedure localmin):
// golden-section steps, replaced by the minimum of the parabola through the
// three best points whenever that falls inside the bracket and moves less
// than half the step before last; never closer than tol to a point already
// evaluated. tol = sqrt(eps) |x| + xatol / 3, the tolerance with which
// mom25d's minimize_scalar(method="bounded", xatol=...) calls it; stops when
// the bracket around the best point x is within 2 tol of it, or after
// maxfun evaluations. *nfun = evaluations made.
template <class F>
__device__ double brent_minimize(F f, double lo, double hi, double xatol, int maxfun, int* nfun) {
  const double cgold = 0.5 * (3.0 - sqrt(5.0));
  const double reps = 1.4901161193847656e-08;  // sqrt(2^-52)
  double a = lo, b = hi;
  double x = a + cgold * (b - a), w = x, v = x;
  double fx = f(x), fw = fx, fv = fx;
  double d = 0.0, e = 0.0;
  int n = 1;
  while (n < maxfun) {
    const double m = 0.5 * (a + b);
    const double tol = reps * fabs(x) + xatol / 3.0, t2 = 2.0 * tol;
    if (fabs(x - m) <= t2 - 0.5 * (b - a)) break;
    bool golden = true;
    if (fabs(e) > tol) {
      // parabola through (x, fx), (w, fw), (v, fv): its vertex is x + p / q
      double r = (x - w) * (fx - fv);
      double q = (x - v) * (fx - fw);
      double p = (x - v) * q - (x - w) * r;
      q = 2.0 * (q - r);
      if (q > 0.0) p = -p;
      else q = -q;
      const double e_prev = e;
      e = d;
      if (fabs(p) < fabs(0.5 * q * e_prev) && p > q * (a - x) && p < q * (b - x)) {
        d = p / q;
        const double u = x + d;
        if (u - a < t2 || b - u < t2) d = x < m ? tol : -tol;  // not too near the ends
        golden = false;
      }
    }
    if (golden) {
      e = (x < m ? b : a) - x;  // into the larger part of the bracket
      d = cgold * e;
    }
    const double u = x + (fabs(d) >= tol ? d : (d > 0.0 ? tol : -tol));
    const double fu = f(u);
    ++n;
    if (fu <= fx) {
      if (u < x) b = x;
      else a = x;
      v = w; fv = fw;
      w = x; fw = fx;
      x = u; fx = fu;
    } else {
      if (u < x) a = u;
      else b = u;
      if (fu <= fw || w == x) {
        v = w; fv = fw;
        w = u; fw = fu;
      } else if (fu <= fv || v == x || v == w) {
        v = u; fv = fu;
      }
    }
  }
  *nfun = n;
  return x;
}

// One CTA of four warps per port group: Nelder-Mead with scipy's
// coefficients (reflection 1, expansion 2, contraction 0.5, shrink 0.5),
// initial simplex 5 % steps, stopping when the simplex spans <= xatol and its
// values <= fatol. Each iteration evaluates its four possible trial points
// (reflection, expansion, outside and inside contraction) at once, one warp
// each (one SM sub-partition and its fp64 unit each), and then takes scipy's
// decisions on those values: the objective is a pure function, so the
// simplex follows the sequential method's path exactly, in about half the
// sequential rounds of objective evaluations.
constexpr int kFitWarps = 4;

__global__ void __launch_bounds__(32 * kFitWarps) fit_kernel(FitArgs a) {
  const int grp = blockIdx.x, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __shared__ double pts[kFitWarps][2];
  __shared__ double vals[kFitWarps];
  if (grp >= a.ngroup) return;
  const double scale = fabs(a.beta0[grp]);
  double Inrm = 0, Vnrm = 0;
  for (int p = 0; p < a.P; ++p) {
    if (a.group_of[p] != grp) continue;
    for (int i = lane; i < a.ns[p]; i += 32)
      for (int e = 0; e < a.E; ++e) {
        Inrm += norm2(a.I[(int64_t)(a.s_off[p] + i) * a.E + e]);
        Vnrm += norm2(a.V[(int64_t)(a.s_off[p] + i) * a.E + e]);
      }
  }
  Inrm = warp_sum(Inrm);
  Vnrm = warp_sum(Vnrm);
  // objective values of the first n points of pts, one warp per point
  auto round = [&](int n) {
    __syncthreads();
    if (warp < n) {
      const double v = wave_objective(a, grp, zd(scale * pts[warp][0], scale * pts[warp][1]), Inrm, Vnrm, false);
      if (lane == 0) vals[warp] = v;
    }
    __syncthreads();
  };
  if (a.lossless) {
    // gamma = j beta (a bound mode: no attenuation to fit), beta = |beta0| b
    // with b in [lo, hi] found by Brent's bounded minimisation (one objective
    // evaluation per step, on warp 0)
    if (warp != 0) return;
    auto f = [&](double b) { return wave_objective(a, grp, zd(0.0, scale * b), Inrm, Vnrm, false); };
    int n = 0;
    const double b = brent_minimize(f, a.lo[grp], a.hi[grp], 1e-12, 500, &n);
    const zd g(0.0, scale * b);
    const double res = wave_objective(a, grp, g, Inrm, Vnrm, true);
    if (lane == 0) {
      const bool at_bound = fmin(b - a.lo[grp], a.hi[grp] - b) < 1e-3;
      a.iters[grp] = at_bound ? -n : n;
      for (int p = 0; p < a.P; ++p)
        if (a.group_of[p] == grp) {
          a.gamma[p] = g;
          a.resid[p] = sqrt(res);
        }
    }
    return;
  }
  const double xatol = 1e-10, fatol = 1e-16;
  double sim[3][2], fs[3];
  // gamma0 = 1e-3 b0 + j b0, scaled by |b0|
  const double x0 = 1e-3 * a.beta0[grp] / scale, x1 = a.beta0[grp] / scale;
  sim[0][0] = x0; sim[0][1] = x1;
  sim[1][0] = x0 != 0 ? 1.05 * x0 : 0.00025; sim[1][1] = x1;
  sim[2][0] = x0; sim[2][1] = x1 != 0 ? 1.05 * x1 : 0.00025;
  if (threadIdx.x == 0)
    for (int k = 0; k < 3; ++k) {
      pts[k][0] = sim[k][0];
      pts[k][1] = sim[k][1];
    }
  round(3);
  for (int k = 0; k < 3; ++k) fs[k] = vals[k];
  auto sort3 = [&]() {  // stable insertion sort by value
    for (int i = 1; i < 3; ++i)
      for (int j = i; j > 0 && fs[j] < fs[j - 1]; --j) {
        double t = fs[j]; fs[j] = fs[j - 1]; fs[j - 1] = t;
        for (int d = 0; d < 2; ++d) { double u = sim[j][d]; sim[j][d] = sim[j - 1][d]; sim[j - 1][d] = u; }
      }
  };
  sort3();
  int it = 1;
  while (it < 4000) {
    double dx = 0, df = 0;
    for (int k = 1; k < 3; ++k) {
      dx = fmax(dx, fmax(fabs(sim[k][0] - sim[0][0]), fabs(sim[k][1] - sim[0][1])));
      df = fmax(df, fabs(fs[0] - fs[k]));
    }
    if (dx <= xatol && df <= fatol) break;
    double xb[2], xr[2], xe[2], xo[2], xi[2];
    for (int d = 0; d < 2; ++d) {
      xb[d] = (sim[0][d] + sim[1][d]) / 2.0;
      xr[d] = 2.0 * xb[d] - sim[2][d];
      xe[d] = 3.0 * xb[d] - 2.0 * sim[2][d];
      xo[d] = 1.5 * xb[d] - 0.5 * sim[2][d];
      xi[d] = 0.5 * xb[d] + 0.5 * sim[2][d];
    }
    if (threadIdx.x == 0)
      for (int d = 0; d < 2; ++d) {
        pts[0][d] = xr[d];
        pts[1][d] = xe[d];
        pts[2][d] = xo[d];
        pts[3][d] = xi[d];
      }
    round(4);
    const double fr = vals[0], fe = vals[1], fo = vals[2], fi = vals[3];
    bool shrink = false;
    if (fr < fs[0]) {
      if (fe < fr) { sim[2][0] = xe[0]; sim[2][1] = xe[1]; fs[2] = fe; }
      else { sim[2][0] = xr[0]; sim[2][1] = xr[1]; fs[2] = fr; }
    } else if (fr < fs[1]) {
      sim[2][0] = xr[0]; sim[2][1] = xr[1]; fs[2] = fr;
    } else if (fr < fs[2]) {
      if (fo <= fr) { sim[2][0] = xo[0]; sim[2][1] = xo[1]; fs[2] = fo; }
      else shrink = true;
    } else {
      if (fi < fs[2]) { sim[2][0] = xi[0]; sim[2][1] = xi[1]; fs[2] = fi; }
      else shrink = true;
    }
    if (shrink) {
      for (int j = 1; j < 3; ++j)
        for (int d = 0; d < 2; ++d) sim[j][d] = sim[0][d] + 0.5 * (sim[j][d] - sim[0][d]);
      if (threadIdx.x == 0)
        for (int j = 1; j < 3; ++j) {
          pts[j - 1][0] = sim[j][0];
          pts[j - 1][1] = sim[j][1];
        }
      round(2);
      fs[1] = vals[0];
      fs[2] = vals[1];
    }
    ++it;
    sort3();
  }
  if (warp == 0) {
    zd g(scale * sim[0][0], scale * sim[0][1]);
    double res = wave_objective(a, grp, g, Inrm, Vnrm, true);
    if (lane == 0) {
      a.iters[grp] = it;
      for (int p = 0; p < a.P; ++p)
        if (a.group_of[p] == grp) {
          a.gamma[p] = g;
          a.resid[p] = sqrt(res);
        }
    }
  }
}

// After the fits of all groups: SI = -B A^-1, the reference impedances and S.
__global__ void fit_finish_kernel(FitArgs a) {
  if (threadIdx.x != 0) return;
  // SI = -B A^-1 (Gauss-Jordan with partial pivoting on [A^T | -B^T]: X^T = A^-T (-B^T))
  const int P = a.P;
  zd M[kMaxPorts][2 * kMaxPorts];
  for (int i = 0; i < P; ++i)
    for (int j = 0; j < P; ++j) {
      M[i][j] = a.A[j * P + i];          // A^T
      M[i][P + j] = -a.B[j * P + i];     // -B^T
    }
  for (int c = 0; c < P; ++c) {
    int pr = c;
    for (int r = c + 1; r < P; ++r)
      if (cabs(M[r][c]) > cabs(M[pr][c])) pr = r;
    for (int j = 0; j < 2 * P; ++j) { zd t = M[c][j]; M[c][j] = M[pr][j]; M[pr][j] = t; }
    zd piv = M[c][c];
    for (int j = 0; j < 2 * P; ++j) M[c][j] = M[c][j] / piv;
    for (int r = 0; r < P; ++r)
      if (r != c) {
        zd f = M[r][c];
        for (int j = 0; j < 2 * P; ++j) M[r][j] -= f * M[c][j];
      }
  }
  zd SI[kMaxPorts][kMaxPorts];
  for (int i = 0; i < P; ++i)
    for (int j = 0; j < P; ++j) SI[i][j] = M[j][P + i];
  // reference impedances: reciprocity between groups + scalar-potential level
  double z[kMaxPorts];
  const int G = a.ngroup;
  if (G == 1) {
    for (int p = 0; p < P; ++p) z[p] = a.zline[p].re;
  } else {
    // weighted least squares on log z per group, normal equations
    double NtN[kMaxPorts][kMaxPorts] = {}, Ntb[kMaxPorts] = {};
    auto add_row = [&](const double* r, double rhs, double w) {
      for (int i = 0; i < G; ++i) {
        Ntb[i] += w * r[i] * rhs;
        for (int j = 0; j < G; ++j) NtN[i][j] += w * r[i] * r[j];
      }
    };
    for (int i = 0; i < P; ++i)
      for (int j = i + 1; j < P; ++j) {
        int gi = a.group_of[i], gj = a.group_of[j];
        if (gi == gj) continue;
        double w = fmin(cabs(SI[i][j]), cabs(SI[j][i]));
        w *= w;
        if (w > 0) {
          double r[kMaxPorts] = {};
          r[gi] = 1;
          r[gj] = -1;
          add_row(r, log(cabs(SI[j][i] / SI[i][j])), w);
        }
      }
    double meanlog_all = 0;
    for (int k = 0; k < G; ++k) {
      double s = 0;
      int c = 0;
      for (int p = 0; p < P; ++p)
        if (a.group_of[p] == k) { s += a.zline[p].re; ++c; }
      double r[kMaxPorts] = {};
      r[k] = 1;
      add_row(r, log(s / c), 1e-4);
    }
    for (int p = 0; p < P; ++p) meanlog_all += log(a.zline[p].re);
    meanlog_all /= P;
    // solve NtN x = Ntb (symmetric positive definite, Gaussian elimination)
    double x[kMaxPorts];
    for (int c = 0; c < G; ++c)
      for (int r = c + 1; r < G; ++r) {
        double f = NtN[r][c] / NtN[c][c];
        for (int j = c; j < G; ++j) NtN[r][j] -= f * NtN[c][j];
        Ntb[r] -= f * Ntb[c];
      }
    for (int c = G - 1; c >= 0; --c) {
      double s = Ntb[c];
      for (int j = c + 1; j < G; ++j) s -= NtN[c][j] * x[j];
      x[c] = s / NtN[c][c];
    }
    double meang = 0;
    for (int p = 0; p < P; ++p) meang += x[a.group_of[p]];
    meang /= P;
    for (int p = 0; p < P; ++p) z[p] = exp(x[a.group_of[p]] + meanlog_all - meang);
  }
  for (int i = 0; i < P; ++i) {
    a.z0[i] = z[i];
    for (int j = 0; j < P; ++j) a.S[i * P + j] = SI[i][j] * (sqrt(z[i]) / sqrt(z[j]));
  }
}

}  // namespace m25

using namespace m25;

struct m25_ports {
  m25_ctx* ctx = nullptr;
  int P = 0, ngroup = 0, nvpt_tot = 0, ncut = 0, lossless = 0;
  int E = 0;  // excitation columns of the solutions de-embedded (P, or P + internal ports)
  double v_weight = 1.0;
  std::vector<int> group_of, ns, s_off, port_level, nvpt;
  std::vector<double> beta0;
  std::vector<double> bounds;    // (ngroup, 2) lossless beta search intervals
  std::vector<int> fit_iters;    // (ngroup) of the last de-embedding
  double* s = nullptr;
  int32_t* cut_off = nullptr;
  int32_t* cut_edge = nullptr;
  double* cut_w = nullptr;
  double* vpts = nullptr;
  int32_t* vpt_level = nullptr;
  // per-call buffers
  zd *q = nullptr, *phi = nullptr, *I = nullptr, *V = nullptr, *x = nullptr, *out = nullptr;
  zd* Bexc = nullptr;  // (n, P) excitation columns
  int* iters = nullptr;
  int nt = 0, n = 0;
  std::vector<zd> waves;  // (P, E) incident current-wave amplitudes A of the last de-embedding
  std::vector<zd> bcoef;  // (P, E) their B (outgoing) amplitudes
  std::vector<void*> allocs;
};

extern "C" int m25_ports_create(m25_ctx* ctx, m25_geom* geom, const m25_port_desc* d, m25_ports** out) {
  if (!ctx || !geom || !d || !out) {
    set_error("m25_ports_create: null argument");
    return M25_ERR_VALUE;
  }
  if (d->nport < 1 || d->nport > kMaxPorts || d->ngroup < 1 || d->ngroup > d->nport) {
    set_error("m25_ports_create: 1..8 ports, 1..nport groups");
    return M25_ERR_VALUE;
  }
  if (d->lossless) {
    if (!d->bounds) {
      set_error("m25_ports_create: a lossless stack needs the beta search bounds of every group");
      return M25_ERR_VALUE;
    }
    for (int gi = 0; gi < d->ngroup; ++gi)
      if (!(d->bounds[2 * gi] > 0.0 && d->bounds[2 * gi + 1] > d->bounds[2 * gi])) {
        set_error("m25_ports_create: beta search bounds must satisfy 0 < lo < hi");
        return M25_ERR_VALUE;
      }
  }
  m25_ports* p = new m25_ports();
  p->E = d->nport;
  p->lossless = d->lossless ? 1 : 0;
  if (p->lossless) p->bounds.assign(d->bounds, d->bounds + 2 * d->ngroup);
  p->ctx = ctx;
  p->P = d->nport;
  p->ngroup = d->ngroup;
  p->v_weight = d->v_weight;
  p->nt = geom->nt;
  p->n = geom->nb + geom->nv;
  int tot_s = 0, tot_v = 0;
  for (int i = 0; i < p->P; ++i) {
    if (d->group_of[i] < 0 || d->group_of[i] >= d->ngroup || d->ns[i] < 2 || d->ns[i] > kMaxSamples ||
        d->nvpt[i] != 8 * d->ns[i] || d->port_level[i] < 0 || d->port_level[i] >= geom->nlev) {
      set_error("m25_ports_create: bad port description (2..64 cuts, 8 voltage points per cut)");
      delete p;
      return M25_ERR_VALUE;
    }
    int members = 0;
    for (int j = 0; j < d->nport; ++j) members += d->group_of[j] == d->group_of[i];
    if (members * d->nport > kMaxDatasets) {
      set_error("m25_ports_create: more than 16 (port, excitation) datasets in one port group");
      delete p;
      return M25_ERR_VALUE;
    }
    p->group_of.push_back(d->group_of[i]);
    p->ns.push_back(d->ns[i]);
    p->s_off.push_back(tot_s);
    p->port_level.push_back(d->port_level[i]);
    p->nvpt.push_back(d->nvpt[i]);
    tot_s += d->ns[i];
    tot_v += d->nvpt[i];
  }
  for (int gi = 0; gi < d->ngroup; ++gi) p->beta0.push_back(d->beta0 ? d->beta0[gi] : 0.0);
  p->ncut = tot_s;
  p->nvpt_tot = tot_v;
  int nent = d->cut_off[tot_s];
  for (int i = 0; i < nent; ++i)
    if (d->cut_edge[i] < 0 || d->cut_edge[i] >= p->n) {
      set_error("m25_ports_create: cut edge out of range");
      delete p;
      return M25_ERR_VALUE;
    }
  std::vector<int32_t> vlev(tot_v);
  {
    int o = 0;
    for (int i = 0; i < p->P; ++i)
      for (int k = 0; k < d->nvpt[i]; ++k) vlev[o++] = d->port_level[i];
  }
  cudaStream_t st = ctx->stream;
  int rc = M25_OK;
#define TRY(x)         \
  do {                 \
    rc = (x);          \
    if (rc) goto fail; \
  } while (0)
  TRY(alloc(p->allocs, (void**)&p->s, sizeof(double) * tot_s));
  TRY(alloc(p->allocs, (void**)&p->cut_off, sizeof(int32_t) * (tot_s + 1)));
  TRY(alloc(p->allocs, (void**)&p->cut_edge, sizeof(int32_t) * std::max(nent, 1)));
  TRY(alloc(p->allocs, (void**)&p->cut_w, sizeof(double) * std::max(nent, 1)));
  TRY(alloc(p->allocs, (void**)&p->vpts, sizeof(double) * 2 * tot_v));
  TRY(alloc(p->allocs, (void**)&p->vpt_level, sizeof(int32_t) * tot_v));
  // per-call buffers for up to kMaxPorts excitation columns (m25_ports_set_excitations)
  TRY(alloc(p->allocs, (void**)&p->q, sizeof(zd) * (size_t)geom->nt * kMaxPorts));
  TRY(alloc(p->allocs, (void**)&p->phi, sizeof(zd) * (size_t)tot_v * kMaxPorts));
  TRY(alloc(p->allocs, (void**)&p->I, sizeof(zd) * (size_t)tot_s * kMaxPorts));
  TRY(alloc(p->allocs, (void**)&p->V, sizeof(zd) * (size_t)tot_s * kMaxPorts));
  TRY(alloc(p->allocs, (void**)&p->x, sizeof(zd) * (size_t)p->n * kMaxPorts));
  TRY(alloc(p->allocs, (void**)&p->out, sizeof(zd) * (size_t)(4 * kMaxPorts * kMaxPorts + 8 * kMaxPorts)));
  TRY(alloc(p->allocs, (void**)&p->iters, sizeof(int) * kMaxPorts));
  TRY(alloc(p->allocs, (void**)&p->Bexc, sizeof(zd) * (size_t)p->n * p->P));
  if (d->excitation) {
    std::vector<zd> hb((size_t)p->n * p->P);
    for (int i = 0; i < p->n; ++i)
      for (int e = 0; e < p->P; ++e) hb[(size_t)i * p->P + e] = zd(d->excitation[(size_t)e * p->n + i], 0.0);
    M25_CUDA(cudaMemcpy(p->Bexc, hb.data(), sizeof(zd) * hb.size(), cudaMemcpyHostToDevice));
  } else {
    M25_CUDA(cudaMemset(p->Bexc, 0, sizeof(zd) * (size_t)p->n * p->P));
  }
  M25_CUDA(cudaMemcpyAsync(p->s, d->s, sizeof(double) * tot_s, cudaMemcpyHostToDevice, st));
  M25_CUDA(cudaMemcpyAsync(p->cut_off, d->cut_off, sizeof(int32_t) * (tot_s + 1), cudaMemcpyHostToDevice, st));
  M25_CUDA(cudaMemcpyAsync(p->cut_edge, d->cut_edge, sizeof(int32_t) * nent, cudaMemcpyHostToDevice, st));
  M25_CUDA(cudaMemcpyAsync(p->cut_w, d->cut_w, sizeof(double) * nent, cudaMemcpyHostToDevice, st));
  M25_CUDA(cudaMemcpyAsync(p->vpts, d->vpts, sizeof(double) * 2 * tot_v, cudaMemcpyHostToDevice, st));
  M25_CUDA(cudaMemcpyAsync(p->vpt_level, vlev.data(), sizeof(int32_t) * tot_v, cudaMemcpyHostToDevice, st));
  M25_CUDA(cudaStreamSynchronize(st));
  *out = p;
  return M25_OK;
fail:
  free_all(p->allocs);
  delete p;
  return rc;
#undef TRY
}

extern "C" int m25_ports_destroy(m25_ports* p) {
  if (!p) return M25_OK;
  cudaStreamSynchronize(p->ctx->stream);
  free_all(p->allocs);
  delete p;
  return M25_OK;
}

static int deembed(m25_ctx* ctx, m25_geom* geom, m25_greens* gr, m25_ports* p, const void* x, int where,
                   const double* beta0, double* S, double* z0, double* gamma, double* z0_line, double* resid,
                   bool mixed);
namespace m25 {
int fill_solve_mixed(m25_ctx* ctx, m25_geom* geom, m25_greens* gr, zd zs, zd zsv, int nrhs, const zd* B, zd* X,
                     double tol, int max_iter, int32_t* info);  // api.cu
}

extern "C" int m25_deembed(m25_ctx* ctx, m25_geom* geom, m25_greens* gr, m25_ports* p, const void* x, int where,
                           const double* beta0, double* S, double* z0, double* gamma, double* z0_line, double* resid) {
  return deembed(ctx, geom, gr, p, x, where, beta0, S, z0, gamma, z0_line, resid, false);
}

static int deembed(m25_ctx* ctx, m25_geom* geom, m25_greens* gr, m25_ports* p, const void* x, int where,
                   const double* beta0, double* S, double* z0, double* gamma, double* z0_line, double* resid,
                   bool mixed) {
  if (!ctx || !geom || !gr || !p || !x) {
    set_error("m25_deembed: null argument");
    return M25_ERR_VALUE;
  }
  if (gr->nlev != geom->nlev) {
    set_error("m25_deembed: Green's tables and mesh have different level counts");
    return M25_ERR_VALUE;
  }
  cudaStream_t st = ctx->stream;
  const int P = p->E, L = geom->nlev;  // P: columns of x (feeds, then internal ports)
  const zd* xd = static_cast<const zd*>(x);
  if (where == M25_ON_HOST) {
    M25_CUDA(cudaMemcpyAsync(p->x, x, sizeof(zd) * (size_t)p->n * P, cudaMemcpyHostToDevice, st));
    xd = p->x;
  }
  StageTimer tm(ctx, ST_DEEMBED);
  charges_kernel<<<(geom->nt + 127) / 128, 128, 0, st>>>(geom->nt, geom->nb, P, geom->td64, geom->tri_basis, xd,
                                                         gr->omega, p->q);
  if (geom->nv)
    via_charges_kernel<<<(geom->nv + 63) / 64, 64, 0, st>>>(geom->nv, geom->nb, P, geom->seg_pad_off, geom->seg_pad,
                                                            geom->seg_pad_w, geom->pad_tris, xd, gr->omega, p->q);
  // W leading coefficients per pair
  zd* cW = reinterpret_cast<zd*>(p->out) + 4 * kMaxPorts * kMaxPorts;
  {
    std::vector<zd> hc(L * L);
    for (int i = 0; i < L * L; ++i) hc[i] = gr->lead_h[2 * L * L + i];
    M25_CUDA(cudaMemcpyAsync(cW, hc.data(), sizeof(zd) * L * L, cudaMemcpyHostToDevice, st));
  }
  if (mixed) {
    const size_t smem = lv_mixed_smem(L, gr->nrho);
    if (smem > 200 * 1024) {
      set_error("m25_sweep_point: Green's tables too large for shared memory");
      return M25_ERR_VALUE;
    }
    // a fixed limit: the tables' size changes with the frequency (other threads)
    M25_CUDA(cudaFuncSetAttribute(line_voltage_mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    line_voltage_mixed_kernel<<<p->nvpt_tot, 256, smem, st>>>(
        geom->nt, P, L, p->vpts, p->vpt_level, geom->cen, geom->td64, geom->td32, geom->tri_layer, geom->level_z,
        gr->nrho, gr->rho, gr->rho32, reinterpret_cast<const zd*>(gr->coef), reinterpret_cast<const zf*>(gr->coef32),
        cW, p->q, p->phi);
  } else {
    line_voltage_kernel<<<p->nvpt_tot, 256, 0, st>>>(geom->nt, P, L, p->vpts, p->vpt_level, geom->cen, geom->td64,
                                                     geom->tri_layer, geom->level_z, gr->nrho, gr->rho,
                                                     reinterpret_cast<const zd*>(gr->coef), cW, p->q, p->phi);
  }
  cuts_kernel<<<(p->ncut * P + 127) / 128, 128, 0, st>>>(p->ncut, P, p->cut_off, p->cut_edge, p->cut_w, xd, p->phi, 8,
                                                         p->I, p->V);
  FitArgs fa;
  fa.P = p->P;
  fa.E = P;
  fa.ngroup = p->ngroup;
  for (int i = 0; i < p->P; ++i) {
    fa.group_of[i] = p->group_of[i];
    fa.ns[i] = p->ns[i];
    fa.s_off[i] = p->s_off[i];
  }
  for (int gi = 0; gi < p->ngroup; ++gi) fa.beta0[gi] = beta0 ? beta0[gi] : p->beta0[gi];
  fa.v_weight = p->v_weight;
  fa.s = p->s;
  fa.I = p->I;
  fa.V = p->V;
  zd* o = reinterpret_cast<zd*>(p->out);
  fa.A = o;
  fa.B = o + kMaxPorts * kMaxPorts;
  fa.S = o + 2 * kMaxPorts * kMaxPorts;
  fa.gamma = o + 3 * kMaxPorts * kMaxPorts;
  fa.zline = fa.gamma + kMaxPorts;
  fa.resid = reinterpret_cast<double*>(fa.zline + kMaxPorts);
  fa.z0 = fa.resid + kMaxPorts;
  fa.iters = p->iters;
  fa.lossless = p->lossless;
  for (int gi = 0; gi < p->ngroup; ++gi) {
    fa.lo[gi] = p->lossless ? p->bounds[2 * gi] : 0.0;
    fa.hi[gi] = p->lossless ? p->bounds[2 * gi + 1] : 0.0;
  }
  fit_kernel<<<p->ngroup, 32 * kFitWarps, 0, st>>>(fa);
  // S of the feeds alone; with internal ports the caller assembles S from
  // the coefficients (m25_deembed_coefs)
  if (p->E == p->P) fit_finish_kernel<<<1, 32, 0, st>>>(fa);
  M25_CHECK_LAUNCH();
  std::vector<zd> h(4 * kMaxPorts * kMaxPorts);
  M25_CUDA(cudaMemcpyAsync(h.data(), p->out, sizeof(zd) * h.size(), cudaMemcpyDeviceToHost, st));
  p->fit_iters.assign(p->ngroup, 0);
  M25_CUDA(cudaMemcpyAsync(p->fit_iters.data(), p->iters, sizeof(int) * p->ngroup, cudaMemcpyDeviceToHost, st));
  M25_CUDA(cudaStreamSynchronize(st));
  const zd* hS = h.data() + 2 * kMaxPorts * kMaxPorts;
  const zd* hg = h.data() + 3 * kMaxPorts * kMaxPorts;
  const zd* hz = hg + kMaxPorts;
  const double* hr = reinterpret_cast<const double*>(hz + kMaxPorts);
  const double* hz0 = hr + kMaxPorts;
  p->waves.assign(h.begin(), h.begin() + (size_t)p->P * P);  // A[port][excitation]
  p->bcoef.assign(h.begin() + kMaxPorts * kMaxPorts, h.begin() + kMaxPorts * kMaxPorts + (size_t)p->P * P);
  for (int i = 0; i < p->P; ++i) {
    for (int j = 0; j < p->P; ++j) {
      if (S && p->E == p->P) {
        S[2 * (i * P + j)] = hS[i * P + j].re;
        S[2 * (i * P + j) + 1] = hS[i * P + j].im;
      }
    }
    if (gamma) { gamma[2 * i] = hg[i].re; gamma[2 * i + 1] = hg[i].im; }
    if (z0_line) { z0_line[2 * i] = hz[i].re; z0_line[2 * i + 1] = hz[i].im; }
    if (resid) resid[i] = hr[i];
    if (z0) z0[i] = hz0[i];
  }
  return M25_OK;
}

extern "C" int m25_deembed_fit_info(m25_ports* p, int32_t* iters) {
  if (!p || !iters) {
    set_error("m25_deembed_fit_info: null argument");
    return M25_ERR_VALUE;
  }
  if (p->fit_iters.size() != (size_t)p->ngroup) {
    set_error("m25_deembed_fit_info: no de-embedding yet");
    return M25_ERR_VALUE;
  }
  for (int gi = 0; gi < p->ngroup; ++gi) iters[gi] = p->fit_iters[gi];
  return M25_OK;
}

extern "C" int m25_ports_set_excitations(m25_ports* p, int32_t nexc) {
  if (!p || nexc < p->P || nexc > kMaxPorts) {
    set_error("m25_ports_set_excitations: null ports or excitations outside nport..8");
    return M25_ERR_VALUE;
  }
  for (int gi = 0; gi < p->ngroup; ++gi) {
    int members = 0;
    for (int i = 0; i < p->P; ++i) members += p->group_of[i] == gi;
    if (members * nexc > kMaxDatasets) {
      set_error("m25_ports_set_excitations: more than 16 (port, excitation) datasets in one port group");
      return M25_ERR_VALUE;
    }
  }
  p->E = nexc;
  p->waves.clear();
  p->bcoef.clear();
  return M25_OK;
}

extern "C" int m25_deembed_coefs(m25_ports* p, double* A, double* B) {
  if (!p || !A || !B) {
    set_error("m25_deembed_coefs: null argument");
    return M25_ERR_VALUE;
  }
  if (p->waves.size() != (size_t)p->P * p->E || p->bcoef.size() != p->waves.size()) {
    set_error("m25_deembed_coefs: no de-embedding yet");
    return M25_ERR_VALUE;
  }
  for (size_t k = 0; k < p->waves.size(); ++k) {
    A[2 * k] = p->waves[k].re;
    A[2 * k + 1] = p->waves[k].im;
    B[2 * k] = p->bcoef[k].re;
    B[2 * k + 1] = p->bcoef[k].im;
  }
  return M25_OK;
}

extern "C" int m25_deembed_waves(m25_ports* p, double* A) {
  if (!p || !A) {
    set_error("m25_deembed_waves: null argument");
    return M25_ERR_VALUE;
  }
  if (p->waves.size() != (size_t)p->P * p->E) {
    set_error("m25_deembed_waves: no de-embedding yet");
    return M25_ERR_VALUE;
  }
  for (size_t k = 0; k < p->waves.size(); ++k) {
    A[2 * k] = p->waves[k].re;
    A[2 * k + 1] = p->waves[k].im;
  }
  return M25_OK;
}

extern "C" int m25_deembed_debug(m25_ctx* ctx, m25_ports* p, double* phi, double* q, double* I, double* V) {
  if (!ctx || !p) {
    set_error("m25_deembed_debug: null argument");
    return M25_ERR_VALUE;
  }
  M25_CUDA(cudaStreamSynchronize(ctx->stream));
  if (phi) M25_CUDA(cudaMemcpy(phi, p->phi, sizeof(zd) * (size_t)p->nvpt_tot * p->E, cudaMemcpyDeviceToHost));
  if (q) M25_CUDA(cudaMemcpy(q, p->q, sizeof(zd) * (size_t)p->nt * p->E, cudaMemcpyDeviceToHost));
  if (I) M25_CUDA(cudaMemcpy(I, p->I, sizeof(zd) * (size_t)p->ncut * p->E, cudaMemcpyDeviceToHost));
  if (V) M25_CUDA(cudaMemcpy(V, p->V, sizeof(zd) * (size_t)p->ncut * p->E, cudaMemcpyDeviceToHost));
  return M25_OK;
}

extern "C" int m25_sweep_point(m25_ctx* ctx, m25_geom* geom, m25_greens* gr, m25_ports* p, double zs_re, double zs_im,
                               double zsv_re, double zsv_im, int precision, const double* beta0, double tol,
                               int32_t max_iter, double* x_out, double* S, double* z0, double* gamma, double* z0_line,
                               double* resid, int32_t* info) {
  if (!ctx || !geom || !gr || !p) {
    set_error("m25_sweep_point: null argument");
    return M25_ERR_VALUE;
  }
  if (precision != M25_FP64 && precision != M25_MIXED && precision != M25_MIXED_FILL32) {
    set_error("m25_sweep_point: unknown precision");
    return M25_ERR_VALUE;
  }
  if (p->E != p->P) {
    set_error("m25_sweep_point: ports with internal-port excitations are de-embedded by m25_deembed");
    return M25_ERR_VALUE;
  }
  const int n = geom->nb + geom->nv, P = p->P;
  const size_t esz = precision == M25_MIXED_FILL32 ? sizeof(zf) : sizeof(zd);
  int rc;
  if (!(precision == M25_MIXED && geom->nv == 0) && (rc = ctx->Zsweep.ensure(esz * (size_t)n * n))) return rc;
  if ((rc = ctx->Xsweep.ensure(sizeof(zd) * (size_t)n * P))) return rc;
  int32_t inf[2] = {0, 0};
  if (precision == M25_MIXED && geom->nv == 0) {
    // fill straight into the solve's double-float planes (no complex128 Z)
    rc = fill_solve_mixed(ctx, geom, gr, zd(zs_re, zs_im), zd(zsv_re, zsv_im), P, p->Bexc, ctx->Xsweep.as<zd>(), tol,
                          max_iter, inf);
  } else {
    if ((rc = m25_assemble(ctx, geom, gr, zs_re, zs_im, zsv_re, zsv_im, precision, ctx->Zsweep.p, n, M25_ON_DEVICE)))
      return rc;
    rc = m25_dense_solve(ctx, n, P, precision, ctx->Zsweep.p, p->Bexc, ctx->Xsweep.p, M25_ON_DEVICE, tol, max_iter,
                         inf);
  }
  int used = precision;
  if (rc == M25_ERR_NUMERIC && precision != M25_FP64) {
    // the refinement with the complex64 LU did not reach the target (or that
    // LU met a zero pivot): this point goes through the fp64 path
    // (refinement steps reported as -1). The complex64 planes and LU go
    // first, so the point's peak memory stays that of the mixed path.
    M25_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->Zsplit.release();
    ctx->Zlu.release();
    if ((rc = ctx->Zsweep.ensure(sizeof(zd) * (size_t)n * n))) return rc;
    if ((rc = m25_assemble(ctx, geom, gr, zs_re, zs_im, zsv_re, zsv_im, M25_FP64, ctx->Zsweep.p, n, M25_ON_DEVICE)))
      return rc;
    inf[0] = inf[1] = 0;
    if ((rc = m25_dense_solve(ctx, n, P, M25_FP64, ctx->Zsweep.p, p->Bexc, ctx->Xsweep.p, M25_ON_DEVICE, tol,
                              max_iter, inf)))
      return rc;
    inf[0] = -1;
    used = M25_FP64;
    M25_CUDA(cudaStreamSynchronize(ctx->stream));
    if (geom->nv == 0) ctx->Zsweep.release();
  }
  if (rc) return rc;
  if (info) {
    info[0] = inf[0];
    info[1] = inf[1];
  }
  if ((rc = deembed(ctx, geom, gr, p, ctx->Xsweep.p, M25_ON_DEVICE, beta0, S, z0, gamma, z0_line, resid,
                    used != M25_FP64)))
    return rc;
  if (x_out) {
    M25_CUDA(cudaMemcpy(x_out, ctx->Xsweep.p, sizeof(zd) * (size_t)n * P, cudaMemcpyDeviceToHost));
  }
  return M25_OK;
}

extern "C" int m25_interp_point(m25_ctx* ctx, m25_geom* geom, m25_greens* gr, m25_ports* p, m25_interp* ip,
                                int32_t nuse, const int32_t* slots, const double* L, double ke, int precision,
                                const double* beta0, double tol, int32_t max_iter, double* x_out, double* S,
                                double* z0, double* gamma, double* z0_line, double* resid, int32_t* info) {
  if (p && p->E != p->P) {
    set_error("m25_interp_point: ports with internal-port excitations are de-embedded by m25_deembed");
    return M25_ERR_VALUE;
  }
  if (!ctx || !geom || !gr || !p || !ip || ip->ctx->device != ctx->device || ip->n != geom->nb + geom->nv) {
    set_error("m25_interp_point: bad argument");
    return M25_ERR_VALUE;
  }
  if (precision != M25_FP64 && precision != M25_MIXED) {
    set_error("m25_interp_point: precision must be M25_FP64 or M25_MIXED");
    return M25_ERR_VALUE;
  }
  const int n = ip->n, P = p->P;
  int rc;
  if ((rc = ctx->Zsweep.ensure(sizeof(zd) * (size_t)n * n))) return rc;
  if ((rc = ctx->Xsweep.ensure(sizeof(zd) * (size_t)n * P))) return rc;
  zd* Z = ctx->Zsweep.as<zd>();
  if ((rc = interp_eval_device(ctx, ip, nuse, slots, L, gr->freq, ke, Z, n))) return rc;
  int32_t inf[2] = {0, 0};
  rc = m25_dense_solve(ctx, n, P, precision, Z, p->Bexc, ctx->Xsweep.p, M25_ON_DEVICE, tol, max_iter, inf);
  int used = precision;
  if (rc == M25_ERR_NUMERIC && precision != M25_FP64) {
    // the mixed refinement stopped above tol: the same interpolated Z in fp64
    // (the solve factored a complex64 copy; Z itself is unchanged)
    inf[0] = inf[1] = 0;
    if ((rc = m25_dense_solve(ctx, n, P, M25_FP64, Z, p->Bexc, ctx->Xsweep.p, M25_ON_DEVICE, tol, max_iter, inf)))
      return rc;
    inf[0] = -1;
    used = M25_FP64;
  }
  if (rc) return rc;
  if (info) {
    info[0] = inf[0];
    info[1] = inf[1];
  }
  if ((rc = deembed(ctx, geom, gr, p, ctx->Xsweep.p, M25_ON_DEVICE, beta0, S, z0, gamma, z0_line, resid,
                    used != M25_FP64)))
    return rc;
  if (x_out) M25_CUDA(cudaMemcpy(x_out, ctx->Xsweep.p, sizeof(zd) * (size_t)n * P, cudaMemcpyDeviceToHost));
  return M25_OK;
}
