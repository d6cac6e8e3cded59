// Tabulated spatial Green's functions at one frequency, computed on the
// device: the remainder of the spectral MPIE kernels after removing the
// leading c e^{-jkR}/(4 pi R) terms, integrated along a lifted Sommerfeld
// path, tabulated on a rho grid and fitted with not-a-knot cubic splines.
// Follows Engine/mom25d/greens.py:111-212 (one grounded slab) and
// Engine/mom25d/layered.py:238-405 (open multilayer stack, Michalski-Zheng
// transmission-line form).
#include <algorithm>
#include <cstring>
#include <vector>

#include "m25_internal.h"

namespace m25 {

constexpr int kMaxLayers = 8;

struct StackDev {
  int nlayer, nlev, single;
  double t[kMaxLayers];
  zd epsc[kMaxLayers], kk[kMaxLayers];
  int il[kMaxLev];
  double zl[kMaxLev];
  double k0, h;
  int top_pec;                     // a PEC cover on the top layer (layered.py:257-275)
  zd lead_c[3][kMaxLev][kMaxLev];  // c_A, c_V, c_W per (observer, source)
  zd kx[2][kMaxLev][kMaxLev];      // k of the A and the V/W leading terms
  double dz[kMaxLev][kMaxLev];
};

// One-slab spectral kernels gA~, gV~, gW~ (greens.py:234-252).
__device__ void slab_spectral(const StackDev& S, zd kr, zd& gA, zd& gV, zd& gW) {
  const double h = S.t[0];
  zd kr2 = kr * kr;
  zd u0 = csqrt(kr2 - zd(S.k0 * S.k0));
  zd u1 = csqrt(kr2 - S.kk[0] * S.kk[0]);
  zd x = u1 * h;
  zd e = cexp(x * -2.0);
  zd u1coth, u1tanh, tanh_over_u1;
  if (cabs(x) < 1e-4) {
    u1coth = zd(1.0 / h) + (u1 * u1) * (h / 3.0);
    u1tanh = (u1 * u1) * h;
    tanh_over_u1 = zd(h);
  } else {
    u1coth = u1 * (zd(1.0) + e) / (zd(1.0) - e);
    u1tanh = u1 * (zd(1.0) - e) / (zd(1.0) + e);
    tanh_over_u1 = u1tanh / (u1 * u1);
  }
  zd dte = u0 + u1coth;
  zd dtm = S.epsc[0] * u0 + u1tanh;
  gA = zd(1.0) / dte;
  gV = (u0 + u1tanh) / (dte * dtm);
  gW = u0 * tanh_over_u1 / dtm;
}

// Multilayer spectral kernels via TE/TM line voltages (layered.py:238-289):
// g[m][i][j], m = A, V, W; i observer level, j source level.
__device__ void layered_spectral(const StackDev& S, zd kr, zd g[3][kMaxLev][kMaxLev]) {
  const int N = S.nlayer, L = S.nlev;
  zd u[kMaxLayers], T[kMaxLayers], Sh[kMaxLayers];
  zd kr2 = kr * kr;
  for (int n = 0; n < N; ++n) {
    u[n] = csqrt(kr2 - S.kk[n] * S.kk[n]);
    zd x = u[n] * S.t[n];
    zd e = cexp(x * -2.0);
    T[n] = (zd(1.0) - e) / (zd(1.0) + e);
    Sh[n] = (cexp(-x) * 2.0) / (zd(1.0) + e);
  }
  zd u0 = csqrt(kr2 - zd(S.k0 * S.k0));
  zd Vmode[2][kMaxLev][kMaxLayers + 1];
  for (int mode = 0; mode < 2; ++mode) {
    zd y[kMaxLayers];
    for (int n = 0; n < N; ++n) y[n] = mode == 0 ? u[n] : S.epsc[n] / u[n];
    zd yair = mode == 0 ? u0 : zd(1.0) / u0;
    zd ydn[kMaxLayers + 1], yup[kMaxLayers + 1];
    ydn[1] = y[0] / T[0];
    for (int k = 2; k <= N; ++k) {
      zd yl = ydn[k - 1], yk = y[k - 1], tk = T[k - 1];
      ydn[k] = yk * (yl + yk * tk) / (yk + yl * tk);
    }
    yup[N] = S.top_pec ? zd(0.0) : yair;  // (unused under a cover: no level on it)
    for (int k = N - 1; k >= 1; --k) {
      zd yk = y[k], tk = T[k];
      if (S.top_pec && k == N - 1) {
        yup[k] = yk / tk;  // layer N shorted by the cover
      } else {
        zd yl = yup[k + 1];
        yup[k] = yk * (yl + yk * tk) / (yk + yl * tk);
      }
    }
    for (int l = 0; l < L; ++l) {
      zd* V = Vmode[mode][l];
      for (int k = 0; k <= N; ++k) V[k] = zd(0.0);
      int s = S.il[l];
      V[s] = zd(1.0) / (ydn[s] + yup[s]);
      for (int k = s; k >= 2; --k) V[k - 1] = V[k] * Sh[k - 1] / (zd(1.0) + ydn[k - 1] / y[k - 1] * T[k - 1]);
      for (int k = s; k < N; ++k) {
        if (S.top_pec && k + 1 == N) break;  // V_N = 0 on the cover
        V[k + 1] = V[k] * Sh[k] / (zd(1.0) + yup[k + 1] / y[k] * T[k]);
      }
    }
  }
  const double k02 = S.k0 * S.k0;
  for (int i = 0; i < L; ++i) {
    const int ii = S.il[i];
    for (int j = 0; j < L; ++j) {
      const zd* Vh = Vmode[0][j];
      const zd* Ve = Vmode[1][j];
      g[0][i][j] = Vh[ii];
      g[1][i][j] = (Ve[ii] + Vh[ii] * k02) / kr2;
      zd cum(0.0);
      for (int n = 0; n < ii; ++n) cum += (Ve[n + 1] - Ve[n]) / (u[n] * u[n]);
      g[2][i][j] = cum;
    }
  }
}

// Leading-term coefficients (greens.py:215-224, layered.py:292-331); gbig:
// the layered spectral kernels at kbig (spectral_g_kernel's last node).
__global__ void leading_kernel(StackDev* S, double kbig, const zd* __restrict__ gbig) {
  if (threadIdx.x || blockIdx.x) return;
  StackDev& s = *S;
  const int L = s.nlev, N = s.nlayer;
  if (s.single) {
    zd k1 = s.kk[0], e = s.epsc[0];
    zd k02(s.k0 * s.k0);
    zd ka = csqrt((k02 + k1 * k1) * 0.5);
    zd cv = zd(2.0) / (e + zd(1.0));
    zd kv = csqrt((e * k02 + k1 * k1) / (e + zd(1.0)));
    s.lead_c[0][0][0] = zd(1.0);
    s.lead_c[1][0][0] = cv;
    s.lead_c[2][0][0] = cv;
    s.kx[0][0][0] = ka;
    s.kx[1][0][0] = kv;
    s.dz[0][0] = 0.0;
    return;
  }
  for (int i = 0; i < L; ++i)
    for (int j = 0; j < L; ++j) {
      s.dz[i][j] = fabs(s.zl[i] - s.zl[j]);
      if (i == j) {
        int n = s.il[i];
        zd eb = s.epsc[n - 1], kb = s.kk[n - 1], ea, ka;
        if (n == N) {
          ea = zd(1.0);
          ka = zd(s.k0);
        } else {
          ea = s.epsc[n];
          ka = s.kk[n];
        }
        zd cv = zd(2.0) / (ea + eb);
        s.lead_c[0][i][j] = zd(1.0);
        s.lead_c[1][i][j] = cv;
        s.lead_c[2][i][j] = cv;
        s.kx[0][i][j] = csqrt((ka * ka + kb * kb) * 0.5);
        s.kx[1][i][j] = csqrt((eb * (ka * ka) + ea * (kb * kb)) / (ea + eb));
        continue;
      }
      zd ux = csqrt(zd(kbig * kbig - s.k0 * s.k0));
      zd f = ux * 2.0 * cexp(ux * s.dz[i][j]);
      zd c[3];
      for (int m = 0; m < 3; ++m) c[m] = f * gbig[(m * L + i) * L + j];
      if (s.zl[j] < s.zl[i]) c[2] = zd(0.0);
      for (int m = 0; m < 3; ++m) {
        // drop the numerical noise of static coefficients' imaginary parts
        if (fabs(c[m].im) < 1e-9 * cabs(c[m])) c[m].im = 0.0;
        s.lead_c[m][i][j] = c[m];
      }
      s.kx[0][i][j] = zd(s.k0);
      s.kx[1][i][j] = zd(s.k0);
    }
}

// The spectral kernels g[(m*L + i)*L + j] at every path node, in one launch:
// nodes q < nkc of the lifted arc into gc, the next nkr of the real axis into
// gr, and (layered stacks) one more node at kbig into gbig for the leading
// terms. Each node is one thread's fp64 chain of square roots, exponentials
// and divisions through the layers; small CTAs spread the nodes over the SMs.
__global__ void __launch_bounds__(64) spectral_g_kernel(const StackDev* __restrict__ Sp, int nkc,
                                                        const double* __restrict__ kc, int nkr,
                                                        const double* __restrict__ kr, double kbig,
                                                        zd* __restrict__ gc, zd* __restrict__ gr,
                                                        zd* __restrict__ gbig) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const StackDev& S = *Sp;
  const int L = S.nlev, NC = 3 * L * L;
  zd k;
  zd* out;
  if (q < nkc) {
    k = zd(kc[2 * q], kc[2 * q + 1]);
    out = gc + (int64_t)q * NC;
  } else if (q < nkc + nkr) {
    k = zd(kr[q - nkc], 0.0);
    out = gr + (int64_t)(q - nkc) * NC;
  } else if (q == nkc + nkr && !S.single) {
    k = zd(kbig, 0.0);
    out = gbig;
  } else {
    return;
  }
  zd g[3][kMaxLev][kMaxLev];
  if (S.single) {
    slab_spectral(S, k, g[0][0][0], g[1][0][0], g[2][0][0]);
  } else {
    layered_spectral(S, k, g);
  }
  for (int m = 0; m < 3; ++m)
    for (int i = 0; i < L; ++i)
      for (int j = 0; j < L; ++j) out[(m * L + i) * L + j] = g[m][i][j];
}

// coef[q][(m*L + i)*L + j] = w k (g - leading term) / 2pi at every path node
// (in place over the spectral kernels g), one thread per (node, column).
__global__ void spectral_coef_kernel(const StackDev* __restrict__ Sp, int nkc, const double* __restrict__ kc,
                                     const double* __restrict__ wc, int nkr, const double* __restrict__ kr,
                                     const double* __restrict__ wr, zd* __restrict__ cc, zd* __restrict__ cr) {
  const StackDev& S = *Sp;
  const int L = S.nlev, NC = 3 * L * L;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)(nkc + nkr) * NC) return;
  const int q = (int)(t / NC), col = (int)(t % NC);
  const int m = col / (L * L), i = (col / L) % L, j = col % L;
  const bool cpath = q < nkc;
  const int qq = cpath ? q : q - nkc;
  const zd k = cpath ? zd(kc[2 * qq], kc[2 * qq + 1]) : zd(kr[qq], 0.0);
  const zd w = cpath ? zd(wc[2 * qq], wc[2 * qq + 1]) : zd(wr[qq], 0.0);
  zd* c = (cpath ? cc : cr) + (int64_t)qq * NC + col;
  const zd kx = S.kx[m == 0 ? 0 : 1][i][j];
  const zd ux = csqrt(k * k - kx * kx);
  const zd lead = S.lead_c[m][i][j] * cexp(ux * (-S.dz[i][j])) / (ux * 2.0);
  const zd scale = (w * k) / (2.0 * kPi);
  *c = scale * (*c - lead);
}

// J0 of a complex argument: the trapezoidal rule on Bessel's integral
// J0(z) = (1/2pi) Int_0^{2pi} cos(z sin t) dt, which converges geometrically
// for this periodic integrand (error ~ 2 J_M(z)); M is a multiple of 4 with
// M >= 1.5 |z| + 24, using the symmetry of sin t over the quarter periods.
__device__ inline zd bessel_j0_complex(zd z) {
  double az = hypot(z.re, z.im);
  int M = 4 * (int)ceil((1.5 * az + 24.0) * 0.25);
  int Q = M / 4;
  double sr = 0.0, si = 0.0;
  for (int m = 1; m < Q; ++m) {
    double s = sinpi(2.0 * m / M);
    double a = z.re * s, b = z.im * s;
    double sa, ca;
    sincos(a, &sa, &ca);
    double eb = exp(b), ebi = 1.0 / eb;
    sr += ca * 0.5 * (eb + ebi);
    si -= sa * 0.5 * (eb - ebi);
  }
  // cos z at the quarter points
  double sa, ca;
  sincos(z.re, &sa, &ca);
  double eb = exp(z.im), ebi = 1.0 / eb;
  double cr = ca * 0.5 * (eb + ebi), ci = -sa * 0.5 * (eb - ebi);
  return {(2.0 + 2.0 * cr + 4.0 * sr) / M, (2.0 * ci + 4.0 * si) / M};
}

// Path nodes per CTA of the Sommerfeld integral: each radius's sum over the
// nk_c + nk_r path nodes is split into ceil(nk / kSomNodes) fixed ranges (at
// most kSomMaxSplit), whatever the radii launched with it, so that a radius's
// value does not depend on which radii share its launch.
constexpr int kSomNodes = 1024;
constexpr int kSomMaxSplit = 32;
inline int som_split(int nk) { return std::min(kSomMaxSplit, std::max(1, (nk + kSomNodes - 1) / kSomNodes)); }

// part[s][e][c] = sum over the nodes of range s of J0(rho k) coef[k][c] at
// radius rho[idx[e]] (idx NULL: rho[e]); complex J0 on the lifted arc, real
// J0 on the real axis. Grid (ne, nsplit), one CTA per (radius, node range).
// With skip set (the learned remainder was accepted) the CTAs return at once.
template <int NC>
__global__ void sommerfeld_kernel(int ne, const int* __restrict__ idx, const double* __restrict__ rho, int nsplit,
                                  int nkc, const double* __restrict__ kc, const zd* __restrict__ coef_c, int nkr,
                                  const double* __restrict__ kr, const zd* __restrict__ coef_r, zd* __restrict__ part,
                                  const int* __restrict__ skip) {
  if (skip && *skip) return;
  const int e = blockIdx.x, s = blockIdx.y;
  const double r = rho[idx ? idx[e] : e];
  const int64_t nk = (int64_t)nkc + nkr;
  const int q0 = (int)(nk * s / nsplit), q1 = (int)(nk * (s + 1) / nsplit);
  double acc_re[NC], acc_im[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) acc_re[c] = acc_im[c] = 0.0;
  for (int q = q0 + threadIdx.x; q < min(q1, nkc); q += blockDim.x) {
    zd J = bessel_j0_complex(zd(r * kc[2 * q], r * kc[2 * q + 1]));
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      zd v = J * coef_c[(int64_t)q * NC + c];
      acc_re[c] += v.re;
      acc_im[c] += v.im;
    }
  }
  for (int q = max(q0, nkc) + threadIdx.x; q < q1; q += blockDim.x) {
    const int qr = q - nkc;
    double J = j0(r * kr[qr]);
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      zd v = coef_r[(int64_t)qr * NC + c];
      acc_re[c] += J * v.re;
      acc_im[c] += J * v.im;
    }
  }
  __shared__ double red[32][2];
  for (int c = 0; c < NC; ++c) {
    double a = acc_re[c], b = acc_im[c];
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
      part[((int64_t)s * ne + e) * NC + c] = zd(sa, sb);
    }
    __syncthreads();
  }
}

// res[idx[e]][c] = sum over the node ranges s (in order) of part[s][e][c].
__global__ void sommerfeld_sum_kernel(int ne, int NC, const int* __restrict__ idx, int nsplit,
                                      const zd* __restrict__ part, zd* __restrict__ res,
                                      const int* __restrict__ skip) {
  if (skip && *skip) return;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ne * NC) return;
  const int e = t / NC, c = t % NC;
  zd v(0.0, 0.0);
  for (int s = 0; s < nsplit; ++s) v = v + part[((int64_t)s * ne + e) * NC + c];
  res[(int64_t)(idx ? idx[e] : e) * NC + c] = v;
}

// S tables: closed-form expm1 part of the leading term, the Sommerfeld
// remainder and, for gA, the ground-plane loss kernel (greens.py:298-335,
// layered.py:391-405).  S layout (3, L, L, nrho).
__global__ void table_kernel(const StackDev* __restrict__ Sp, int nrho, const double* __restrict__ rho,
                             const zd* __restrict__ res, double omega, zd zs_ground, zd* __restrict__ Stab) {
  const StackDev& S = *Sp;
  const int L = S.nlev, NC = 3 * L * L;
  int gid = blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= NC * nrho) return;
  int c = gid / nrho, ir = gid % nrho;
  int m = c / (L * L), i = (c / L) % L, j = c % L;
  double r = rho[ir];
  double dz = S.dz[i][j];
  double R = sqrt(r * r + dz * dz);
  zd k = S.kx[m == 0 ? 0 : 1][i][j];
  zd f;
  if (R > 0) {
    f = cexpm1(zd(0.0, -1.0) * k * R) / (4.0 * kPi * R);
  } else {
    f = (zd(0.0, -1.0) * k) / (4.0 * kPi);
  }
  zd v = S.lead_c[m][i][j] * f + res[(int64_t)ir * NC + c];
  if (m == 0 && (zs_ground.re != 0.0 || zs_ground.im != 0.0)) {
    double d = S.zl[i] + S.zl[j];
    double p = d / (2.0 * kPi * pow(r * r + d * d, 1.5));
    v += zs_ground / zd(0.0, omega * kMu0) * p;
  }
  Stab[(int64_t)c * nrho + ir] = v;
}

// Not-a-knot cubic spline of every column (scipy CubicSpline's system for
// the nodal slopes, solved by forward elimination / back substitution), as
// piecewise coefficients c[interval][p] of (r - x_i)^(3-p).
// coef layout (pair, interval, power, {A, V, W}).
// One CTA per column: radii, values and the sweep's arrays in shared memory
// (the elimination is a chain of dependent steps: it runs on one thread from
// shared memory), the coefficients of the intervals in parallel.
// Tridiagonal system a_i x_{i-1} + b_i x_i + c_i x_{i+1} = d_i, i < m (a_0 =
// c_{m-1} = 0), diagonally dominant, solved by parallel cyclic reduction
// (Hockney) with every thread of the CTA: round r combines each row with the
// rows 2^r above and below, which removes their couplings; after ceil(log2 m)
// rounds every row reads b_i x_i = d_i. Shared-memory arrays of m entries:
// a, b, c, d and the copies a2, b2, c2, d2 (ping-pong); x receives the
// solution (it may be d). The caller synchronises before the call; the call
// ends with the CTA synchronised. A serial elimination would chain m
// dependent fp64 divisions; here the chain is ceil(log2 m) rounds deep.
template <class T>
__device__ void pcr_solve(int m, double* a, double* b, double* c, T* d, double* a2, double* b2, double* c2, T* d2,
                          T* x) {
  for (int st = 1; st < m; st <<= 1) {
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
      double na = 0.0, nc = 0.0, nb = b[i];
      T nd = d[i];
      if (i - st >= 0) {
        const double k1 = a[i] / b[i - st];
        na = -a[i - st] * k1;
        nb -= c[i - st] * k1;
        nd = nd - d[i - st] * k1;
      }
      if (i + st < m) {
        const double k2 = c[i] / b[i + st];
        nc = -c[i + st] * k2;
        nb -= a[i + st] * k2;
        nd = nd - d[i + st] * k2;
      }
      a2[i] = na;
      b2[i] = nb;
      c2[i] = nc;
      d2[i] = nd;
    }
    __syncthreads();
    double* t;
    t = a, a = a2, a2 = t;
    t = b, b = b2, b2 = t;
    t = c, c = c2, c2 = t;
    T* td = d;
    d = d2, d2 = td;
  }
  for (int i = threadIdx.x; i < m; i += blockDim.x) x[i] = d[i] / b[i];
  __syncthreads();
}

__host__ __device__ inline size_t spline_smem(int n) { return (size_t)n * (2 * sizeof(double) + 4 * sizeof(zd)); }
// with the reduced system solved by pcr_solve (n - 2 rows)
__host__ __device__ inline size_t spline_smem_pcr(int n) {
  return (size_t)n * (2 * sizeof(double) + 3 * sizeof(zd)) + (size_t)(n - 2) * (6 * sizeof(double) + 2 * sizeof(zd));
}

// Not-a-knot cubic spline of one table column (scipy CubicSpline's slope
// form): rows a_i s_{i-1} + b_i s_i + c_i s_{i+1} = d_i for the slopes s,
// the first and last rows the not-a-knot conditions. PCR: rows 0 and n - 1
// are eliminated into rows 1 and n - 2, which leaves a strictly diagonally
// dominant system for s_1 .. s_{n-2} (pcr_solve); else (tables too long for
// its shared memory) one thread eliminates and substitutes serially.
template <bool PCR>
__global__ void __launch_bounds__(128) spline_kernel(int L, int nrho, const double* __restrict__ xg,
                                                     const zd* __restrict__ Stab, zd* __restrict__ coef) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int col = blockIdx.x;
  const int n = nrho;
  zd* y = reinterpret_cast<zd*>(smem_raw);  // (n) values
  zd* s = y + n;                            // (n) slopes
  zd* sl = s + n;                           // (n - 1) secant slopes
  double* x = reinterpret_cast<double*>(sl + n);
  double* dx = x + n;                       // (n - 1) interval widths
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    x[i] = xg[i];
    y[i] = Stab[(int64_t)col * n + i];
  }
  __syncthreads();
  // the widths and secant slopes (independent of the recurrence), in parallel
  for (int i = threadIdx.x; i < n - 1; i += blockDim.x) {
    dx[i] = x[i + 1] - x[i];
    sl[i] = (y[i + 1] - y[i]) / dx[i];
  }
  __syncthreads();
  // row i of the slope system
  auto row = [&](int i, double& a, double& b, double& c, zd& d) {
    if (i == 0) {
      const double dx0 = dx[0], dx1 = dx[1], d0 = x[2] - x[0];
      a = 0;
      b = dx1;
      c = d0;
      d = (sl[0] * ((dx0 + 2 * d0) * dx1) + sl[1] * (dx0 * dx0)) / d0;
    } else if (i == n - 1) {
      const double dxl = dx[n - 2], dxm = dx[n - 3], d1 = x[n - 1] - x[n - 3];
      a = d1;
      b = dxm;
      c = 0;
      d = (sl[n - 3] * (dxl * dxl) + sl[n - 2] * ((2 * d1 + dxl) * dxm)) / d1;
    } else {
      a = dx[i];
      b = 2 * (dx[i - 1] + dx[i]);
      c = dx[i - 1];
      d = (sl[i - 1] * dx[i] + sl[i] * dx[i - 1]) * 3.0;
    }
  };
  if constexpr (PCR) {
    const int m = n - 2;
    double* ra = dx + n;
    double* rb = ra + m;
    double* rc = rb + m;
    double* ra2 = rc + m;
    double* rb2 = ra2 + m;
    double* rc2 = rb2 + m;
    zd* rd = reinterpret_cast<zd*>(rc2 + m);
    zd* rd2 = rd + m;
    for (int i = 1 + threadIdx.x; i <= n - 2; i += blockDim.x) {
      double a, b, c;
      zd d;
      row(i, a, b, c, d);
      if (i == 1) {  // s_0 = (d_0 - c_0 s_1) / b_0
        double a0, b0, c0;
        zd d0;
        row(0, a0, b0, c0, d0);
        b -= a * c0 / b0;
        d = d - d0 * (a / b0);
        a = 0.0;
      }
      if (i == n - 2) {  // s_{n-1} = (d_{n-1} - a_{n-1} s_{n-2}) / b_{n-1}
        double al, bl, cl;
        zd dl;
        row(n - 1, al, bl, cl, dl);
        b -= c * al / bl;
        d = d - dl * (c / bl);
        c = 0.0;
      }
      ra[i - 1] = a;
      rb[i - 1] = b;
      rc[i - 1] = c;
      rd[i - 1] = d;
    }
    __syncthreads();
    pcr_solve<zd>(m, ra, rb, rc, rd, ra2, rb2, rc2, rd2, s + 1);
    if (threadIdx.x == 0) {
      double a, b, c;
      zd d;
      row(0, a, b, c, d);
      s[0] = (d - s[1] * c) / b;
      row(n - 1, a, b, c, d);
      s[n - 1] = (d - s[n - 2] * a) / b;
    }
  } else {
    zd* cp = reinterpret_cast<zd*>(dx + n);  // (n) modified diagonal (re), upper diagonal (im)
    if (threadIdx.x == 0) {
      // forward sweep
      double bprev = 0, cprev = 0;
      for (int i = 0; i < n; ++i) {
        double a, b, c;
        zd d;
        row(i, a, b, c, d);
        if (i > 0) {
          double mlt = a / bprev;
          b -= mlt * cprev;
          d -= s[i - 1] * mlt;
        }
        s[i] = d;       // holds the modified rhs
        cp[i] = zd(b);  // modified diagonal
        bprev = b;
        cprev = c;
        if (i < n - 1) cp[i].im = c;
      }
      // back substitution
      s[n - 1] = s[n - 1] / cp[n - 1].re;
      for (int i = n - 2; i >= 0; --i) s[i] = (s[i] - s[i + 1] * cp[i].im) / cp[i].re;
    }
  }
  __syncthreads();
  const int pair = col % (L * L), m = col / (L * L);
  for (int i = threadIdx.x; i < n - 1; i += blockDim.x) {
    const double h = dx[i];
    const zd si = sl[i];
    zd t = (s[i] + s[i + 1] - si * 2.0) / h;
    zd* o = coef + (((int64_t)pair * (n - 1) + i) * 4) * 3;
    o[0 * 3 + m] = t / h;
    o[1 * 3 + m] = (si - s[i]) / h - t;
    o[2 * 3 + m] = s[i];
    o[3 * 3 + m] = y[i];
  }
}

__global__ void to_f32_kernel(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = float(a[i]);
}

// ------------------------------------------------------ learned remainder
// network inputs of n radii at frequency f
__global__ void sur_features_kernel(int n, const double* __restrict__ rho, double a, double rho_ref, double f,
                                    double fmin, double fmax, float* __restrict__ X) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  X[2 * i] = (float)(2.0 * log1p(rho[i] / a) / log1p(rho_ref / a) - 1.0);
  X[2 * i + 1] = (float)(2.0 * (f - fmin) / (fmax - fmin) - 1.0);
}

// Not-a-knot cubic spline through (x_j, y_j), j < K (K >= 4), with every
// thread of the CTA: the second derivatives M_j. The end conditions (third
// derivative continuous at x_1 and x_{K-2}) give M_0 and M_{K-1} in terms of
// their neighbours; substituted into rows 1 and K - 2 they leave a strictly
// diagonally dominant tridiagonal system for M_1 .. M_{K-2}, solved by
// pcr_solve. scratch: 8 (K - 2) doubles of shared memory. The caller
// synchronises before the call; the call ends synchronised.
template <class XF, class YF>
__device__ void spline_notaknot(int K, XF x, YF y, double* M, double* scratch) {
  const int m = K - 2;  // unknowns M_1 .. M_{K-2}
  double *a = scratch, *b = a + m, *c = b + m, *d = c + m;
  double *a2 = d + m, *b2 = a2 + m, *c2 = b2 + m, *d2 = c2 + m;
  auto h = [&](int j) { return x(j + 1) - x(j); };
  for (int k = 1 + threadIdx.x; k <= m; k += blockDim.x) {
    double ak = h(k - 1), bk = 2.0 * (h(k - 1) + h(k)), ck = h(k);
    const double dk = 6.0 * ((y(k + 1) - y(k)) / h(k) - (y(k) - y(k - 1)) / h(k - 1));
    if (k == 1) {  // M_0 = ((h_0 + h_1) M_1 - h_0 M_2) / h_1
      bk += h(0) * (h(0) + h(1)) / h(1);
      ck -= h(0) * h(0) / h(1);
      ak = 0.0;
    }
    if (k == m) {  // M_{K-1} = ((h_{K-3} + h_{K-2}) M_{K-2} - h_{K-2} M_{K-3}) / h_{K-3}
      const double p = h(K - 3), q = h(K - 2);
      ak -= q * q / p;
      bk += q * (p + q) / p;
      ck = 0.0;
    }
    a[k - 1] = ak;
    b[k - 1] = bk;
    c[k - 1] = ck;
    d[k - 1] = dk;
  }
  __syncthreads();
  pcr_solve<double>(m, a, b, c, d, a2, b2, c2, d2, M + 1);
  if (threadIdx.x == 0) {
    M[0] = ((h(0) + h(1)) * M[1] - h(0) * M[2]) / h(1);
    M[K - 1] = ((h(K - 3) + h(K - 2)) * M[K - 2] - h(K - 2) * M[K - 3]) / h(K - 3);
  }
  __syncthreads();
}

// The cubic of interval j of a spline with second derivatives M at x.
__device__ inline double spline_eval(double x0, double x1, double y0, double y1, double M0, double M1, double xv) {
  const double h = x1 - x0, t = xv - x0;
  const double b = (y1 - y0) / h - h * (2.0 * M0 + M1) / 6.0;
  return y0 + t * (b + t * (0.5 * M0 + t * (M1 - M0) / (6.0 * h)));
}

// Learned remainder. The Sommerfeld integral has been evaluated at the ne
// radii ie[] (sorted; res holds it there): the knots (every radius below the
// near limit, then every stride-th radius and the last) at positions kpos[]
// of ie, and one validation radius in the middle of each gap between knots at
// positions vpos[]. Y: the network at every table radius (2 NC scaled
// outputs, res = scale x Y).
//
// Judge, one CTA per real column (re / im of each of the NC columns): the
// residual (integral - network) at the knots is interpolated by a not-a-knot
// spline, and the network + spline compared with the integral at the
// validation radii. colerr[2 col] = the largest error there, colerr[2 col +
// 1] = the largest |remainder| of the column's complex column over the ne
// radii. Shared memory: (2 ne + 11 nk) doubles.
__global__ void __launch_bounds__(256) sur_judge_kernel(int NC, const double* __restrict__ rho, int ne,
                                                        const int* __restrict__ ie, int nk,
                                                        const int* __restrict__ kpos, int nv,
                                                        const int* __restrict__ vpos, const float* __restrict__ Y,
                                                        const double* __restrict__ scale, const zd* __restrict__ res,
                                                        double* __restrict__ colerr) {
  extern __shared__ double sm[];
  __shared__ double red_e[8], red_s[8];
  const int ncol = 2 * NC, col = blockIdx.x;
  double* xs = sm;       // radius of integrated radius e
  double* ys = xs + ne;  // residual there
  double* xk = ys + ne;
  double* yk = xk + nk;
  double* M = yk + nk;
  double* scratch = M + nk;
  double smax = 0.0;
  for (int e = threadIdx.x; e < ne; e += blockDim.x) {
    const int i = ie[e];
    const zd v = res[(int64_t)i * NC + (col >> 1)];
    xs[e] = rho[i];
    ys[e] = ((col & 1) ? v.im : v.re) - scale[col] * (double)Y[(int64_t)i * ncol + col];
    smax = fmax(smax, sqrt(v.re * v.re + v.im * v.im));
  }
  __syncthreads();
  for (int j = threadIdx.x; j < nk; j += blockDim.x) {
    xk[j] = xs[kpos[j]];
    yk[j] = ys[kpos[j]];
  }
  __syncthreads();
  spline_notaknot(
      nk, [&](int j) { return xk[j]; }, [&](int j) { return yk[j]; }, M, scratch);
  double emax = 0.0;
  for (int v = threadIdx.x; v < nv; v += blockDim.x) {
    const int e = vpos[v];
    const double xv = xs[e];
    int lo = 0, hi = nk - 1;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (xv < xk[mid]) hi = mid; else lo = mid;
    }
    emax = fmax(emax, fabs(ys[e] - spline_eval(xk[lo], xk[lo + 1], yk[lo], yk[lo + 1], M[lo], M[lo + 1], xv)));
  }
  for (int o = 16; o; o >>= 1) {
    emax = fmax(emax, __shfl_down_sync(0xffffffffu, emax, o));
    smax = fmax(smax, __shfl_down_sync(0xffffffffu, smax, o));
  }
  if ((threadIdx.x & 31) == 0) {
    red_e[threadIdx.x >> 5] = emax;
    red_s[threadIdx.x >> 5] = smax;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double e = 0, sx = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      e = fmax(e, red_e[w]);
      sx = fmax(sx, red_s[w]);
    }
    colerr[2 * col] = e;
    colerr[2 * col + 1] = sx;
  }
}

// Decision and fill-in, one CTA per real column: accepted when the largest
// column error <= tol x the largest |remainder| (every CTA reaches the same
// decision; CTA 0 records it in flag / err_out). When accepted, the table's
// other radii ir[] get network + a not-a-knot spline of the residual through
// all ne integrated radii (a denser spline than the judged one). Shared
// memory: 11 ne doubles.
__global__ void __launch_bounds__(256) sur_fill_kernel(int NC, const double* __restrict__ rho, int ne,
                                                       const int* __restrict__ ie, int nr, const int* __restrict__ ir,
                                                       const float* __restrict__ Y, const double* __restrict__ scale,
                                                       const double* __restrict__ colerr, double tol,
                                                       zd* __restrict__ res, int* __restrict__ flag,
                                                       double* __restrict__ err_out) {
  extern __shared__ double sm[];
  __shared__ int accepted;
  const int ncol = 2 * NC, col = blockIdx.x;
  if (threadIdx.x == 0) {
    double e = 0, sx = 0;
    for (int c = 0; c < ncol; ++c) {
      e = fmax(e, colerr[2 * c]);
      sx = fmax(sx, colerr[2 * c + 1]);
    }
    const double rel = sx > 0 ? e / sx : INFINITY;
    accepted = rel <= tol ? 1 : 0;
    if (blockIdx.x == 0) {
      *flag = accepted;
      *err_out = rel;
    }
  }
  __syncthreads();
  if (!accepted) return;
  double* xs = sm;
  double* ys = xs + ne;
  double* M = ys + ne;
  double* scratch = M + ne;
  for (int e = threadIdx.x; e < ne; e += blockDim.x) {
    const int i = ie[e];
    const zd v = res[(int64_t)i * NC + (col >> 1)];
    xs[e] = rho[i];
    ys[e] = ((col & 1) ? v.im : v.re) - scale[col] * (double)Y[(int64_t)i * ncol + col];
  }
  __syncthreads();
  spline_notaknot(
      ne, [&](int e) { return xs[e]; }, [&](int e) { return ys[e]; }, M, scratch);
  for (int r = threadIdx.x; r < nr; r += blockDim.x) {
    const int i = ir[r];
    const double xv = rho[i];
    int lo = 0, hi = ne - 1;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (xv < xs[mid]) hi = mid; else lo = mid;
    }
    const double v = scale[col] * (double)Y[(int64_t)i * ncol + col] +
                     spline_eval(xs[lo], xs[lo + 1], ys[lo], ys[lo + 1], M[lo], M[lo + 1], xv);
    double* out = reinterpret_cast<double*>(res + (int64_t)i * NC + (col >> 1));
    out[col & 1] = v;
  }
}

// shared memory of the two kernels above, and its limit
inline size_t sur_judge_smem(int ne, int nk) { return sizeof(double) * (2 * (size_t)ne + 11 * (size_t)nk); }
inline size_t sur_fill_smem(int ne) { return sizeof(double) * 11 * (size_t)ne; }
constexpr size_t kSurSmemMax = 200 * 1024;

int mlp_forward_device(const m25_mlp* m, int n, const float* X, float* Y, cudaStream_t st);  // mlp.cu
int mlp_dims(const m25_mlp* m, int* n_in, int* n_out);

}  // namespace m25

using namespace m25;

extern "C" int m25_greens_create(m25_ctx* ctx, const m25_greens_desc* d, m25_greens** out) {
  if (!ctx || !d || !out) {
    set_error("m25_greens_create: null argument");
    return M25_ERR_VALUE;
  }
  if (d->nlayer < 1 || d->nlayer > kMaxLayers || d->nlev < 1 || d->nlev > kMaxLev || d->nrho < 4 ||
      d->nk_c < 1 || d->nk_r < 1 || (d->single && (d->nlayer != 1 || d->nlev != 1))) {
    set_error("m25_greens_create: unsupported stack (1-8 layers, 1-3 metal levels, >= 4 radii)");
    return M25_ERR_VALUE;
  }
  for (int l = 0; l < d->nlev; ++l)
    if (d->lev_iface[l] < 1 || d->lev_iface[l] > d->nlayer || (d->top_pec && d->lev_iface[l] == d->nlayer)) {
      set_error("m25_greens_create: level interface out of range (or on the PEC cover)");
      return M25_ERR_VALUE;
    }
  if (d->top_pec && (d->single || d->nlayer < 2)) {
    set_error("m25_greens_create: a PEC cover needs a layer above the metal");
    return M25_ERR_VALUE;
  }
  M25_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  StackDev S{};
  S.nlayer = d->nlayer;
  S.nlev = d->nlev;
  S.single = d->single;
  S.top_pec = d->top_pec ? 1 : 0;
  double omega = 2.0 * kPi * d->freq;
  S.k0 = omega / kC0;
  S.h = d->stack_h;
  for (int n = 0; n < d->nlayer; ++n) {
    S.t[n] = d->layer_t[n];
    S.epsc[n] = zd(d->layer_eps[n], 0.0) * zd(1.0, -d->layer_tand[n]);
    S.kk[n] = csqrt(S.epsc[n]) * S.k0;
  }
  for (int l = 0; l < d->nlev; ++l) {
    S.il[l] = d->lev_iface[l];
    S.zl[l] = d->lev_z[l];
  }
  const int L = d->nlev, NC = 3 * L * L;
  m25_greens* g = new m25_greens();
  g->ctx = ctx;
  g->nlev = L;
  g->nrho = d->nrho;
  g->single = d->single;
  g->freq = d->freq;
  g->omega = omega;
  g->stack_h = d->stack_h;
  g->rho_h.assign(d->rho, d->rho + d->nrho);
  int rc = M25_OK;
  StackDev* Sd = nullptr;
  double *kc = nullptr, *wc = nullptr, *kr = nullptr, *wr = nullptr;
  zd *cc = nullptr, *cr = nullptr, *res = nullptr;
  std::vector<void*> tmp;
  const int n = d->nrho;
#define TRY(x)         \
  do {                 \
    rc = (x);          \
    if (rc) goto fail; \
  } while (0)
  TRY(alloc_async(tmp, (void**)&Sd, sizeof(StackDev), st));
  TRY(alloc_async(tmp, (void**)&kc, sizeof(double) * 2 * d->nk_c, st));
  TRY(alloc_async(tmp, (void**)&wc, sizeof(double) * 2 * d->nk_c, st));
  TRY(alloc_async(tmp, (void**)&kr, sizeof(double) * d->nk_r, st));
  TRY(alloc_async(tmp, (void**)&wr, sizeof(double) * d->nk_r, st));
  TRY(alloc_async(tmp, (void**)&cc, sizeof(zd) * (size_t)d->nk_c * NC, st));
  TRY(alloc_async(tmp, (void**)&cr, sizeof(zd) * (size_t)d->nk_r * NC, st));
  TRY(alloc_async(g->allocs, (void**)&res, sizeof(zd) * (size_t)n * NC, st));
  g->res = res;
  TRY(alloc_async(g->allocs, &g->sur, 16, st));
  M25_CUDA(cudaMemsetAsync(g->sur, 0, 16, st));
  TRY(alloc_async(g->allocs, (void**)&g->rho, sizeof(double) * n, st));
  TRY(alloc_async(g->allocs, (void**)&g->rho32, sizeof(float) * n, st));
  TRY(alloc_async(g->allocs, (void**)&g->S, sizeof(zd) * (size_t)NC * n, st));
  TRY(alloc_async(g->allocs, (void**)&g->coef, sizeof(zd) * (size_t)L * L * (n - 1) * 12, st));
  TRY(alloc_async(g->allocs, (void**)&g->coef32, sizeof(float) * 2 * (size_t)L * L * (n - 1) * 12, st));
  TRY(alloc_async(g->allocs, (void**)&g->lead, sizeof(StackDev), st));
  M25_CUDA(cudaMemcpyAsync(Sd, &S, sizeof(StackDev), cudaMemcpyHostToDevice, st));
  M25_CUDA(cudaMemcpyAsync(kc, d->kc, sizeof(double) * 2 * d->nk_c, cudaMemcpyHostToDevice, st));
  M25_CUDA(cudaMemcpyAsync(wc, d->wc, sizeof(double) * 2 * d->nk_c, cudaMemcpyHostToDevice, st));
  M25_CUDA(cudaMemcpyAsync(kr, d->kr, sizeof(double) * d->nk_r, cudaMemcpyHostToDevice, st));
  M25_CUDA(cudaMemcpyAsync(wr, d->wr, sizeof(double) * d->nk_r, cudaMemcpyHostToDevice, st));
  M25_CUDA(cudaMemcpyAsync(g->rho, d->rho, sizeof(double) * n, cudaMemcpyHostToDevice, st));
  {
  StageTimer tm(ctx, ST_GREENS);
  {
    zd* gbig = nullptr;
    TRY(alloc_async(tmp, (void**)&gbig, sizeof(zd) * NC, st));
    const int nodes = d->nk_c + d->nk_r + 1;
    spectral_g_kernel<<<(nodes + 63) / 64, 64, 0, st>>>(Sd, d->nk_c, kc, d->nk_r, kr, d->kbig, cc, cr, gbig);
    leading_kernel<<<1, 1, 0, st>>>(Sd, d->kbig, gbig);
    const int64_t ncoef = (int64_t)(d->nk_c + d->nk_r) * NC;
    spectral_coef_kernel<<<(unsigned)((ncoef + 127) / 128), 128, 0, st>>>(Sd, d->nk_c, kc, wc, d->nk_r, kr, wr, cc,
                                                                          cr);
  }
  {
    // the Sommerfeld integral at the radii rho[idx[e]], e < ne (idx NULL:
    // all n) into res; skip: see sommerfeld_kernel
    const int nsplit = som_split(d->nk_c + d->nk_r);
    zd* part = nullptr;
    TRY(alloc_async(tmp, (void**)&part, sizeof(zd) * (size_t)nsplit * n * NC, st));
    auto sommerfeld = [&](int ne, const int* idx, const int* skip) {
      if (ne <= 0) return;
      dim3 grid(ne, nsplit);
      switch (NC) {
        case 3:
          sommerfeld_kernel<3><<<grid, 256, 0, st>>>(ne, idx, g->rho, nsplit, d->nk_c, kc, cc, d->nk_r, kr, cr, part,
                                                     skip);
          break;
        case 12:
          sommerfeld_kernel<12><<<grid, 256, 0, st>>>(ne, idx, g->rho, nsplit, d->nk_c, kc, cc, d->nk_r, kr, cr, part,
                                                      skip);
          break;
        default:
          sommerfeld_kernel<27><<<grid, 256, 0, st>>>(ne, idx, g->rho, nsplit, d->nk_c, kc, cc, d->nk_r, kr, cr, part,
                                                      skip);
          break;
      }
      sommerfeld_sum_kernel<<<(ne * NC + 255) / 256, 256, 0, st>>>(ne, NC, idx, nsplit, part, res, skip);
    };
    // learned remainder: which radii get the Sommerfeld integral first
    std::vector<int> ie, kpos, vpos, ir;
    if (d->surrogate) {
      int nin = 0, nout = 0;
      mlp_dims(d->surrogate, &nin, &nout);
      if (nin != 2 || nout != 2 * NC || d->sur_stride < 2 || d->sur_stride > 64 || !(d->sur_near >= 0) ||
          !d->sur_scale || !(d->sur_fmax > d->sur_fmin) || !(d->sur_a > 0) || !(d->sur_rho_ref > 0)) {
        set_error("m25_greens_create: surrogate does not match the stack (2 inputs, 2 NC outputs, stride 2-64)");
        rc = M25_ERR_VALUE;
        goto fail;
      }
      std::vector<int> knots;
      int n0 = 0;
      while (n0 < n && d->rho[n0] < d->sur_near) knots.push_back(n0++);
      for (int i = n0; i < n; i += d->sur_stride) knots.push_back(i);
      if (knots.back() != n - 1) knots.push_back(n - 1);
      std::vector<char> exact(n, 0), val(n, 0);
      for (int i : knots) exact[i] = 1;
      for (size_t j = 0; j + 1 < knots.size(); ++j)
        if (knots[j + 1] - knots[j] >= 2) val[(knots[j] + knots[j + 1]) / 2] = 1;
      for (int i = 0; i < n; ++i) {
        if (exact[i] || val[i]) {
          if (exact[i]) kpos.push_back((int)ie.size());
          if (val[i]) vpos.push_back((int)ie.size());
          ie.push_back(i);
        } else {
          ir.push_back(i);
        }
      }
      if (kpos.size() < 4 || vpos.empty() || ir.empty() ||
          std::max(sur_judge_smem((int)ie.size(), (int)kpos.size()), sur_fill_smem((int)ie.size())) >
              kSurSmemMax) {  // the plain tabulation
        ie.clear();
        kpos.clear();
        vpos.clear();
        ir.clear();
      }
    }
    if (!ie.empty()) {
      // the network at every radius, the Sommerfeld integral at the knots and
      // validation radii, the judge, then the integral at the other radii
      // unless the judge accepted
      const int ne = (int)ie.size(), nk = (int)kpos.size(), nv = (int)vpos.size(), nr = (int)ir.size();
      std::vector<int> lists;
      lists.insert(lists.end(), ie.begin(), ie.end());
      lists.insert(lists.end(), kpos.begin(), kpos.end());
      lists.insert(lists.end(), vpos.begin(), vpos.end());
      lists.insert(lists.end(), ir.begin(), ir.end());
      int* dl = nullptr;
      double *scl = nullptr, *colerr = nullptr;
      float *X = nullptr, *Y = nullptr;
      TRY(alloc_async(tmp, (void**)&dl, sizeof(int) * lists.size(), st));
      TRY(alloc_async(tmp, (void**)&scl, sizeof(double) * 2 * NC, st));
      TRY(alloc_async(tmp, (void**)&X, sizeof(float) * 2 * (size_t)n, st));
      TRY(alloc_async(tmp, (void**)&Y, sizeof(float) * 2 * NC * (size_t)n, st));
      TRY(alloc_async(tmp, (void**)&colerr, sizeof(double) * 2 * 2 * NC, st));
      M25_CUDA(cudaMemcpyAsync(dl, lists.data(), sizeof(int) * lists.size(), cudaMemcpyHostToDevice, st));
      M25_CUDA(cudaMemcpyAsync(scl, d->sur_scale, sizeof(double) * 2 * NC, cudaMemcpyHostToDevice, st));
      const int *d_ie = dl, *d_kpos = dl + ne, *d_vpos = dl + ne + nk, *d_ir = dl + ne + nk + nv;
      sur_features_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, g->rho, d->sur_a, d->sur_rho_ref, d->freq, d->sur_fmin,
                                                           d->sur_fmax, X);
      TRY(mlp_forward_device(d->surrogate, n, X, Y, st));
      sommerfeld(ne, d_ie, nullptr);
      int* flag = static_cast<int*>(g->sur);
      double* err = reinterpret_cast<double*>(static_cast<char*>(g->sur) + 8);
      static const bool smem_attr =
          cudaFuncSetAttribute(sur_judge_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSurSmemMax) ==
              cudaSuccess &&
          cudaFuncSetAttribute(sur_fill_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSurSmemMax) ==
              cudaSuccess;
      if (!smem_attr) {
        set_error("m25_greens_create: the learned remainder's shared memory could not be reserved");
        rc = M25_ERR_CUDA;
        goto fail;
      }
      sur_judge_kernel<<<2 * NC, 256, sur_judge_smem(ne, nk), st>>>(NC, g->rho, ne, d_ie, nk, d_kpos, nv, d_vpos, Y,
                                                                    scl, res, colerr);
      sur_fill_kernel<<<2 * NC, 256, sur_fill_smem(ne), st>>>(NC, g->rho, ne, d_ie, nr, d_ir, Y, scl, colerr,
                                                            d->sur_tol, res, flag, err);
      sommerfeld(nr, d_ir, flag);  // the integral at the other radii unless the judge accepted
      g->sur_planned = ne;
    } else {
      sommerfeld(n, nullptr, nullptr);
    }
  }
  table_kernel<<<(NC * n + 127) / 128, 128, 0, st>>>(Sd, n, g->rho, res, omega, zd(d->zs_ground_re, d->zs_ground_im),
                                                   reinterpret_cast<zd*>(g->S));
  {
    const bool pcr = spline_smem_pcr(n) <= 200 * 1024;
    if (!pcr && spline_smem(n) > 200 * 1024) {
      set_error("m25_greens_create: too many tabulation radii for the spline in shared memory");
      rc = M25_ERR_VALUE;
      goto fail;
    }
    static const bool spline_attr =
        cudaFuncSetAttribute(spline_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) ==
            cudaSuccess &&
        cudaFuncSetAttribute(spline_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) ==
            cudaSuccess;
    if (!spline_attr) {
      set_error("m25_greens_create: the spline's shared memory could not be reserved");
      rc = M25_ERR_CUDA;
      goto fail;
    }
    if (pcr)
      spline_kernel<true><<<NC, 128, spline_smem_pcr(n), st>>>(L, n, g->rho, reinterpret_cast<zd*>(g->S),
                                                               reinterpret_cast<zd*>(g->coef));
    else
      spline_kernel<false><<<NC, 128, spline_smem(n), st>>>(L, n, g->rho, reinterpret_cast<zd*>(g->S),
                                                            reinterpret_cast<zd*>(g->coef));
  }
  {
    int64_t nc = (int64_t)L * L * (n - 1) * 12 * 2;
    to_f32_kernel<<<(unsigned)((nc + 255) / 256), 256, 0, st>>>(g->coef, g->coef32, nc);
    to_f32_kernel<<<(n + 255) / 256, 256, 0, st>>>(g->rho, g->rho32, n);
  }
  }
  M25_CUDA(cudaMemcpyAsync(g->lead, Sd, sizeof(StackDev), cudaMemcpyDeviceToDevice, st));
  M25_CHECK_LAUNCH();
  // temporaries are released once the stream has consumed them
  free_all_async(tmp, st);
  {
    StackDev h;
    M25_CUDA(cudaMemcpyAsync(&h, g->lead, sizeof(StackDev), cudaMemcpyDeviceToHost, st));
    M25_CUDA(cudaStreamSynchronize(st));
    g->lead_h.resize(3 * L * L);
    g->dz_h.resize(L * L);
    for (int m = 0; m < 3; ++m)
      for (int i = 0; i < L; ++i)
        for (int j = 0; j < L; ++j) g->lead_h[(m * L + i) * L + j] = h.lead_c[m][i][j];
    for (int i = 0; i < L; ++i)
      for (int j = 0; j < L; ++j) g->dz_h[i * L + j] = h.dz[i][j];
  }
  if (d->surrogate) {
    char hs[16];
    M25_CUDA(cudaMemcpy(hs, g->sur, 16, cudaMemcpyDeviceToHost));  // the stream is idle here
    int acc;
    memcpy(&acc, hs, sizeof(int));
    memcpy(&g->sur_info[1], hs + 8, sizeof(double));
    g->sur_info[0] = acc;
    g->sur_info[2] = acc ? g->sur_planned : n;
  } else {
    g->sur_info[2] = n;
  }
  *out = g;
  return M25_OK;
fail:
  cudaStreamSynchronize(st);
  free_all_async(tmp, st);
  free_all_async(g->allocs, st);
  delete g;
  return rc;
#undef TRY
}

extern "C" int m25_greens_destroy(m25_greens* g) {
  if (!g) return M25_OK;
  free_all_async(g->allocs, g->ctx->stream);
  delete g;
  return M25_OK;
}

extern "C" int m25_greens_remainder(m25_greens* g, double* res, double* info) {
  if (!g) {
    set_error("m25_greens_remainder: null greens");
    return M25_ERR_VALUE;
  }
  M25_CUDA(cudaStreamSynchronize(g->ctx->stream));
  if (res)
    M25_CUDA(cudaMemcpy(res, g->res, sizeof(zd) * (size_t)g->nrho * 3 * g->nlev * g->nlev, cudaMemcpyDeviceToHost));
  if (info) {
    info[0] = g->sur_info[0];
    info[1] = g->sur_info[1];
    info[2] = g->sur_info[2];
  }
  return M25_OK;
}

extern "C" int m25_greens_tables(m25_greens* g, double* S, double* c, double* coef) {
  if (!g) {
    set_error("m25_greens_tables: null greens");
    return M25_ERR_VALUE;
  }
  const int L = g->nlev, n = g->nrho;
  M25_CUDA(cudaStreamSynchronize(g->ctx->stream));
  if (S) M25_CUDA(cudaMemcpy(S, g->S, sizeof(zd) * 3 * L * L * n, cudaMemcpyDeviceToHost));
  if (c)
    for (int k = 0; k < 3 * L * L; ++k) {
      c[2 * k] = g->lead_h[k].re;
      c[2 * k + 1] = g->lead_h[k].im;
    }
  if (coef) M25_CUDA(cudaMemcpy(coef, g->coef, sizeof(zd) * (size_t)L * L * (n - 1) * 12, cudaMemcpyDeviceToHost));
  return M25_OK;
}
