// Tabulated spatial Green's functions at one frequency, computed on the
// device: the remainder of the spectral MPIE kernels after removing the
// leading c e^{-jkR}/(4 pi R) terms, integrated along a lifted Sommerfeld
// path, tabulated on a rho grid and fitted with not-a-knot cubic splines.
// Follows Engine/mom25d/greens.py:111-212 (one grounded slab) and
// Engine/mom25d/layered.py:238-405 (open multilayer stack, Michalski-Zheng
// transmission-line form).
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
    yup[N] = yair;
    for (int k = N - 1; k >= 1; --k) {
      zd yk = y[k], tk = T[k], yl = yup[k + 1];
      yup[k] = yk * (yl + yk * tk) / (yk + yl * tk);
    }
    for (int l = 0; l < L; ++l) {
      zd* V = Vmode[mode][l];
      for (int k = 0; k <= N; ++k) V[k] = zd(0.0);
      int s = S.il[l];
      V[s] = zd(1.0) / (ydn[s] + yup[s]);
      for (int k = s; k >= 2; --k) V[k - 1] = V[k] * Sh[k - 1] / (zd(1.0) + ydn[k - 1] / y[k - 1] * T[k - 1]);
      for (int k = s; k < N; ++k) V[k + 1] = V[k] * Sh[k] / (zd(1.0) + yup[k + 1] / y[k] * T[k]);
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

// Leading-term coefficients (greens.py:215-224, layered.py:292-331).
__global__ void leading_kernel(StackDev* S, double kbig) {
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
  bool have_big = false;
  zd big[3][kMaxLev][kMaxLev];
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
      if (!have_big) {
        layered_spectral(s, zd(kbig), big);
        have_big = true;
      }
      zd ux = csqrt(zd(kbig * kbig - s.k0 * s.k0));
      zd f = ux * 2.0 * cexp(ux * s.dz[i][j]);
      zd c[3];
      for (int m = 0; m < 3; ++m) c[m] = f * big[m][i][j];
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

// coef[k][(m*L + i)*L + j] = w k g_rem(k) / 2pi at every path point.
__global__ void spectral_coef_kernel(const StackDev* __restrict__ Sp, int nk, const double* __restrict__ kpts,
                                     const double* __restrict__ wpts, int complex_path, zd* __restrict__ coef) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nk) return;
  const StackDev& S = *Sp;
  const int L = S.nlev;
  zd kr = complex_path ? zd(kpts[2 * q], kpts[2 * q + 1]) : zd(kpts[q], 0.0);
  zd w = complex_path ? zd(wpts[2 * q], wpts[2 * q + 1]) : zd(wpts[q], 0.0);
  zd g[3][kMaxLev][kMaxLev];
  if (S.single) {
    slab_spectral(S, kr, g[0][0][0], g[1][0][0], g[2][0][0]);
  } else {
    layered_spectral(S, kr, g);
  }
  zd kr2 = kr * kr;
  zd scale = (w * kr) / (2.0 * kPi);
  for (int m = 0; m < 3; ++m)
    for (int i = 0; i < L; ++i)
      for (int j = 0; j < L; ++j) {
        zd kx = S.kx[m == 0 ? 0 : 1][i][j];
        zd ux = csqrt(kr2 - kx * kx);
        zd lead = S.lead_c[m][i][j] * cexp(ux * (-S.dz[i][j])) / (ux * 2.0);
        coef[(int64_t)q * (3 * L * L) + (m * L + i) * L + j] = scale * (g[m][i][j] - lead);
      }
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

// res[rho][c] = sum_k J0(rho k) coef[k][c] over the lifted arc (complex J0)
// and the real axis (real J0), one CTA per radius.
// With skip set (the learned remainder was accepted) the CTAs return at once.
template <int NC>
__global__ void sommerfeld_kernel(int nrho, const double* __restrict__ rho, int nkc, const double* __restrict__ kc,
                                  const zd* __restrict__ coef_c, int nkr, const double* __restrict__ kr,
                                  const zd* __restrict__ coef_r, zd* __restrict__ res, const int* __restrict__ skip) {
  if (skip && *skip) return;
  int ir = blockIdx.x;
  double r = rho[ir];
  double acc_re[NC], acc_im[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) acc_re[c] = acc_im[c] = 0.0;
  for (int q = threadIdx.x; q < nkc; q += blockDim.x) {
    zd J = bessel_j0_complex(zd(r * kc[2 * q], r * kc[2 * q + 1]));
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      zd v = J * coef_c[(int64_t)q * NC + c];
      acc_re[c] += v.re;
      acc_im[c] += v.im;
    }
  }
  for (int q = threadIdx.x; q < nkr; q += blockDim.x) {
    double J = j0(r * kr[q]);
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      zd v = coef_r[(int64_t)q * NC + c];
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
      res[(int64_t)ir * NC + c] = zd(sa, sb);
    }
    __syncthreads();
  }
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
__host__ __device__ inline size_t spline_smem(int n) { return (size_t)n * (2 * sizeof(double) + 4 * sizeof(zd)); }

__global__ void __launch_bounds__(128) spline_kernel(int L, int nrho, const double* __restrict__ xg,
                                                     const zd* __restrict__ Stab, zd* __restrict__ coef) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int col = blockIdx.x;
  const int n = nrho;
  zd* y = reinterpret_cast<zd*>(smem_raw);  // (n) values
  zd* s = y + n;                            // (n) slopes
  zd* cp = s + n;                           // (n) modified diagonal (re), upper diagonal (im)
  zd* sl = cp + n;                          // (n - 1) secant slopes
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
  // rows: a_i s_{i-1} + b_i s_i + c_i s_{i+1} = d_i
  auto dxf = [&](int i) { return dx[i]; };
  auto slope = [&](int i) { return sl[i]; };
  if (threadIdx.x == 0) {
    // forward sweep
    double bprev = 0, cprev = 0;
    for (int i = 0; i < n; ++i) {
      double a, b, c;
      zd d;
      if (i == 0) {
        double dx0 = dxf(0), dx1 = dxf(1), d0 = x[2] - x[0];
        a = 0;
        b = dx1;
        c = d0;
        d = (slope(0) * ((dx0 + 2 * d0) * dx1) + slope(1) * (dx0 * dx0)) / d0;
      } else if (i == n - 1) {
        double dxl = dxf(n - 2), dxm = dxf(n - 3), d1 = x[n - 1] - x[n - 3];
        a = d1;
        b = dxm;
        c = 0;
        d = (slope(n - 3) * (dxl * dxl) + slope(n - 2) * ((2 * d1 + dxl) * dxm)) / d1;
      } else {
        a = dxf(i);
        b = 2 * (dxf(i - 1) + dxf(i));
        c = dxf(i - 1);
        d = (slope(i - 1) * dxf(i) + slope(i) * dxf(i - 1)) * 3.0;
      }
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

constexpr int kSurMaxCheck = 128;
constexpr int kSurMaxCols = 2 * 3 * kMaxLevSq;
// dynamic shared memory of the judge: the residuals and spline moments at
// the K check radii, K x 2 NC doubles each
inline size_t sur_judge_smem(int K, int NC) { return sizeof(double) * 2 * (size_t)K * 2 * NC; }

// Residual correction and judge (one CTA): natural cubic splines in rho of
// the Sommerfeld-minus-network residual of every real column through the K
// check radii; res (table radii) = network + spline; accepted when the
// largest error at the K - 1 validation radii is <= tol x the largest
// |remainder| at the check radii.
__global__ void __launch_bounds__(256) sur_judge_kernel(int NC, int n, const double* __restrict__ rho, int K,
                                                        const double* __restrict__ rchk, const float* __restrict__ ytab,
                                                        const float* __restrict__ ychk, const double* __restrict__ scale,
                                                        const zd* __restrict__ schk, double tol, zd* __restrict__ res,
                                                        int* __restrict__ flag, double* __restrict__ err_out) {
  extern __shared__ double judge_smem[];
  __shared__ double red_e[8], red_s[8];
  const int ncol = 2 * NC;
  const int c = threadIdx.x;
  double* rs = judge_smem;              // residual at check radius k, column c: rs[k ncol + c]
  double* Ms = judge_smem + K * ncol;   // its spline's second derivative there
#define r(k, col) rs[(k) * ncol + (col)]
#define M(k, col) Ms[(k) * ncol + (col)]
  auto truth = [&](int k, int col) {
    const zd v = schk[(int64_t)k * NC + (col >> 1)];
    return (col & 1) ? v.im : v.re;
  };
  if (c < ncol) {
    for (int k = 0; k < K; ++k) r(k, c) = truth(k, c) - scale[c] * (double)ychk[(int64_t)k * ncol + c];
    // natural spline: M_0 = M_{K-1} = 0, tridiagonal system for the interior (Thomas)
    double cp[kSurMaxCheck], dp[kSurMaxCheck];
    cp[0] = 0.0;
    dp[0] = 0.0;
    for (int k = 1; k < K - 1; ++k) {
      const double h0 = rchk[k] - rchk[k - 1], h1 = rchk[k + 1] - rchk[k];
      const double rhs = 6.0 * ((r(k + 1, c) - r(k, c)) / h1 - (r(k, c) - r(k - 1, c)) / h0);
      const double den = 2.0 * (h0 + h1) - h0 * cp[k - 1];
      cp[k] = h1 / den;
      dp[k] = (rhs - h0 * dp[k - 1]) / den;
    }
    M(K - 1, c) = 0.0;
    for (int k = K - 2; k >= 1; --k) M(k, c) = dp[k] - cp[k] * M(k + 1, c);
    M(0, c) = 0.0;
  }
  __syncthreads();
  auto spline = [&](double x, int col) {
    int lo = 0, hi = K - 1;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (x < rchk[mid]) hi = mid; else lo = mid;
    }
    const double h = rchk[lo + 1] - rchk[lo], t = x - rchk[lo];
    const double b = (r(lo + 1, col) - r(lo, col)) / h - h * (2.0 * M(lo, col) + M(lo + 1, col)) / 6.0;
    return r(lo, col) + t * (b + t * (0.5 * M(lo, col) + t * (M(lo + 1, col) - M(lo, col)) / (6.0 * h)));
  };
  // validation radii rchk[K .. 2K-2]
  double emax = 0.0, smax = 0.0;
  for (int e = threadIdx.x; e < (K - 1) * ncol; e += blockDim.x) {
    const int v = K + e / ncol, col = e % ncol;
    const double pred = scale[col] * (double)ychk[(int64_t)v * ncol + col] + spline(rchk[v], col);
    emax = fmax(emax, fabs(pred - truth(v, col)));
  }
  for (int e = threadIdx.x; e < K * NC; e += blockDim.x) {
    const zd v = schk[e];
    smax = fmax(smax, sqrt(v.re * v.re + v.im * v.im));
  }
  for (int o = 16; o; o >>= 1) {
    emax = fmax(emax, __shfl_down_sync(0xffffffffu, emax, o));
    smax = fmax(smax, __shfl_down_sync(0xffffffffu, smax, o));
  }
  if ((threadIdx.x & 31) == 0) {
    red_e[threadIdx.x >> 5] = emax;
    red_s[threadIdx.x >> 5] = smax;
  }
  // the corrected network values at the table radii
  for (int e = threadIdx.x; e < n * ncol; e += blockDim.x) {
    const int i = e / ncol, col = e % ncol;
    const double v = scale[col] * (double)ytab[(int64_t)i * ncol + col] + spline(rho[i], col);
    double* out = reinterpret_cast<double*>(res + (int64_t)i * NC + (col >> 1));
    out[col & 1] = v;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double e = 0, sm = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      e = fmax(e, red_e[w]);
      sm = fmax(sm, red_s[w]);
    }
    const double rel = sm > 0 ? e / sm : INFINITY;
    *err_out = rel;
    *flag = rel <= tol ? 1 : 0;
  }
#undef r
#undef M
}

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
    if (d->lev_iface[l] < 1 || d->lev_iface[l] > d->nlayer) {
      set_error("m25_greens_create: level interface out of range");
      return M25_ERR_VALUE;
    }
  M25_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  StackDev S{};
  S.nlayer = d->nlayer;
  S.nlev = d->nlev;
  S.single = d->single;
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
  leading_kernel<<<1, 1, 0, st>>>(Sd, d->kbig);
  spectral_coef_kernel<<<(d->nk_c + 127) / 128, 128, 0, st>>>(Sd, d->nk_c, kc, wc, 1, cc);
  spectral_coef_kernel<<<(d->nk_r + 127) / 128, 128, 0, st>>>(Sd, d->nk_r, kr, wr, 0, cr);
  {
    // the Sommerfeld integral at nr radii (rr) into out; skip: see sommerfeld_kernel
    auto sommerfeld = [&](int nr, const double* rr, zd* outp, const int* skip) {
      switch (NC) {
        case 3: sommerfeld_kernel<3><<<nr, 256, 0, st>>>(nr, rr, d->nk_c, kc, cc, d->nk_r, kr, cr, outp, skip); break;
        case 12: sommerfeld_kernel<12><<<nr, 256, 0, st>>>(nr, rr, d->nk_c, kc, cc, d->nk_r, kr, cr, outp, skip); break;
        default: sommerfeld_kernel<27><<<nr, 256, 0, st>>>(nr, rr, d->nk_c, kc, cc, d->nk_r, kr, cr, outp, skip); break;
      }
    };
    if (d->surrogate) {
      // learned remainder: the network at the table radii and at K check +
      // K - 1 validation radii, the Sommerfeld integral at the latter only
      const int K = d->sur_ncheck, nv = 2 * K - 1;
      int nin = 0, nout = 0;
      mlp_dims(d->surrogate, &nin, &nout);
      if (nin != 2 || nout != 2 * NC || K < 4 || K > kSurMaxCheck || !d->sur_scale || !(d->sur_fmax > d->sur_fmin) ||
          !(d->sur_a > 0) || !(d->sur_rho_ref > 0)) {
        set_error("m25_greens_create: surrogate does not match the stack (2 inputs, 2 NC outputs, 4-128 check radii)");
        rc = M25_ERR_VALUE;
        goto fail;
      }
      std::vector<double> hr(nv);
      const double rlast = d->rho[n - 1];
      for (int k = 0; k < K; ++k) hr[k] = rlast * ((double)k / (K - 1)) * ((double)k / (K - 1));
      for (int k = 0; k + 1 < K; ++k) hr[K + k] = rlast * ((k + 0.5) / (K - 1)) * ((k + 0.5) / (K - 1));
      double *rchk = nullptr, *scl = nullptr;
      float *X = nullptr, *Y = nullptr;
      zd* schk = nullptr;
      TRY(alloc_async(tmp, (void**)&rchk, sizeof(double) * nv, st));
      TRY(alloc_async(tmp, (void**)&scl, sizeof(double) * 2 * NC, st));
      TRY(alloc_async(tmp, (void**)&X, sizeof(float) * 2 * (size_t)(n + nv), st));
      TRY(alloc_async(tmp, (void**)&Y, sizeof(float) * 2 * NC * (size_t)(n + nv), st));
      TRY(alloc_async(tmp, (void**)&schk, sizeof(zd) * NC * (size_t)nv, st));
      M25_CUDA(cudaMemcpyAsync(rchk, hr.data(), sizeof(double) * nv, cudaMemcpyHostToDevice, st));
      M25_CUDA(cudaMemcpyAsync(scl, d->sur_scale, sizeof(double) * 2 * NC, cudaMemcpyHostToDevice, st));
      sur_features_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, g->rho, d->sur_a, d->sur_rho_ref, d->freq, d->sur_fmin,
                                                           d->sur_fmax, X);
      sur_features_kernel<<<(nv + 127) / 128, 128, 0, st>>>(nv, rchk, d->sur_a, d->sur_rho_ref, d->freq, d->sur_fmin,
                                                            d->sur_fmax, X + 2 * (size_t)n);
      TRY(mlp_forward_device(d->surrogate, n + nv, X, Y, st));
      sommerfeld(nv, rchk, schk, nullptr);
      int* flag = static_cast<int*>(g->sur);
      double* err = reinterpret_cast<double*>(static_cast<char*>(g->sur) + 8);
      static const bool judge_attr = cudaFuncSetAttribute(sur_judge_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                          (int)sur_judge_smem(kSurMaxCheck, kSurMaxCols / 2)) ==
                                     cudaSuccess;
      if (!judge_attr) {
        set_error("m25_greens_create: the surrogate judge's shared memory could not be reserved");
        rc = M25_ERR_CUDA;
        goto fail;
      }
      sur_judge_kernel<<<1, 256, sur_judge_smem(K, NC), st>>>(NC, n, g->rho, K, rchk, Y, Y + 2 * NC * (size_t)n, scl,
                                                             schk, d->sur_tol, res, flag, err);
      sommerfeld(n, g->rho, res, flag);  // the full integral unless the judge accepted
    } else {
      sommerfeld(n, g->rho, res, nullptr);
    }
  }
  table_kernel<<<(NC * n + 127) / 128, 128, 0, st>>>(Sd, n, g->rho, res, omega, zd(d->zs_ground_re, d->zs_ground_im),
                                                   reinterpret_cast<zd*>(g->S));
  if (spline_smem(n) > 200 * 1024) {
    set_error("m25_greens_create: too many tabulation radii for the spline in shared memory");
    rc = M25_ERR_VALUE;
    goto fail;
  }
  M25_CUDA(cudaFuncSetAttribute(spline_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
  spline_kernel<<<NC, 128, spline_smem(n), st>>>(L, n, g->rho, reinterpret_cast<zd*>(g->S),
                                                 reinterpret_cast<zd*>(g->coef));
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
