// MPIE / RWG impedance fill (Engine/mom25d/solver.py:429-524 and the
// compiled form of the same fill, Engine/mom25d/_fast.py:82-158):
//
//   Z_mn = jw mu0 <f_m, gA * f_n> + 1/(jw eps0) <div f_m, gV * div f_n> + Zs <f_m, f_n>
//
// Stage 1 (fill_tri_kernel): one CTA per test block of 32 Morton-ordered
// triangles of one level, one warp lane per test triangle; the warps walk the
// source triangles, so every lane of a warp sees the same source and the same
// near/mid/far class (no divergence). Each (test, source) triangle pair gives
// a 3x3 block of half-basis values, written to the scratch H laid out
// [source half-basis][test half-basis slot] so the 32 lanes store one
// contiguous run per source half-basis.
// Stage 2 (gather_sym_kernel): each RWG entry sums its 2 x 2 half-basis values
// and the symmetrisation 0.5 (Z + Z^T) is applied, so every Z entry has a
// single writer (no atomics).
// Stage 3 (via_rows_kernel, via_block_kernel): rows / columns of the via
// segment unknowns (Engine/mom25d/solver.py:527-566).
#include <algorithm>
#include <type_traits>
#include <vector>

#include "m25_internal.h"

namespace m25 {

// mixed fill: H32's entry of a near pair, a quiet NaN carrying the pair's code
// (< 2^22) in its payload; the gather reads the fp64 value from Hn
constexpr uint32_t kNearTag = 0x7FC00000u;
constexpr int64_t kMaxNearTagged = (1 << 22) - 1;

template <class T>
struct FillArgs {
  int nt, nb, nlev, nblocks, n_src_chunk, n_chunks;
  const TriData<T>* td;
  const double* cen;
  const float4* cen_df;  // mixed fill: the centroids in double-float
  const int32_t* tri_layer;
  const int32_t* block_tris;
  const int32_t* block_level;
  const int32_t* cls;
  const T* stat;
  const float2* stat6;  // mixed fill: test-point sums of the near pairs' closed-form parts (double-float)
  const TriDF* tddf;    // mixed fill: the triangles' vertices and amplitudes in double-float
  const int32_t* pad_pos;
  int nrho;
  const T* rho;        // (nrho)
  const T* coef;       // (L*L, nrho-1, 4, 3) complex: A, V, W
  cx<T> lead[kMaxLevSq][2];  // cA, cV of pair (lt*L + ls)
  T dz[kMaxLevSq];
  cx<T> jwmu, inv_jwe, zs;
  cx<T>* H;            // (3 nt, ldh) (fp64 fill)
  int64_t ldh;
  cx<float>* H32;      // mixed fill: (3 nt, ldh), the mid / far pairs' values (computed in fp32)
  float4* Hn;          // mixed fill: (nnear, 3 j, 3 i, 32 lanes), the near pairs' values in double-float
  cx<T>* IVpad;        // (npad, nt)
  // fp32 copies for far pairs evaluated in fp32 (fill_tri_kernel<double, true>)
  const TriData<float>* td32;
  const float* coef32;
  cx<float> lead32[kMaxLevSq][2];
  float dz32[kMaxLevSq];
  cx<float> jwmu32, inv_jwe32;
  float4 lead_df[kMaxLevSq][2];  // mixed fill, near pairs: cA, cV in double-float
  float4 jwmu_df, inv_jwe_df, zs_df;  // and the surface impedance (has_zs: not 0)
  int has_zs;
  int* work_counter;   // items handed out beyond the first gridDim.x (zeroed before the launch)
  // listed fill (fp64; the compressed operator's near field): per (test
  // block, source triangle) -1 skip, -2 compute for the via pads' IVpad
  // only, >= 0 the slot of the pair's values in Hc; nullptr: every pair, into H
  const int32_t* cidx = nullptr;
  cx<T>* Hc = nullptr;  // (slots, 3 j, 3 i, 32 lanes)
  int nbk;             // mixed fill: buckets of the radius index (0: binary search)
  float bk_scale;      // buckets per unit radius
};

// scipy PPoly interval: x[i] <= r < x[i+1], clamped to the end intervals.
template <class T>
__device__ __forceinline__ int find_interval(const T* __restrict__ x, int n, T r) {
  if (r < x[1]) return 0;
  if (r >= x[n - 2]) return n - 2;
  int lo = 1, hi = n - 2;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (r < x[mid]) hi = mid; else lo = mid;
  }
  return lo;
}

// The same interval with the search in fp32 on a rounded copy xf of the
// radii (the fp64 pipe of this GPU is the fill's bottleneck): rounding is
// monotone and the radii are far apart against fp32 resolution, so the fp32
// index is the fp64 one or one above it; one fp64 comparison settles it.
// Bucket index of the fp32 radii (mixed fill): t[j] = the interval of radius
// j / scale; buckets are no wider than the smallest radius step, so a radius
// lies in t[j] or a step or two from it.
struct Bk {
  const uint16_t* t = nullptr;
  float scale = 0.f;
  int nb = 0;
};

template <class T>
__device__ __forceinline__ int find_interval_f(const T* __restrict__ x, const float* __restrict__ xf, int n, T r,
                                               Bk bk = Bk()) {
  const float rf = (float)r;
  int lo;
  if (bk.t) {
    lo = bk.t[min((int)(rf * bk.scale), bk.nb - 1)];
    if (lo > 0 && rf < xf[lo]) --lo;  // rf * scale rounded into the next bucket
    while (lo < n - 2 && xf[lo + 1] <= rf) ++lo;
  } else if (rf < xf[1]) {
    lo = 0;
  } else if (rf >= xf[n - 2]) {
    lo = n - 2;
  } else {
    lo = 1;
    int hi = n - 2;
    while (hi - lo > 1) {
      int mid = (lo + hi) >> 1;
      if (rf < xf[mid]) hi = mid; else lo = mid;
    }
  }
  if (lo > 0 && r < x[lo]) --lo;
  return lo;
}

// Smooth parts S_A, S_V at radius r from the shared-memory table of one pair:
// sum_p c[3-p] (r - x_i)^p, the order PPoly evaluates.
template <class T>
__device__ __forceinline__ void spline_av(const T* __restrict__ xs, const float* __restrict__ xf,
                                          const T* __restrict__ tab, int n, T r, cx<T>& sa, cx<T>& sv,
                                          Bk bk = Bk()) {
  int i = find_interval_f(xs, xf, n, r, bk);
  T dx = r - xs[i];
  const T* c = tab + (size_t)i * 16;  // [power 0..3][A re, A im, V re, V im], highest power first
  T z = dx, z2 = dx * dx, z3 = z2 * dx;
  sa.re = c[12] + c[8] * z + c[4] * z2 + c[0] * z3;
  sa.im = c[13] + c[9] * z + c[5] * z2 + c[1] * z3;
  sv.re = c[14] + c[10] * z + c[6] * z2 + c[2] * z3;
  sv.im = c[15] + c[11] * z + c[7] * z2 + c[3] * z3;
}

template <class T, int NQ, bool NEAR>
__device__ __forceinline__ void source_pass(int nrho, const TriData<T>& S, T dcx, T dcy,
                                            const T (&tq)[7][2], const T (&tw)[7], const T* xs, const float* xf,
                                            const T* tab,
                                            cx<T> cA, cx<T> cV, T dz, const T* st, int lane, cx<T> (&Q)[3],
                                            cx<T> (&Px)[3], cx<T> (&Py)[3], cx<T>& IV, const T (&tv)[3][2],
                                            Bk bk = Bk()) {
  const T inv4pi = T(1.0 / (4.0 * kPi));
  cx<T> S0, SX, SY, T0, T1, T2;  // sums of w_k K over the test points k, weighted by 1, x_k, y_k
  T sq[NQ][2], sw[NQ];
#pragma unroll
  for (int l = 0; l < NQ; ++l) {
    if (NQ == 7) {
      sq[l][0] = S.q7[l][0];
      sq[l][1] = S.q7[l][1];
      sw[l] = S.w7[l];
    } else if (NQ == 3) {
      sq[l][0] = S.q3[l][0];
      sq[l][1] = S.q3[l][1];
      sw[l] = S.w3[l];
    } else {
      sq[l][0] = T(0);
      sq[l][1] = T(0);
      sw[l] = S.area;
    }
  }
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    cx<T> K0A, K1x, K1y, K0V;
    if (NEAR) {
      T s0 = st[(0 * 7 + k) * 32 + lane], s1x = st[(1 * 7 + k) * 32 + lane], s2y = st[(2 * 7 + k) * 32 + lane];
      K0A = cA * s0;
      K1x = cA * s1x;
      K1y = cA * s2y;
      K0V = cV * s0;
    }
    // test point relative to the source centroid
    const T rx = dcx + tq[k][0], ry = dcy + tq[k][1];
#pragma unroll
    for (int l = 0; l < NQ; ++l) {
      T ddx = rx - sq[l][0], ddy = ry - sq[l][1];
      const T R2 = ddx * ddx + ddy * ddy;
      T R, inv = T(0);
      if (NEAR) {
        R = sqrt(R2);  // may be 0 (coincident points of a self pair)
      } else {
        // distinct triangles: one reciprocal square root gives R and 1/R
        const T ri = rsqrt(R2);
        R = R2 * ri;
        inv = inv4pi * (dz == T(0) ? ri : rsqrt(R2 + dz * dz));
      }
      cx<T> sa, sv;
      spline_av(xs, xf, tab, nrho, R, sa, sv, bk);
      if (!NEAR) {
        sa += cA * inv;
        sv += cV * inv;
      }
      cx<T> saw = sa * sw[l];
      K0A += saw;
      if (NQ > 1) {  // the one-point rule sits on the centroid: no first moments
        K1x += saw * sq[l][0];
        K1y += saw * sq[l][1];
      }
      K0V += sv * sw[l];
    }
    // sums over the test points; the vertex terms a_i are applied once below
    const T wk = tw[k], wx = wk * tq[k][0], wy = wk * tq[k][1];
    IV += K0V * wk;
    S0 += K0A * wk;
    SX += K0A * wx;
    SY += K0A * wy;
    if (NEAR || NQ > 1) {  // the one-point rule has no first moments
      T1 += K1x * wk;
      T2 += K1y * wk;
      T0 += K1x * wx + K1y * wy;
    }
  }
  // sum_k w_k (r_k - a_i) K, lengths about the test centroid
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    Px[i] = SX - S0 * tv[i][0];
    Py[i] = SY - S0 * tv[i][1];
    Q[i] = T0 - (T1 * tv[i][0] + T2 * tv[i][1]);
  }
}

// ---- double-float arithmetic on the fp32 pipes (GB300 issues fp64 at 1/64
// of the fp32 rate): a value is h + l with h its fp32 rounding; the error-free
// sum (Knuth) and product (FMA) keep about 2^-46 relative, against 2^-53 for
// fp64 and 2^-24 for fp32. The _rn intrinsics keep the compiler from fusing
// the steps whose rounding the transforms recover.
struct dff {
  float h, l;
};
struct dfc {
  dff re, im;
};
__device__ __forceinline__ dff df_add(dff a, dff b) {
  const float s = __fadd_rn(a.h, b.h), z = __fsub_rn(s, a.h);
  float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, z)), __fsub_rn(b.h, z));
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  const float h = __fadd_rn(s, e);
  return {h, __fsub_rn(e, __fsub_rn(h, s))};
}
__device__ __forceinline__ dff df_neg(dff a) { return {-a.h, -a.l}; }
__device__ __forceinline__ dff df_mul(dff a, dff b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, fmaf(a.l, b.h, e));
  const float h = __fadd_rn(p, e);
  return {h, __fsub_rn(e, __fsub_rn(h, p))};
}
__device__ __forceinline__ dfc dfc_add(dfc a, dfc b) { return {df_add(a.re, b.re), df_add(a.im, b.im)}; }
__device__ __forceinline__ dfc dfc_sub(dfc a, dfc b) { return {df_add(a.re, df_neg(b.re)), df_add(a.im, df_neg(b.im))}; }
__device__ __forceinline__ dfc dfc_mul(dfc a, dff r) { return {df_mul(a.re, r), df_mul(a.im, r)}; }
__device__ __forceinline__ dfc dfc_mul(dfc a, dfc b) {
  return {df_add(df_mul(a.re, b.re), df_neg(df_mul(a.im, b.im))), df_add(df_mul(a.re, b.im), df_mul(a.im, b.re))};
}
__device__ __forceinline__ dfc dfc_of(cx<float> v) { return {{v.re, 0.f}, {v.im, 0.f}}; }
__device__ __forceinline__ dfc dfc_of(float4 v) { return {{v.x, v.y}, {v.z, v.w}}; }
__device__ __forceinline__ float4 dfc_pack(dfc v) { return make_float4(v.re.h, v.re.l, v.im.h, v.im.l); }
__host__ __device__ inline float4 dfc_split(double re, double im) {
  const float rh = (float)re, ih = (float)im;
  return make_float4(rh, (float)(re - (double)rh), ih, (float)(im - (double)ih));
}

// Near pair of the mixed precision: the closed-form singular parts enter
// through their frequency-independent test-point sums (precomputed per sweep
// in fp64, held in double-float: st6 = [sum w S0, sum w x S0, sum w y S0,
// sum w S1x, sum w S1y, sum w (x S1x + y S1y)]) times cA, cV; the smooth parts
// S_A, S_V - their 7 x 7 point evaluations and both sums - run in fp32; they
// join, and the 3x3 block is formed (pair_block_df), in double-float.
__device__ __forceinline__ void near_pass_df(int nrho, const TriData<float>& S32, const TriData<float>& A32, float dcx,
                                             float dcy, const float* xf, const float* tab32, dfc cA, dfc cV,
                                             const float2* st6, int lane, const TriDF& At, dfc (&Q)[3],
                                             dfc (&Px)[3], dfc (&Py)[3], dfc& IV, Bk bk) {
  float sq[7][2], sw[7];
#pragma unroll
  for (int l = 0; l < 7; ++l) {
    sq[l][0] = S32.q7[l][0];
    sq[l][1] = S32.q7[l][1];
    sw[l] = S32.w7[l];
  }
  cx<float> s0, sx, sy, t0, t1, t2, iv;  // the smooth parts' test-point sums
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    const float qx = A32.q7[k][0], qy = A32.q7[k][1], wk = A32.w7[k];
    const float rx = dcx + qx, ry = dcy + qy;
    cx<float> a0, ax, ay, v0;
#pragma unroll
    for (int l = 0; l < 7; ++l) {
      const float ddx = rx - sq[l][0], ddy = ry - sq[l][1];
      const float R = sqrtf(ddx * ddx + ddy * ddy);  // 0 for coincident points of a self pair
      cx<float> sa, sv;
      spline_av<float>(xf, xf, tab32, nrho, R, sa, sv, bk);
      const cx<float> saw = sa * sw[l];
      a0 += saw;
      ax += saw * sq[l][0];
      ay += saw * sq[l][1];
      v0 += sv * sw[l];
    }
    const float wx = wk * qx, wy = wk * qy;
    iv += v0 * wk;
    s0 += a0 * wk;
    sx += a0 * wx;
    sy += a0 * wy;
    t1 += ax * wk;
    t2 += ay * wk;
    t0 += ax * wx + ay * wy;
  }
  auto st = [&](int q) {
    const float2 v = st6[q * 32 + lane];
    return dff{v.x, v.y};
  };
  IV = dfc_add(dfc_mul(cV, st(0)), dfc_of(iv));
  const dfc S0 = dfc_add(dfc_mul(cA, st(0)), dfc_of(s0)), SX = dfc_add(dfc_mul(cA, st(1)), dfc_of(sx)),
            SY = dfc_add(dfc_mul(cA, st(2)), dfc_of(sy));
  const dfc T1 = dfc_add(dfc_mul(cA, st(3)), dfc_of(t1)), T2 = dfc_add(dfc_mul(cA, st(4)), dfc_of(t2)),
            T0 = dfc_add(dfc_mul(cA, st(5)), dfc_of(t0));
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const dff tx{At.vh[i][0], At.vl[i][0]}, ty{At.vh[i][1], At.vl[i][1]};
    Px[i] = dfc_sub(SX, dfc_mul(S0, tx));
    Py[i] = dfc_sub(SY, dfc_mul(S0, ty));
    Q[i] = dfc_sub(T0, dfc_add(dfc_mul(T1, tx), dfc_mul(T2, ty)));
  }
}

// pair_block (below) in double-float: the near pair's 3x3 block of the mixed fill
__device__ __forceinline__ void pair_block_df(const TriDF& Sd, const TriDF& At, dfc jwmu, dfc inv_jwe,
                                              const dfc (&Q)[3], const dfc (&Px)[3], const dfc (&Py)[3], dfc IV,
                                              dfc (&out)[3][3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const dfc ja = dfc_mul(jwmu, dff{At.cAh[i], At.cAl[i]}), jv = dfc_mul(inv_jwe, dff{At.cVh[i], At.cVl[i]});
    const dfc JQ = dfc_mul(ja, Q[i]), JPx = dfc_mul(ja, Px[i]), JPy = dfc_mul(ja, Py[i]), JV = dfc_mul(jv, IV);
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const dff bx{Sd.vh[j][0], Sd.vl[j][0]}, by{Sd.vh[j][1], Sd.vl[j][1]};
      const dfc ia = dfc_sub(JQ, dfc_add(dfc_mul(JPx, bx), dfc_mul(JPy, by)));
      out[i][j] = dfc_add(dfc_mul(ia, dff{Sd.cAh[j], Sd.cAl[j]}), dfc_mul(JV, dff{Sd.cVh[j], Sd.cVl[j]}));
    }
  }
}

// IA[i][j] = Q_i - (b_j - c_s) . P_i ; vals = jw mu cA cA IA + inv_jwe cV cV IV,
// with the test triangle's factors jw mu cA_i, inv_jwe cV_i applied to Q, P
// and IV once per i instead of once per (i, j)
template <class T>
__device__ __forceinline__ void pair_block(const TriData<T>& S, const T (&tcA)[3], const T (&tcV)[3], cx<T> jwmu,
                                           cx<T> inv_jwe, const cx<T> (&Q)[3], const cx<T> (&Px)[3],
                                           const cx<T> (&Py)[3], cx<T> IV, cx<T> (&out)[3][3]) {
  T scA[3], scV[3], bx[3], by[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    scA[j] = S.cA[j];
    scV[j] = S.cV[j];
    bx[j] = S.v[j][0];
    by[j] = S.v[j][1];
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const cx<T> ja = jwmu * tcA[i], jv = inv_jwe * tcV[i];
    const cx<T> JQ = ja * Q[i], JPx = ja * Px[i], JPy = ja * Py[i], JV = jv * IV;
#pragma unroll
    for (int j = 0; j < 3; ++j) out[i][j] = (JQ - (JPx * bx[j] + JPy * by[j])) * scA[j] + JV * scV[j];
  }
}

// FAR32 (T = double, the mixed precision): mid and far pairs (three- and
// one-point source rules) are evaluated in fp32 - interval search, spline,
// leading term, test-point sums and the 3x3 block - from fp32 copies of the
// tables and triangle data; near pairs keep their closed-form singular parts
// and the accumulation in fp64 with the smooth parts in fp32
// (near_pass_mixed). In the mixed path's error budget (S within 1e-5 of
// mom25d) the fp32 rounding moves S by ~1e-7.
//
// PASS (mixed precision): 1 = near pairs only, 2 = mid and far pairs only,
// two launches over the same work items, each built for two CTAs per SM
// (the fp64 fill's single pass needs ~240 registers a thread) and staging
// only the fp32 tables.
template <class T, bool FAR32, int PASS>
__global__ void __launch_bounds__(256, PASS != 0 ? 2 : 1) fill_tri_kernel(FillArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  const int L = a.nlev;
  const int n = a.nrho;
  // tables of the pairs (lt, ls): radii, then per source level (n-1) x 16
  // values [A, V]; FAR32 reads only the fp32 copies (radii and tables)
  T* xs = FAR32 ? nullptr : reinterpret_cast<T*>(smem_raw);
  T* tabs = FAR32 ? nullptr : xs + ((n + 3) & ~3);
  float* xf = FAR32 ? reinterpret_cast<float*>(smem_raw)
                    : reinterpret_cast<float*>(tabs + (size_t)L * (n - 1) * 16);  // radii rounded to fp32
  float* tabs32 = xf + ((n + 3) & ~3);  // FAR32: fp32 tables, same layout as tabs
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    if (!FAR32) xs[i] = a.rho[i];
    xf[i] = (float)a.rho[i];
  }
  Bk bk;
  if (FAR32 && a.nbk > 0) {
    uint16_t* bkt = reinterpret_cast<uint16_t*>(tabs32 + (size_t)L * (n - 1) * 16);
    __syncthreads();  // xf complete
    for (int j = threadIdx.x; j < a.nbk; j += blockDim.x) {
      const float rj = (float)j / a.bk_scale;
      int lo = 0, hi = n - 2;  // largest i <= n - 2 with xf[i] <= rj
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (xf[mid] <= rj) lo = mid; else hi = mid - 1;
      }
      bkt[j] = (uint16_t)lo;
    }
    bk.t = bkt;
    bk.scale = a.bk_scale;
    bk.nb = a.nbk;
  }  // the first work item's table load ends with a barrier
  int loaded = -1;
  // persistent grid: work items (test block, source chunk) handed out by a
  // counter, so that CTAs which start late (the SMs busy with the kernels of
  // concurrent sweeps) take fewer items
  __shared__ int next_item;
  const int nitems = a.nblocks * a.n_chunks;
  for (int item = blockIdx.x; item < nitems;) {
  const int blk = item / a.n_chunks, chunk = item % a.n_chunks;
  const int lt = a.block_level[blk];
  if (lt != loaded) {  // same for the whole CTA
    __syncthreads();
    for (int ls = 0; ls < L; ++ls) {
      const cx<T>* src = reinterpret_cast<const cx<T>*>(a.coef) + (size_t)(lt * L + ls) * (n - 1) * 12;
      T* dst = FAR32 ? nullptr : tabs + (size_t)ls * (n - 1) * 16;
      for (int e = threadIdx.x; e < (FAR32 ? 0 : (n - 1) * 8); e += blockDim.x) {
        int iv = e >> 3, r = e & 7, p = r >> 1, which = r & 1;  // power p, kernel A(0) / V(1)
        cx<T> v = src[((size_t)iv * 4 + p) * 3 + which];
        dst[(size_t)iv * 16 + p * 4 + which * 2] = v.re;
        dst[(size_t)iv * 16 + p * 4 + which * 2 + 1] = v.im;
      }
      if (FAR32) {
        const cx<float>* src32 = reinterpret_cast<const cx<float>*>(a.coef32) + (size_t)(lt * L + ls) * (n - 1) * 12;
        float* dst32 = tabs32 + (size_t)ls * (n - 1) * 16;
        for (int e = threadIdx.x; e < (n - 1) * 8; e += blockDim.x) {
          int iv = e >> 3, r = e & 7, p = r >> 1, which = r & 1;
          cx<float> v = src32[((size_t)iv * 4 + p) * 3 + which];
          dst32[(size_t)iv * 16 + p * 4 + which * 2] = v.re;
          dst32[(size_t)iv * 16 + p * 4 + which * 2 + 1] = v.im;
        }
      }
    }
    __syncthreads();
    loaded = lt;
  }

  const int t = a.block_tris[blk * 32 + lane];
  const bool active = t >= 0;
  const int tt = active ? t : a.block_tris[blk * 32];
  T tq[7][2], tw[7], tv[3][2], tcA[3], tcV[3];
  {
    const TriData<T>& A = a.td[tt];
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      tq[k][0] = A.q7[k][0];
      tq[k][1] = A.q7[k][1];
      tw[k] = A.w7[k];
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      tv[i][0] = A.v[i][0];
      tv[i][1] = A.v[i][1];
      tcA[i] = A.cA[i];
      tcV[i] = A.cV[i];
    }
  }
  const double tcx = a.cen[2 * tt], tcy = a.cen[2 * tt + 1];
  float4 tcd = make_float4(0.f, 0.f, 0.f, 0.f);
  if constexpr (FAR32) tcd = a.cen_df[tt];
  // mixed fill: the centroid difference to source s in fp32 from the
  // double-float centroids (the high parts' difference is exact for nearby
  // triangles, the low parts carry the rest): no fp64 operation per pair
  auto dcen = [&](int s, float& dx, float& dy) {
    const float4 sc = a.cen_df[s];
    dx = __fadd_rn(__fsub_rn(tcd.x, sc.x), __fsub_rn(tcd.y, sc.y));
    dy = __fadd_rn(__fsub_rn(tcd.z, sc.z), __fsub_rn(tcd.w, sc.w));
  };
  const int pad = active ? a.pad_pos[tt] : -1;
  const int64_t col0 = (int64_t)(blk * 32 + lane) * 3;

  const int s_begin = chunk * a.n_src_chunk;
  const int s_end = min(a.nt, s_begin + a.n_src_chunk);
  for (int s = s_begin + warp; s < s_end; s += nwarp) {
    int slot = -1;
    if constexpr (!FAR32) {
      if (a.cidx) {
        slot = a.cidx[(int64_t)blk * a.nt + s];
        if (slot == -1) continue;
      }
    }
    const int code = a.cls[(int64_t)blk * a.nt + s];
    if ((PASS == 1 && code < 0) || (PASS == 2 && code >= 0)) continue;  // the other pass's pair
    const int ls = a.tri_layer[s];
    if constexpr (FAR32 && PASS == 1) {
      // near pair of the mixed fill, in double-float
      float dcx, dcy;
      dcen(s, dcx, dcy);
      const TriDF& At = a.tddf[tt];
      dfc Q[3], Px[3], Py[3], IV, out[3][3];
      near_pass_df(n, a.td32[s], a.td32[tt], dcx, dcy, xf, tabs32 + (size_t)ls * (n - 1) * 16,
                   dfc_of(a.lead_df[lt * L + ls][0]), dfc_of(a.lead_df[lt * L + ls][1]), a.stat6 + (int64_t)code * 192,
                   lane, At, Q, Px, Py, IV, bk);
      pair_block_df(a.tddf[s], At, dfc_of(a.jwmu_df), dfc_of(a.inv_jwe_df), Q, Px, Py, IV, out);
      if (active && s == t && a.has_zs) {
        // conductor loss of the self pair: Zs x its precomputed factor
        const dfc zs = dfc_of(a.zs_df);
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) out[i][j] = dfc_add(out[i][j], dfc_mul(zs, dff{At.gzh[i][j], At.gzl[i][j]}));
      }
      if (active) {
        // [code][j][i][lane], the 32 lanes' words consecutive; in H32 a quiet
        // NaN whose payload is the code (kNearTag)
        float4* hn = a.Hn + (int64_t)code * 288 + lane;
        const cx<float> tag(__uint_as_float(kNearTag | (uint32_t)code), 0.f);
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          cx<float>* row = a.H32 + (int64_t)(3 * s + j) * a.ldh + col0;
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            hn[(j * 3 + i) * 32] = dfc_pack(out[i][j]);
            row[i] = tag;
          }
        }
        if (pad >= 0)
          a.IVpad[(int64_t)pad * a.nt + s] =
              cx<T>(T((double)IV.re.h + (double)IV.re.l), T((double)IV.im.h + (double)IV.im.l));
      }
      continue;
    }
    const TriData<T>& S = a.td[s];
    T dcx = T(0), dcy = T(0);
    float fx = 0.f, fy = 0.f;  // mixed fill: the difference in fp32 (dcen)
    if constexpr (FAR32) {
      dcen(s, fx, fy);
    } else {
      dcx = T(tcx - a.cen[2 * s]);
      dcy = T(tcy - a.cen[2 * s + 1]);
    }
    const T* tab = FAR32 ? nullptr : tabs + (size_t)ls * (n - 1) * 16;
    const cx<T> cA = a.lead[lt * L + ls][0], cV = a.lead[lt * L + ls][1];
    const T dz = a.dz[lt * L + ls];
    cx<T> Q[3], Px[3], Py[3], IV;
    if (code >= 0) {
      if constexpr (!FAR32)
        source_pass<T, 7, true>(n, S, dcx, dcy, tq, tw, xs, xf, tab, cA, cV, dz, a.stat + (int64_t)code * 672, lane,
                                Q, Px, Py, IV, tv);
    } else if (code == -1 && !FAR32) {
      source_pass<T, 3, false>(n, S, dcx, dcy, tq, tw, xs, xf, tab, cA, cV, dz, nullptr, lane, Q, Px, Py, IV, tv);
    }
    cx<T> out[3][3];
    if (FAR32 && code < 0) {
      // mid or far pair in fp32 (test data re-read from the fp32 copy, L1-resident)
      const TriData<float>& A32 = a.td32[tt];
      const TriData<float>& S32 = a.td32[s];
      float tq32[7][2], tw32[7], tv32[3][2], tcA32[3], tcV32[3];
#pragma unroll
      for (int k = 0; k < 7; ++k) {
        tq32[k][0] = A32.q7[k][0];
        tq32[k][1] = A32.q7[k][1];
        tw32[k] = A32.w7[k];
      }
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        tv32[i][0] = A32.v[i][0];
        tv32[i][1] = A32.v[i][1];
        tcA32[i] = A32.cA[i];
        tcV32[i] = A32.cV[i];
      }
      cx<float> Qf[3], Pxf[3], Pyf[3], IVf, outf[3][3];
      const float* tab32 = tabs32 + (size_t)ls * (n - 1) * 16;
      const cx<float> cA32 = a.lead32[lt * L + ls][0], cV32 = a.lead32[lt * L + ls][1];
      if (code == -1)
        source_pass<float, 3, false>(n, S32, fx, fy, tq32, tw32, xf, xf, tab32, cA32, cV32,
                                     a.dz32[lt * L + ls], nullptr, lane, Qf, Pxf, Pyf, IVf, tv32, bk);
      else
        source_pass<float, 1, false>(n, S32, fx, fy, tq32, tw32, xf, xf, tab32, cA32, cV32,
                                     a.dz32[lt * L + ls], nullptr, lane, Qf, Pxf, Pyf, IVf, tv32, bk);
      pair_block<float>(S32, tcA32, tcV32, a.jwmu32, a.inv_jwe32, Qf, Pxf, Pyf, IVf, outf);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) out[i][j] = cx<T>(outf[i][j]);
      IV = cx<T>(IVf);
    } else {
      if (code < -1)
        source_pass<T, 1, false>(n, S, dcx, dcy, tq, tw, xs, xf, tab, cA, cV, dz, nullptr, lane, Q, Px, Py, IV, tv);
      pair_block<T>(S, tcA, tcV, a.jwmu, a.inv_jwe, Q, Px, Py, IV, out);
    }
    if (PASS != 2 && active && s == t && (a.zs.re != T(0) || a.zs.im != T(0))) {
      // conductor loss: Zs Int_T (r - a_i).(r - a_j) dS cA_i cA_j
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          T gsum = T(0);
#pragma unroll
          for (int k = 0; k < 7; ++k)
            gsum += tw[k] * ((tq[k][0] - tv[i][0]) * (tq[k][0] - tv[j][0]) + (tq[k][1] - tv[i][1]) * (tq[k][1] - tv[j][1]));
          out[i][j] += a.zs * (gsum * tcA[i] * tcA[j]);
        }
    }
    if (active) {
      if (FAR32) {
        // mid / far pair: fp32 values, exactly as computed
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          cx<float>* row = a.H32 + (int64_t)(3 * s + j) * a.ldh + col0;
#pragma unroll
          for (int i = 0; i < 3; ++i) row[i] = cx<float>(float(out[i][j].re), float(out[i][j].im));
        }
      } else if (a.cidx) {
        if (slot >= 0) {
          cx<T>* hc = a.Hc + (int64_t)slot * 288 + lane;
#pragma unroll
          for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int i = 0; i < 3; ++i) hc[(j * 3 + i) * 32] = out[i][j];
        }
      } else {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          cx<T>* row = a.H + (int64_t)(3 * s + j) * a.ldh + col0;
          row[0] = out[0][j];
          row[1] = out[1][j];
          row[2] = out[2][j];
        }
      }
      if (pad >= 0) a.IVpad[(int64_t)pad * a.nt + s] = IV;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) next_item = (int)gridDim.x + atomicAdd(a.work_counter, 1);
  __syncthreads();
  item = next_item;
  }  // work items
}

// Z[m][n] = 0.5 (Zr[m][n] + Zr[n][m]), Zr[m][n] = sum over the two triangles
// t_m, local edges i_m of m (test) and t_n, j_n of n (source) of the
// half-basis value h(t_m, i_m; t_n, j_n), held in H at [3 t_n + j_n][3
// slot(t_m) + i_m] (the fp64 fill). SPLIT: Z itself is not stored but its
// double-float planes Zh = fl32(Z), Zl = fl32(Z - Zh) (rows nb apart) and the
// complex64 LU input (Zh, rows ldl apart).
// Each pair (m, n) of the upper triangle is formed once: one CTA per 32 x 32
// tile (tile row <= tile column) computes Z[m][n] and writes it to Z[n][m] as
// well through a shared-memory transpose (Z is symmetric by construction).
// The half-sum over h(test m, source n) is taken with the lanes along m and
// the one over h(test n, source m) with the lanes along n, so that both read
// runs of one row of H. Diagonal tiles form all their entries directly.
template <class T, class TO, bool SPLIT>
__global__ void __launch_bounds__(256) gather_sym_kernel(int nb, const cx<T>* __restrict__ H, int64_t ldh,
                                                         const int32_t* __restrict__ etri,
                                                         const int32_t* __restrict__ eloc,
                                                         const int32_t* __restrict__ tpos, cx<TO>* __restrict__ Z,
                                                         int64_t ldz, zf* __restrict__ Zh, zf* __restrict__ Zl,
                                                         zf* __restrict__ LU, int64_t ldl) {
  const int tm = blockIdx.y, tn = blockIdx.x;
  if (tm > tn) return;
  __shared__ cx<T> tile[32][33];
  __shared__ cx<T> s1t[32][33];  // s1t[n][m]: the half-sum over h(test m, source n)
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  auto store = [&](int m, int n, cx<T> z) {
    if constexpr (SPLIT) {
      const float hr = (float)z.re, hi = (float)z.im;
      const zf hv(hr, hi);
      Zh[(int64_t)m * nb + n] = hv;
      Zl[(int64_t)m * nb + n] = zf((float)(z.re - (double)hr), (float)(z.im - (double)hi));
      LU[(int64_t)m * ldl + n] = hv;
    } else {
      Z[(int64_t)m * ldz + n] = cx<TO>(z);
    }
  };
  auto rwg = [&](int e, int (&t)[2], int (&l)[2], int (&sl)[2]) {
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      t[a] = etri[2 * e + a];
      l[a] = eloc[2 * e + a];
      sl[a] = tpos[t[a]];
    }
  };
  auto h = [&](int sl, int i, int s, int j) { return H[(int64_t)(3 * s + j) * ldh + 3 * (int64_t)sl + i]; };
  {
    const int m = tm * 32 + tx;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int n = tn * 32 + ty + 8 * k;
      cx<T> s1;
      if (m < nb && n < nb) {
        int tma[2], lma[2], sma[2], tnb[2], lnb[2], snb[2];
        rwg(m, tma, lma, sma);
        rwg(n, tnb, lnb, snb);
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
          for (int b = 0; b < 2; ++b) s1 += h(sma[a], lma[a], tnb[b], lnb[b]);  // test m, source n
      }
      s1t[ty + 8 * k][tx] = s1;
    }
  }
  __syncthreads();
  const int nn = tn * 32 + tx;
  const bool nok = nn < nb;
  int tnb[2], lnb[2], snb[2];
  if (nok) rwg(nn, tnb, lnb, snb);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int m = tm * 32 + ty + 8 * k;
    cx<T> z;
    if (nok && m < nb) {
      int tma[2], lma[2], sma[2];
      rwg(m, tma, lma, sma);
      cx<T> s2;
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) s2 += h(snb[b], lnb[b], tma[a], lma[a]);  // test n, source m
      z = (s1t[tx][ty + 8 * k] + s2) * T(0.5);
      store(m, nn, z);
    }
    tile[ty + 8 * k][tx] = z;
  }
  if (tm == tn) return;  // uniform over the CTA
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int n2 = tn * 32 + ty + 8 * k, m2 = tm * 32 + tx;
    if (n2 < nb && m2 < nb) store(n2, m2, tile[tx][ty + 8 * k]);
  }
}

// Double-float sums on the fp32 pipes (the fp64 pipe of this GPU would bound
// the gather: ~26 fp64 operations per entry): a running fp32 sum h and its
// rounding errors (Knuth's two-sum) summed in l.
struct DF2 {
  float hr = 0.f, lr = 0.f, hi = 0.f, li = 0.f;  // re = hr + lr, im = hi + li
};
__device__ __forceinline__ void df_acc(float& h, float& l, float x) {
  const float s = h + x, z = s - h;
  l += (h - (s - z)) + (x - z);
  h = s;
}

// The same Z for the mixed fill: the mid / far pairs' h are complex64 in H32
// (exactly as computed, in fp32), the near pairs' are double-float in Hn at
// [code][j_n][i_m][lane of t_m], code = the pair's index among the near pairs,
// which H32 carries in a NaN at the pair's place (kNearTag). Sums in
// double-float (DF2), about 2^-46 relative. SPLIT writes Zh, Zl (the
// normalised double-float) and the LU input; else Z in complex128.
template <bool SPLIT>
__global__ void __launch_bounds__(256) gather_mix_kernel(int nb, const cx<float>* __restrict__ H32,
                                                         const float4* __restrict__ Hn, int64_t nnear, int64_t ldh,
                                                         const int32_t* __restrict__ etri,
                                                         const int32_t* __restrict__ eloc,
                                                         const int32_t* __restrict__ tpos, zd* __restrict__ Z,
                                                         int64_t ldz, zf* __restrict__ Zh, zf* __restrict__ Zl,
                                                         zf* __restrict__ LU, int64_t ldl) {
  const int tm = blockIdx.y, tn = blockIdx.x;
  if (tm > tn) return;
  __shared__ float4 tile[32][33];  // (Zh re, Zl re, Zh im, Zl im) of the transposed entries
  __shared__ float4 s1t[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  auto store = [&](int m, int n, float4 z) {
    if constexpr (SPLIT) {
      const zf hv(z.x, z.z);
      Zh[(int64_t)m * nb + n] = hv;
      Zl[(int64_t)m * nb + n] = zf(z.y, z.w);
      LU[(int64_t)m * ldl + n] = hv;
    } else {
      Z[(int64_t)m * ldz + n] = zd((double)z.x + (double)z.y, (double)z.z + (double)z.w);
    }
  };
  auto rwg = [&](int e, int (&t)[2], int (&l)[2], int (&sl)[2]) {
#pragma unroll
    for (int a = 0; a < 2; ++a) {
      t[a] = etri[2 * e + a];
      l[a] = eloc[2 * e + a];
      sl[a] = tpos[t[a]];
    }
  };
  // the scratch entry of h(test slot sl, local i; source s, local j)
  auto at = [&](int sl, int i, int s, int j) { return H32[(int64_t)(3 * s + j) * ldh + 3 * (int64_t)sl + i]; };
  // acc += that h, given the entry v read from H32 (a near pair's tag: its double-float value from Hn)
  auto add = [&](DF2& acc, cx<float> v, int sl, int i, int j) {
    const uint32_t u = __float_as_uint(v.re);
    if ((u & 0xFFC00000u) == kNearTag && (int64_t)(u & 0x3FFFFFu) < nnear) {
      const float4 w = Hn[(int64_t)(u & 0x3FFFFFu) * 288 + (j * 3 + i) * 32 + (sl & 31)];
      df_acc(acc.hr, acc.lr, w.x);
      acc.lr += w.y;
      df_acc(acc.hi, acc.li, w.z);
      acc.li += w.w;
    } else {
      df_acc(acc.hr, acc.lr, v.re);
      df_acc(acc.hi, acc.li, v.im);
    }
  };
  // the four rows' or columns' scratch entries are read before any is summed
  // (sixteen independent loads in flight per thread: the gather waits on
  // memory latency)
  {
    const int m = tm * 32 + tx;
    const bool mok = m < nb;
    int tma[2] = {0, 0}, lma[2] = {0, 0}, sma[2] = {0, 0};
    if (mok) rwg(m, tma, lma, sma);
    int t4[4][2], l4[4][2];
    bool ok[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int n = tn * 32 + ty + 8 * k;
      ok[k] = mok && n < nb;
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        t4[k][b] = ok[k] ? etri[2 * n + b] : 0;
        l4[k][b] = ok[k] ? eloc[2 * n + b] : 0;
      }
    }
    cx<float> v[4][2][2];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) v[k][a][b] = ok[k] ? at(sma[a], lma[a], t4[k][b], l4[k][b]) : cx<float>();
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      DF2 s1;
      if (ok[k])
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
          for (int b = 0; b < 2; ++b) add(s1, v[k][a][b], sma[a], lma[a], l4[k][b]);  // test m, source n
      s1t[ty + 8 * k][tx] = make_float4(s1.hr, s1.lr, s1.hi, s1.li);
    }
  }
  __syncthreads();
  const int nn = tn * 32 + tx;
  const bool nok = nn < nb;
  int tnb[2] = {0, 0}, lnb[2] = {0, 0}, snb[2] = {0, 0};
  if (nok) rwg(nn, tnb, lnb, snb);
  {
    int t4[4][2], l4[4][2];
    bool ok[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int m = tm * 32 + ty + 8 * k;
      ok[k] = nok && m < nb;
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        t4[k][a] = ok[k] ? etri[2 * m + a] : 0;
        l4[k][a] = ok[k] ? eloc[2 * m + a] : 0;
      }
    }
    cx<float> v[4][2][2];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) v[k][a][b] = ok[k] ? at(snb[b], lnb[b], t4[k][a], l4[k][a]) : cx<float>();
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int m = tm * 32 + ty + 8 * k;
      float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
      if (ok[k]) {
        const float4 a1 = s1t[tx][ty + 8 * k];
        DF2 s;
        s.hr = a1.x;
        s.lr = a1.y;
        s.hi = a1.z;
        s.li = a1.w;
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
          for (int b = 0; b < 2; ++b) add(s, v[k][a][b], snb[b], lnb[b], l4[k][a]);  // test n, source m
        // 0.5 (s1 + s2), normalised: Zh = fl32(h + l), Zl = the remainder
        const float hr = 0.5f * s.hr, lr = 0.5f * s.lr, hi = 0.5f * s.hi, li = 0.5f * s.li;
        const float zr = hr + lr, zi = hi + li;
        z = make_float4(zr, lr - (zr - hr), zi, li - (zi - hi));
        store(m, nn, z);
      }
      tile[ty + 8 * k][tx] = z;
    }
  }
  if (tm == tn) return;  // uniform over the CTA
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int n2 = tn * 32 + ty + 8 * k, m2 = tm * 32 + tx;
    if (n2 < nb && m2 < nb) store(n2, m2, tile[tx][ty + 8 * k]);
  }
}

// Via rows: Zvb[k][n] = inv_jwe sum_pad D[pad][k] sum_{T of n} cV IV(pad, T)
// (written to row nb+k and column nb+k).
template <class T, class TO>
__global__ void via_rows_kernel(int nb, int nv, int nt, const cx<T>* __restrict__ IVpad,
                                const int32_t* __restrict__ seg_pad_off, const int32_t* __restrict__ seg_pad,
                                const double* __restrict__ seg_pad_w, const int32_t* __restrict__ etri,
                                const int32_t* __restrict__ eloc, const TriData<T>* __restrict__ td, cx<T> inv_jwe,
                                cx<TO>* __restrict__ Z, int64_t ldz) {
  int nn = blockIdx.x * blockDim.x + threadIdx.x;
  int k = blockIdx.y;
  if (nn >= nb || k >= nv) return;
  int ta = etri[2 * nn], la = eloc[2 * nn], tb = etri[2 * nn + 1], lb = eloc[2 * nn + 1];
  T ca = td[ta].cV[la], cb = td[tb].cV[lb];
  cx<T> acc;
  for (int e = seg_pad_off[k]; e < seg_pad_off[k + 1]; ++e) {
    int p = seg_pad[e];
    cx<T> y = IVpad[(int64_t)p * nt + ta] * ca + IVpad[(int64_t)p * nt + tb] * cb;
    acc += y * T(seg_pad_w[e]);
  }
  cx<TO> z(inv_jwe * acc);
  Z[(int64_t)(nb + k) * ldz + nn] = z;
  Z[(int64_t)nn * ldz + nb + k] = z;
}

// The same rows for the compressed operator: ZxbT[i][k] = Zvb[k][perm[i]]
// (tree order of the RWG unknowns, the via index fastest).
__global__ void via_rows_tree_kernel(int nb, int nv, int nt, const zd* __restrict__ IVpad,
                                     const int32_t* __restrict__ seg_pad_off, const int32_t* __restrict__ seg_pad,
                                     const double* __restrict__ seg_pad_w, const int32_t* __restrict__ etri,
                                     const int32_t* __restrict__ eloc, const TriData<double>* __restrict__ td,
                                     zd inv_jwe, const int32_t* __restrict__ perm, zd* __restrict__ ZxbT) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  if (i >= nb || k >= nv) return;
  const int nn = perm[i];
  const int ta = etri[2 * nn], la = eloc[2 * nn], tb = etri[2 * nn + 1], lb = eloc[2 * nn + 1];
  const double ca = td[ta].cV[la], cb = td[tb].cV[lb];
  zd acc;
  for (int e = seg_pad_off[k]; e < seg_pad_off[k + 1]; ++e) {
    const int p = seg_pad[e];
    const zd y = IVpad[(int64_t)p * nt + ta] * ca + IVpad[(int64_t)p * nt + tb] * cb;
    acc += y * seg_pad_w[e];
  }
  ZxbT[(int64_t)i * nv + k] = inv_jwe * acc;
}

__device__ inline double filament_f(double s, double d) { return s * asinh(s / d) - sqrt(s * s + d * d); }

// Grover's partial mutual inductance of parallel z filaments [a1,a2], [b1,b2]
// at lateral distance d.
__device__ inline double filament_mutual_z(double a1, double a2, double b1, double b2, double d) {
  return kMu0 / (4.0 * kPi) *
         (filament_f(a2 - b1, d) - filament_f(a2 - b2, d) - filament_f(a1 - b1, d) + filament_f(a1 - b2, d));
}

// Via-via block (Engine/mom25d/solver.py:527-566 with the open-section case
// of via_impedance, 125-199): charge coupling through gV, removal of the
// Im gV(0) part of the segment end charges, quasi-static inductance of the
// segments and their ground images, via-wall loss.
template <class T, class TO>
__global__ void via_block_kernel(int nb, int nv, int nt, int L, const cx<T>* __restrict__ IVpad,
                                 const int32_t* __restrict__ pad_tris, const int32_t* __restrict__ seg_pad_off,
                                 const int32_t* __restrict__ seg_pad, const double* __restrict__ seg_pad_w,
                                 const int32_t* __restrict__ seg_end_lev, const double* __restrict__ seg_span,
                                 const double* __restrict__ seg_xy, const double* __restrict__ seg_drill,
                                 const double* __restrict__ im_gv0, double omega, zd zsv, double h_sec,
                                 cx<TO>* __restrict__ Z, int64_t ldz) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  int m = blockIdx.y;
  if (k >= nv || m >= nv) return;
  const zd inv_jwe = zd(1.0) / zd(0.0, omega * eps0());
  // charge part, both orders (the matrix is symmetrised)
  zd acc[2];
  for (int o = 0; o < 2; ++o) {
    int r = o == 0 ? k : m, c = o == 0 ? m : k;
    zd s(0.0);
    for (int e = seg_pad_off[r]; e < seg_pad_off[r + 1]; ++e)
      for (int f = seg_pad_off[c]; f < seg_pad_off[c + 1]; ++f) {
        cx<T> iv = IVpad[(int64_t)seg_pad[e] * nt + pad_tris[seg_pad[f]]];
        s += zd(double(iv.re), double(iv.im)) * (seg_pad_w[e] * seg_pad_w[f]);
      }
    // Im gV(0) of the end charges
    double im = 0.0;
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) {
        int la = seg_end_lev[2 * r + a], lb = seg_end_lev[2 * c + b];
        if (la < 0 || lb < 0) continue;
        double sa = a == 0 ? 1.0 : -1.0, sb = b == 0 ? 1.0 : -1.0;
        im += sa * sb * im_gv0[la * L + lb];
      }
    acc[o] = inv_jwe * s - inv_jwe * zd(0.0, im);
  }
  zd z = (acc[0] + acc[1]) * 0.5;
  // inductance of the vertical currents (+ images in the ground plane)
  double dx = seg_xy[2 * k] - seg_xy[2 * m], dy = seg_xy[2 * k + 1] - seg_xy[2 * m + 1];
  double rk = 0.5 * seg_drill[k], rm = 0.5 * seg_drill[m];
  double rho = sqrt(dx * dx + dy * dy);
  if (rho < 1e-12) rho = fmin(rk, rm);
  if (k == m) rho = rk;
  double p1 = fmin(fmax(seg_span[2 * k], 0.0), h_sec), p2 = fmin(fmax(seg_span[2 * k + 1], 0.0), h_sec);
  double q1 = fmin(fmax(seg_span[2 * m], 0.0), h_sec), q2 = fmin(fmax(seg_span[2 * m + 1], 0.0), h_sec);
  double Lkm = filament_mutual_z(p1, p2, q1, q2, rho) + filament_mutual_z(p1, p2, -q2, -q1, rho);
  double Lmk = filament_mutual_z(q1, q2, p1, p2, rho) + filament_mutual_z(q1, q2, -p2, -p1, rho);
  z += zd(0.0, omega) * (0.5 * (Lkm + Lmk));
  if (k == m && (zsv.re != 0.0 || zsv.im != 0.0)) {
    double len = seg_span[2 * k + 1] - seg_span[2 * k];
    z += zsv * (len / (kPi * seg_drill[k]));
  }
  Z[(int64_t)(nb + k) * ldz + nb + m] = cx<TO>(cx<T>(T(z.re), T(z.im)));
}

// Im gV at rho0 (0 between levels, 1e-6 h on a level) for every level pair.
__global__ void im_gv0_kernel(int L, int nrho, const double* __restrict__ rho, const zd* __restrict__ coef,
                              const zd* __restrict__ lead, const double* __restrict__ dzp, double h,
                              double* __restrict__ out) {
  int p = threadIdx.x;
  if (p >= L * L) return;
  double dz = dzp[p];
  double r = dz != 0.0 ? 0.0 : 1e-6 * h;
  int i = find_interval(rho, nrho, r);
  double dx = r - rho[i];
  const zd* c = coef + ((size_t)p * (nrho - 1) + i) * 12;
  zd v = c[3 * 3 + 1] + c[2 * 3 + 1] * dx + c[1 * 3 + 1] * (dx * dx) + c[0 * 3 + 1] * (dx * dx * dx);
  double R = sqrt(r * r + dz * dz);
  zd g = lead[p] / (4.0 * kPi * R) + v;
  out[p] = g.im;
}

// The fill's arguments shared by the dense and the listed fill: geometry,
// tables, constants; the scratch pointers are the caller's. smem: the
// kernel's dynamic shared memory (the tables).
template <class T>
static int fill_setup(m25_geom* geom, m25_greens* gr, zd zs, bool f32, FillArgs<T>& a, size_t& smem) {
  const int nt = geom->nt, nb = geom->nb, L = geom->nlev;
  const int nrho = gr->nrho;
  a.nt = nt;
  a.nb = nb;
  a.nlev = L;
  a.nblocks = geom->nblocks;
  a.td = std::is_same<T, double>::value ? reinterpret_cast<const TriData<T>*>(geom->td64)
                                        : reinterpret_cast<const TriData<T>*>(geom->td32);
  a.cen = geom->cen;
  a.cen_df = geom->cen_df;
  a.tri_layer = geom->tri_layer;
  a.block_tris = geom->block_tris;
  a.block_level = geom->block_level;
  a.cls = geom->cls;
  a.stat = std::is_same<T, double>::value ? reinterpret_cast<const T*>(geom->stat64)
                                          : reinterpret_cast<const T*>(geom->stat32);
  a.stat6 = geom->stat6;
  a.tddf = geom->tddf;
  a.pad_pos = geom->pad_pos;
  a.nrho = nrho;
  a.rho = std::is_same<T, double>::value ? reinterpret_cast<const T*>(gr->rho) : reinterpret_cast<const T*>(gr->rho32);
  a.coef = std::is_same<T, double>::value ? reinterpret_cast<const T*>(gr->coef)
                                          : reinterpret_cast<const T*>(gr->coef32);
  for (int p = 0; p < L * L; ++p) {
    zd ca = gr->lead_h[0 * L * L + p], cv = gr->lead_h[1 * L * L + p];
    a.lead[p][0] = cx<T>(T(ca.re), T(ca.im));
    a.lead[p][1] = cx<T>(T(cv.re), T(cv.im));
    a.dz[p] = T(gr->dz_h[p]);
  }
  const double omega = gr->omega;
  zd jwmu(0.0, omega * kMu0);
  zd inv_jwe = zd(1.0) / zd(0.0, omega * eps0());
  a.jwmu = cx<T>(T(jwmu.re), T(jwmu.im));
  a.inv_jwe = cx<T>(T(inv_jwe.re), T(inv_jwe.im));
  a.zs = cx<T>(T(zs.re), T(zs.im));
  a.td32 = geom->td32;
  a.coef32 = gr->coef32;
  for (int p = 0; p < L * L; ++p) {
    zd ca = gr->lead_h[0 * L * L + p], cv = gr->lead_h[1 * L * L + p];
    a.lead32[p][0] = cx<float>(float(ca.re), float(ca.im));
    a.lead32[p][1] = cx<float>(float(cv.re), float(cv.im));
    a.dz32[p] = float(gr->dz_h[p]);
  }
  a.jwmu32 = cx<float>(float(jwmu.re), float(jwmu.im));
  a.inv_jwe32 = cx<float>(float(inv_jwe.re), float(inv_jwe.im));
  for (int p = 0; p < L * L; ++p) {
    const zd ca = gr->lead_h[0 * L * L + p], cv = gr->lead_h[1 * L * L + p];
    a.lead_df[p][0] = dfc_split(ca.re, ca.im);
    a.lead_df[p][1] = dfc_split(cv.re, cv.im);
  }
  a.jwmu_df = dfc_split(jwmu.re, jwmu.im);
  a.zs_df = dfc_split(zs.re, zs.im);
  a.has_zs = zs.re != 0.0 || zs.im != 0.0;
  a.inv_jwe_df = dfc_split(inv_jwe.re, inv_jwe.im);
  // mixed fill: bucket index of the fp32 radii, buckets no wider than the
  // smallest radius step (at most 16384)
  a.nbk = 0;
  a.bk_scale = 0.f;
  if (f32) {
    const std::vector<double>& hr = gr->rho_h;
    float gap = INFINITY;
    for (int i = 0; i + 1 < nrho; ++i) gap = std::min(gap, (float)hr[i + 1] - (float)hr[i]);
    const float last = (float)hr[nrho - 1];
    if (gap > 0.f && last > 0.f) {
      a.nbk = std::min(16384, (int)std::ceil(last / gap) + 1);
      a.bk_scale = (float)a.nbk / last;
    }
  }
  // fp64 fill: both tables; mixed (f32): the fp32 radii and tables only (+ the bucket index)
  smem = f32 ? sizeof(float) * (((nrho + 3) & ~3) + (size_t)L * (nrho - 1) * 16) +
                   sizeof(uint16_t) * (((size_t)a.nbk + 7) & ~(size_t)7)
             : sizeof(T) * (((nrho + 3) & ~3) + (size_t)L * (nrho - 1) * 16) + sizeof(float) * ((nrho + 3) & ~3);
  if (smem > 220 * 1024) {
    set_error("m25_assemble: Green's tables too large for shared memory (reduce rho_max or levels)");
    return M25_ERR_VALUE;
  }
  return M25_OK;
}

// Stage 1 + 2 + 3 on the context's stream; Z is host or device memory.
template <class T>
int fill_driver(m25_ctx* ctx, m25_geom* geom, m25_greens* gr, zd zs, zd zsv, void* Zout, int64_t ldz, int where,
                bool far32, const FillSplit* split) {
  cudaStream_t st = ctx->stream;
  const int nt = geom->nt, nb = geom->nb, nv = geom->nv, L = geom->nlev, n = nb + nv;
  const int nrho = gr->nrho;
  const int64_t ldh = (int64_t)geom->nblocks * 96;
  int rc;
  // scratch: the half-basis values (fp64 fill: H, complex of T; mixed fill:
  // H32 for the mid / far pairs and Hn for the near pairs), the via pads'
  // charge integrals and Im gV(0)
  const bool f32 = far32 && std::is_same<T, double>::value;
  const size_t hbytes = f32 ? sizeof(cx<float>) * (size_t)3 * nt * ldh +
                                  sizeof(float4) * 288 * (size_t)std::max<int64_t>(geom->nnear, 1)
                            : sizeof(cx<T>) * (size_t)3 * nt * ldh;
  if ((rc = ctx->H.ensure(hbytes + sizeof(cx<T>) * (size_t)std::max(geom->npad, 1) * nt + sizeof(double) * 16)))
    return rc;
  if (f32 && geom->nnear > kMaxNearTagged) {
    set_error("m25_assemble: too many near pairs for the mixed fill's tagged scratch");
    return M25_ERR_VALUE;
  }
  cx<T>* H = f32 ? nullptr : ctx->H.as<cx<T>>();
  cx<float>* H32 = f32 ? ctx->H.as<cx<float>>() : nullptr;
  float4* Hn = f32 ? reinterpret_cast<float4*>(H32 + (size_t)3 * nt * ldh) : nullptr;
  cx<T>* IVpad = reinterpret_cast<cx<T>*>(ctx->H.as<char>() + hbytes);
  double* imgv = reinterpret_cast<double*>(IVpad + (size_t)std::max(geom->npad, 1) * nt);
  cx<T>* Z = static_cast<cx<T>*>(Zout);
  int64_t ldzd = ldz;
  if (where == M25_ON_HOST) {
    if ((rc = ctx->Zw.ensure(sizeof(cx<T>) * (size_t)n * n))) return rc;
    Z = ctx->Zw.as<cx<T>>();
    ldzd = n;
  }
  FillArgs<T> a;
  size_t smem = 0;
  if ((rc = fill_setup<T>(geom, gr, zs, f32, a, smem))) return rc;
  const double omega = gr->omega;
  a.H = H;
  a.ldh = ldh;
  a.H32 = H32;
  a.Hn = Hn;
  a.IVpad = IVpad;
  // the passes: fp64 = one kernel over all pairs; mixed = near, then mid / far
  using Kern = void (*)(FillArgs<T>);
  Kern kerns[2] = {f32 ? fill_tri_kernel<T, true, 1> : fill_tri_kernel<T, false, 0>, fill_tri_kernel<T, true, 2>};
  const int npass = f32 ? 2 : 1;
  int grids[2] = {0, 0};
  for (int k = 0; k < npass; ++k) {
    // one fixed limit for every call: the tables' size changes with the
    // frequency, and concurrent sweeps on other threads launch the same kernel
    M25_CUDA(cudaFuncSetAttribute(kerns[k], cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
    int occ = 1;
    M25_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kerns[k], 256, smem));
    grids[k] = std::max(1, occ) * ctx->num_sms;  // persistent grid: a whole number of waves
  }
  // ~16 work items per CTA of at least 64 sources each keep the tail short
  const int grid = grids[npass - 1];
  int nchunk = std::max(1, std::min((16 * grid + geom->nblocks - 1) / geom->nblocks, (nt + 63) / 64));
  a.n_src_chunk = (nt + nchunk - 1) / nchunk;
  nchunk = (nt + a.n_src_chunk - 1) / a.n_src_chunk;
  a.n_chunks = nchunk;
  if (nv) M25_CUDA(cudaMemsetAsync(IVpad, 0, sizeof(cx<T>) * (size_t)geom->npad * nt, st));
  if ((rc = ctx->sched.ensure(256))) return rc;
  M25_CUDA(cudaMemsetAsync(ctx->sched.p, 0, 2 * sizeof(int), st));
  {
    StageTimer tm(ctx, ST_FILL);
    for (int k = 0; k < npass; ++k) {
      a.work_counter = ctx->sched.as<int>() + k;
      kerns[k]<<<std::min(grids[k], geom->nblocks * nchunk), 256, smem, st>>>(a);
    }
  }
  M25_CHECK_LAUNCH();
  {
  StageTimer tm(ctx, ST_GATHER);
  const dim3 gtiles((nb + 31) / 32, (nb + 31) / 32);
  if (split) {
    if (nv || !std::is_same<T, double>::value) {
      set_error("m25_assemble: split output needs the mixed fill without vias");
      return M25_ERR_VALUE;
    }
    if constexpr (std::is_same<T, double>::value) {
      if (f32)
        gather_mix_kernel<true><<<gtiles, 256, 0, st>>>(nb, H32, Hn, geom->nnear, ldh, geom->edge_tri,
                                                        geom->edge_loc, geom->tpos, nullptr, 0, split->Zh, split->Zl,
                                                        split->LU, split->ldl);
      else
        gather_sym_kernel<T, T, true><<<gtiles, 256, 0, st>>>(nb, H, ldh, geom->edge_tri, geom->edge_loc,
                                                              geom->tpos, nullptr, 0, split->Zh, split->Zl, split->LU,
                                                              split->ldl);
    }
  } else if (f32) {
    if constexpr (std::is_same<T, double>::value)
      gather_mix_kernel<false><<<gtiles, 256, 0, st>>>(nb, H32, Hn, geom->nnear, ldh, geom->edge_tri, geom->edge_loc,
                                                       geom->tpos, Z, ldzd, nullptr, nullptr, nullptr, 0);
  } else {
    gather_sym_kernel<T, T, false><<<gtiles, 256, 0, st>>>(nb, H, ldh, geom->edge_tri, geom->edge_loc, geom->tpos, Z,
                                                           ldzd, nullptr, nullptr, nullptr, 0);
  }
  }
  M25_CHECK_LAUNCH();
  if (nv) {
    zd* lead_dev = reinterpret_cast<zd*>(imgv + 9);  // unused slot guard
    (void)lead_dev;
    // Im gV(rho0) per level pair from the double tables
    std::vector<zd> hv(L * L);
    std::vector<double> hdz(L * L);
    for (int p = 0; p < L * L; ++p) {
      hv[p] = gr->lead_h[1 * L * L + p];
      hdz[p] = gr->dz_h[p];
    }
    if ((rc = ctx->Dw.ensure(sizeof(zd) * 2 * kMaxLevSq))) return rc;
    zd* dv = ctx->Dw.as<zd>();
    double* ddz = reinterpret_cast<double*>(dv + kMaxLevSq);
    M25_CUDA(cudaMemcpyAsync(dv, hv.data(), sizeof(zd) * L * L, cudaMemcpyHostToDevice, st));
    M25_CUDA(cudaMemcpyAsync(ddz, hdz.data(), sizeof(double) * L * L, cudaMemcpyHostToDevice, st));
    StageTimer tm(ctx, ST_VIA);
    im_gv0_kernel<<<1, 32, 0, st>>>(L, nrho, gr->rho, reinterpret_cast<const zd*>(gr->coef), dv, ddz, gr->stack_h,
                                    imgv);
    via_rows_kernel<T, T><<<dim3((nb + 127) / 128, nv), 128, 0, st>>>(
        nb, nv, nt, IVpad, geom->seg_pad_off, geom->seg_pad, geom->seg_pad_w, geom->edge_tri, geom->edge_loc, a.td,
        a.inv_jwe, Z, ldzd);
    via_block_kernel<T, T><<<dim3((nv + 31) / 32, nv), 32, 0, st>>>(
        nb, nv, nt, L, IVpad, geom->pad_tris, geom->seg_pad_off, geom->seg_pad, geom->seg_pad_w, geom->seg_end_lev,
        geom->seg_span, geom->seg_xy, geom->seg_drill, imgv, omega, zsv, gr->stack_h, Z, ldzd);
    M25_CHECK_LAUNCH();
  }
  if (where == M25_ON_HOST) {
    M25_CUDA(cudaMemcpy2DAsync(Zout, sizeof(cx<T>) * ldz, Z, sizeof(cx<T>) * n, sizeof(cx<T>) * n, n,
                               cudaMemcpyDeviceToHost, st));
    M25_CUDA(cudaStreamSynchronize(st));
  }
  return M25_OK;
}

// The compressed operator's near field (fp64): the listed (test block,
// source triangle) pairs' half-basis values into Hc, the via pads' charge
// integrals, then the via unknowns' rows in tree order (ZxbT, nb x nv) and
// their block (Zxx, nv x nv). cidx: per (block, source) -1 skip, -2 compute
// for the pads only, >= 0 the slot in Hc.
int fill_listed(m25_ctx* ctx, m25_geom* geom, m25_greens* gr, zd zs, zd zsv, const int32_t* cidx, zd* Hc,
                const int32_t* perm, zd* ZxbT, zd* Zxx) {
  cudaStream_t st = ctx->stream;
  const int nt = geom->nt, nb = geom->nb, nv = geom->nv, L = geom->nlev;
  const int nrho = gr->nrho;
  int rc;
  if ((rc = ctx->H.ensure(sizeof(zd) * (size_t)std::max(geom->npad, 1) * nt + sizeof(double) * 16))) return rc;
  zd* IVpad = ctx->H.as<zd>();
  double* imgv = reinterpret_cast<double*>(IVpad + (size_t)std::max(geom->npad, 1) * nt);
  FillArgs<double> a;
  size_t smem = 0;
  if ((rc = fill_setup<double>(geom, gr, zs, false, a, smem))) return rc;
  a.H = nullptr;
  a.ldh = 0;
  a.H32 = nullptr;
  a.Hn = nullptr;
  a.IVpad = IVpad;
  a.cidx = cidx;
  a.Hc = Hc;
  auto kern = fill_tri_kernel<double, false, 0>;
  M25_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
  int occ = 1;
  M25_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, 256, smem));
  const int grid = std::max(1, occ) * ctx->num_sms;
  int nchunk = std::max(1, std::min((16 * grid + geom->nblocks - 1) / geom->nblocks, (nt + 63) / 64));
  a.n_src_chunk = (nt + nchunk - 1) / nchunk;
  nchunk = (nt + a.n_src_chunk - 1) / a.n_src_chunk;
  a.n_chunks = nchunk;
  if (nv) M25_CUDA(cudaMemsetAsync(IVpad, 0, sizeof(zd) * (size_t)geom->npad * nt, st));
  if ((rc = ctx->sched.ensure(256))) return rc;
  M25_CUDA(cudaMemsetAsync(ctx->sched.p, 0, 2 * sizeof(int), st));
  a.work_counter = ctx->sched.as<int>();
  {
    StageTimer tm(ctx, ST_FILL);
    kern<<<std::min(grid, geom->nblocks * nchunk), 256, smem, st>>>(a);
  }
  M25_CHECK_LAUNCH();
  if (nv) {
    std::vector<zd> hv(L * L);
    std::vector<double> hdz(L * L);
    for (int p = 0; p < L * L; ++p) {
      hv[p] = gr->lead_h[1 * L * L + p];
      hdz[p] = gr->dz_h[p];
    }
    if ((rc = ctx->Dw.ensure(sizeof(zd) * 2 * kMaxLevSq))) return rc;
    zd* dv = ctx->Dw.as<zd>();
    double* ddz = reinterpret_cast<double*>(dv + kMaxLevSq);
    M25_CUDA(cudaMemcpyAsync(dv, hv.data(), sizeof(zd) * L * L, cudaMemcpyHostToDevice, st));
    M25_CUDA(cudaMemcpyAsync(ddz, hdz.data(), sizeof(double) * L * L, cudaMemcpyHostToDevice, st));
    StageTimer tm(ctx, ST_VIA);
    im_gv0_kernel<<<1, 32, 0, st>>>(L, nrho, gr->rho, reinterpret_cast<const zd*>(gr->coef), dv, ddz, gr->stack_h,
                                    imgv);
    via_rows_tree_kernel<<<dim3((nb + 127) / 128, nv), 128, 0, st>>>(
        nb, nv, nt, IVpad, geom->seg_pad_off, geom->seg_pad, geom->seg_pad_w, geom->edge_tri, geom->edge_loc,
        geom->td64, a.inv_jwe, perm, ZxbT);
    // the via block: via_block_kernel writes Z[(nb + k) ldz + nb + m]; nb = 0, ldz = nv address Zxx
    via_block_kernel<double, double><<<dim3((nv + 31) / 32, nv), 32, 0, st>>>(
        0, nv, nt, L, IVpad, geom->pad_tris, geom->seg_pad_off, geom->seg_pad, geom->seg_pad_w, geom->seg_end_lev,
        geom->seg_span, geom->seg_xy, geom->seg_drill, imgv, gr->omega, zsv, gr->stack_h, Zxx, nv);
    M25_CHECK_LAUNCH();
  }
  return M25_OK;
}

template int fill_driver<double>(m25_ctx*, m25_geom*, m25_greens*, zd, zd, void*, int64_t, int, bool,
                                 const FillSplit*);
template int fill_driver<float>(m25_ctx*, m25_geom*, m25_greens*, zd, zd, void*, int64_t, int, bool,
                                const FillSplit*);

}  // namespace m25
