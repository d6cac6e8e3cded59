// Compressed MoM operator (H-matrix) and its preconditioned GMRES solve
// (Engine/mom25d/hmatrix.py:145-606). The host builds the cluster tree, the
// block partition and the index lists (mom25d_gb300/hmatrix.py); here:
//
//   near blocks  (near_kernel): the exact entries of the dense fill, summed
//                from the half-basis values of the listed fill (fill.cu,
//                fill_listed) and symmetrised 0.5 (Z + Z^T) like the dense
//                gather; stored row-major per leaf pair, both orders;
//   far blocks   (aca_kernel, one CTA per block): adaptive cross
//                approximation with partial pivoting and mom25d's stopping
//                rule on entries of the 3-point (or centroid) rule
//                (far_entry, hmatrix.py:322-353); far_dense_kernel for the
//                blocks kept as they are (side <= 64, or not low rank);
//   matvec       (far_t_kernel, rows_kernel, via_out_kernel): one warp per
//                low-rank term projects x, then one warp per row sums its
//                leaf's near blocks, far blocks as rows or as columns, and
//                its via columns, in double-float on the fp32 pipes; every
//                output entry has one writer (deterministic, no atomics);
//   precondition (diag_kernel, ginv_kernel, psolve_kernel): restricted
//                additive Schwarz over clusters of <= 256 unknowns extended
//                by their near-coupled leaves and the vias whose pads they
//                hold; the blocks scaled to a unit diagonal and inverted in
//                complex64 (Gauss-Jordan, partial pivoting), applied as one
//                batched GEMV that writes each block's own unknowns;
//   GMRES        on the symmetrically scaled system W Z W, W = |Z_ii|^-1/2
//                (the via unknowns' diagonal is ~1e10 times the RWG
//                unknowns'), restarted, flexible (right-preconditioned,
//                keeping each M^-1 v_j), classical Gram-Schmidt applied
//                twice, Givens rotations on the host.
// Vectors inside are in tree order: RWG unknowns perm[0..nb), then vias.
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "m25_internal.h"

// one far block: rows [r0, r0+m), columns [c0, c0+n) of the tree order
struct FarB {
  int r0, m, c0, n;
  int kind;   // 0 low rank (rank terms), 1 stored as it is
  int rank, kcap, cen;
  int64_t uv;     // U at pool + uv (kcap x m, term-major), V after it (kcap x n)
  int64_t dense;  // B at dense_pool + dense (m x n), B^T after it
  int64_t t;      // the matvec's V^T x (kcap) then U^T x (kcap) at t_df + t
  int64_t flag;   // ACA's used rows (m) then columns (n)
};

struct m25_hmat {
  m25_ctx* ctx = nullptr;
  m25_geom* geom = nullptr;
  int nb = 0, nv = 0, n = 0, nleaf = 0, nnear = 0, nfar = 0, npc = 0, npblk = 0;
  int64_t nkeys = 0;
  double tol = 1e-4;
  int kcap = 96;
  // host copies of the block lists
  std::vector<int32_t> far_h, cen_h, near_h;
  std::vector<int64_t> near_off_h;
  // device: structure
  int32_t *perm = nullptr, *lev = nullptr, *leaf_lo = nullptr, *near = nullptr, *ent = nullptr;
  int64_t *near_off = nullptr, *ent_off = nullptr, *keys = nullptr;
  int32_t *pblk = nullptr, *pc_gidx = nullptr, *pc_items = nullptr, *row_leaf = nullptr;
  int8_t* pc_own = nullptr;
  int32_t* self_near = nullptr;  // (nleaf) the near pair (a, a) of each leaf
  double* wsc = nullptr;         // (n) |Z_ii|^-1/2: the GMRES system's symmetric scaling
  m25::zd* sx = nullptr;         // (n) scratch of the scaled products
  int2* terms = nullptr;  // (block, term) of every low-rank term
  int nterm = 0;
  int64_t *pc_off = nullptr, *pc_doff = nullptr, *pc_item_off = nullptr;
  double* rules = nullptr;
  FarB* fb = nullptr;  // (nfar) device
  std::vector<FarB> fb_h;
  // device: values
  m25::zd *Zn = nullptr, *pool = nullptr, *ZxbT = nullptr, *Zxx = nullptr;
  m25::zf* D = nullptr;       // preconditioner blocks (their inverses, in place)
  uint8_t* flags = nullptr;   // ACA's used rows / columns
  int64_t near_entries = 0, uv_entries = 0, dense_entries = 0, t_entries = 0, flag_bytes = 0, d_entries = 0;
  int32_t *aca_ids = nullptr, *rank = nullptr, *status = nullptr, *dense_ids = nullptr;
  int naca = 0;
  m25::zd* dense_pool = nullptr;  // far blocks kept as they are (B, then B^T)
  float4* dense_df = nullptr;     // the same in double-float (the matvec's)
  float4 *Zn_df = nullptr, *pool_df = nullptr, *ZxbT_df = nullptr, *x_df = nullptr, *t_df = nullptr;
  size_t dense_bytes = 0;
  bool assembled = false;
  // GMRES workspace
  m25::zd *Vb = nullptr, *Zb = nullptr, *w = nullptr, *xv = nullptr, *zv = nullptr, *bv = nullptr, *hv = nullptr;
  double* nrm = nullptr;
  int restart_cap = 0;
  std::vector<void*> allocs;       // structure (freed on destroy)
  std::vector<void*> gm_allocs;    // GMRES workspace
  std::vector<void*> dense_allocs; // dense far pool (per assembly)
};

namespace m25 {
namespace {

constexpr int kRule = 40;  // values per basis: p (12), u (12), q (6), centroid p (4), u (4), q (2)

struct Tabs {
  const zd* coef;
  const double* rho;
  int nrho, L;
  zd cA[kMaxLevSq], cV[kMaxLevSq];
  double dz[kMaxLevSq];
  zd jwmu, inv_jwe;
};

__device__ __forceinline__ int interval(const double* __restrict__ x, int n, double r) {
  // scipy PPoly: x[i] <= r < x[i+1], clamped to the end intervals
  if (r < x[1]) return 0;
  if (r >= x[n - 2]) return n - 2;
  int lo = 1, hi = n - 2;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (r < x[mid]) hi = mid; else lo = mid;
  }
  return lo;
}

// Z between bases i and j (tree positions) by the 3-point rule on both sides
// or the centroid rule: jw mu sum (u_ik . u_jl) gA + 1/(jw eps) sum q_ik q_jl gV,
// g = c / (4 pi R) + S(rho) (Engine/mom25d/hmatrix.py:322-353, layered.py:199-206)
__device__ zd far_entry(const Tabs& t, const double* __restrict__ rules, const int32_t* __restrict__ lev, int i,
                        int j, int cen) {
  const double* A = rules + (int64_t)i * kRule;
  const double* B = rules + (int64_t)j * kRule;
  const int pair = lev[i] * t.L + lev[j];
  const zd cA = t.cA[pair], cV = t.cV[pair];
  const double dz = t.dz[pair];
  const int K = cen ? 2 : 6;
  const int op = cen ? 30 : 0, ou = cen ? 34 : 12, oq = cen ? 38 : 24;
  const zd* cf = t.coef + (int64_t)pair * (t.nrho - 1) * 12;
  zd za, zv;
  for (int k = 0; k < K; ++k) {
    const double ax = A[op + 2 * k], ay = A[op + 2 * k + 1];
    const double uax = A[ou + 2 * k], uay = A[ou + 2 * k + 1], qa = A[oq + k];
    for (int l = 0; l < K; ++l) {
      const double dx = ax - B[op + 2 * l], dy = ay - B[op + 2 * l + 1];
      const double rho = sqrt(dx * dx + dy * dy);
      const double R = sqrt(rho * rho + dz * dz);
      const int iv = interval(t.rho, t.nrho, rho);
      const double h = rho - t.rho[iv];
      const zd* c = cf + (int64_t)iv * 12;
      const zd sa = c[9] + c[6] * h + c[3] * (h * h) + c[0] * (h * h * h);
      const zd sv = c[10] + c[7] * h + c[4] * (h * h) + c[1] * (h * h * h);
      const double inv = 1.0 / (4.0 * kPi * R);
      const zd gA = cA * inv + sa, gV = cV * inv + sv;
      za += gA * (uax * B[ou + 2 * l] + uay * B[ou + 2 * l + 1]);
      zv += gV * (qa * B[oq + l]);
    }
  }
  return t.jwmu * za + t.inv_jwe * zv;
}

// -------------------------------------------------------------- reductions
__device__ __forceinline__ zd warp_sum(zd v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    v.re += __shfl_xor_sync(0xffffffffu, v.re, o);
    v.im += __shfl_xor_sync(0xffffffffu, v.im, o);
  }
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// largest value (ties: smallest index) over a CTA of blockDim.x <= 1024 threads; every thread gets it
__device__ void block_argmax(double& v, int& idx, double* sv, int* si) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const double ov = __shfl_xor_sync(0xffffffffu, v, o);
    const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
    if (ov > v || (ov == v && oi < idx)) {
      v = ov;
      idx = oi;
    }
  }
  __syncthreads();
  if (lane == 0) {
    sv[wid] = v;
    si[wid] = idx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    for (int k = 1; k < nw; ++k)
      if (sv[k] > sv[0] || (sv[k] == sv[0] && si[k] < si[0])) {
        sv[0] = sv[k];
        si[0] = si[k];
      }
  }
  __syncthreads();
  v = sv[0];
  idx = si[0];
}

__device__ double block_sum(double v, double* sv) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sv[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    double s = 0.0;
    for (int k = 0; k < nw; ++k) s += sv[k];
    sv[0] = s;
  }
  __syncthreads();
  v = sv[0];
  return v;
}

__device__ zd block_sum(zd v, double* sv) {
  const double re = block_sum(v.re, sv);
  const double im = block_sum(v.im, sv);
  return zd(re, im);
}

// ------------------------------------------------------------ near field
__global__ void cidx_pad_kernel(const int32_t* __restrict__ pblk, int npblk, int nt, int32_t* __restrict__ cidx) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (s < nt && b < npblk) cidx[(int64_t)pblk[b] * nt + s] = -2;
}

__global__ void cidx_keys_kernel(const int64_t* __restrict__ keys, int64_t nkeys, int32_t* __restrict__ cidx) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q < nkeys) cidx[keys[q]] = (int32_t)q;
}

// Z[m][n] = 0.5 (Zr[m][n] + Zr[n][m]) over the leaf pair's block, Zr[m][n] =
// sum of the half-basis values h(test t_m, i_m; source t_n, j_n), held at
// Hc[cidx[block(t_m), t_n]][j_n][i_m][lane(t_m)]
__global__ void near_kernel(const int32_t* __restrict__ near, const int64_t* __restrict__ noff,
                            const int32_t* __restrict__ perm, const int32_t* __restrict__ etri,
                            const int32_t* __restrict__ eloc, const int32_t* __restrict__ tpos,
                            const int32_t* __restrict__ cidx, int nt, const zd* __restrict__ Hc, zd* __restrict__ Zn,
                            int* __restrict__ err) {
  const int p = blockIdx.x;
  const int a0 = near[4 * p], am = near[4 * p + 1], b0 = near[4 * p + 2], bn = near[4 * p + 3];
  auto h = [&](int t, int it, int s, int js) -> zd {
    const int sl = tpos[t];
    const int slot = cidx[(int64_t)(sl >> 5) * nt + s];
    if (slot < 0) {
      atomicOr(err, 1);
      return zd();
    }
    return Hc[(int64_t)slot * 288 + (js * 3 + it) * 32 + (sl & 31)];
  };
  for (int e = threadIdx.x; e < am * bn; e += blockDim.x) {
    const int i = e / bn, j = e - i * bn;
    const int m = perm[a0 + i], n = perm[b0 + j];
    zd s1, s2;
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b) {
        const int tm = etri[2 * m + a], lm = eloc[2 * m + a], tn = etri[2 * n + b], ln = eloc[2 * n + b];
        s1 += h(tm, lm, tn, ln);
        s2 += h(tn, ln, tm, lm);
      }
    Zn[noff[p] + e] = (s1 + s2) * 0.5;
  }
}

// --------------------------------------------------------------- far field
__global__ void __launch_bounds__(256) far_dense_kernel(Tabs t, const double* __restrict__ rules,
                                                        const int32_t* __restrict__ lev,
                                                        const FarB* __restrict__ fb, const int32_t* __restrict__ ids,
                                                        zd* __restrict__ dpool) {
  const FarB F = fb[ids[blockIdx.x]];
  zd* B = dpool + F.dense;
  zd* BT = B + (int64_t)F.m * F.n;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i = wid; i < F.m; i += nw)  // one warp per row, the lanes along it
    for (int j = lane; j < F.n; j += 32) {
      const zd z = far_entry(t, rules, lev, F.r0 + i, F.c0 + j, F.cen);
      B[(int64_t)i * F.n + j] = z;
      BT[(int64_t)j * F.m + i] = z;
    }
}

// Adaptive cross approximation with partial pivoting (Engine/mom25d/
// hmatrix.py:100-136): block ~ U V^T, terms added until |u| |v| <= tol x the
// Frobenius norm of the sum so far. rank[b] = terms, status[b] = 0 low rank,
// 1 keep the block as it is (not low rank within kmax = min(m, n) / 3
// iterations, or more than kcap terms).
__global__ void __launch_bounds__(256) aca_kernel(Tabs t, const double* __restrict__ rules,
                                                  const int32_t* __restrict__ lev, const FarB* __restrict__ fb,
                                                  const int32_t* __restrict__ ids, zd* __restrict__ pool,
                                                  uint8_t* __restrict__ flags, double tol, int32_t* __restrict__ rank,
                                                  int32_t* __restrict__ status) {
  __shared__ double sv[32];
  __shared__ int si[32];
  const FarB F = fb[ids[blockIdx.x]];
  const int m = F.m, n = F.n, tid = threadIdx.x;
  zd* U = pool + F.uv;
  zd* V = U + (int64_t)F.kcap * m;
  uint8_t* used_r = flags + F.flag;
  uint8_t* used_c = used_r + m;
  const int kmax = max(2, min(m, n) / 3);
  int i = 0, k = 0, st = 1;
  double fro2 = 0.0;
  for (int it = 0; it < kmax; ++it) {
    if (k >= F.kcap) {  // no room for another term: keep the block as it is
      st = 1;
      break;
    }
    zd* Vk = V + (int64_t)k * n;
    // the residual's row i
    double best = -1.0;
    int bj = 0x7fffffff;
    for (int j = tid; j < n; j += blockDim.x) {
      zd z = far_entry(t, rules, lev, F.r0 + i, F.c0 + j, F.cen);
      for (int l = 0; l < k; ++l) z -= V[(int64_t)l * n + j] * U[(int64_t)l * m + i];
      Vk[j] = z;
      const double a = used_c[j] ? 0.0 : cabs(z);
      if (a > best) {
        best = a;
        bj = j;
      }
    }
    __syncthreads();
    if (tid == 0) used_r[i] = 1;
    block_argmax(best, bj, sv, si);
    if (!(best > 0.0) || bj >= n) {  // a zero row (or no finite entry): take the first unused row instead
      int fr = 0x7fffffff;
      for (int r = tid; r < m; r += blockDim.x)
        if (!used_r[r]) {
          fr = r;
          break;
        }
      double dummy = -(double)fr;
      block_argmax(dummy, fr, sv, si);
      if (fr == 0x7fffffff) {
        st = 0;
        break;
      }
      i = fr;
      continue;
    }
    const zd piv = Vk[bj];
    __syncthreads();
    double nv2 = 0.0;
    for (int j = tid; j < n; j += blockDim.x) {
      const zd v = Vk[j] / piv;
      Vk[j] = v;
      nv2 += norm2(v);
    }
    // the residual's column bj
    zd* Uk = U + (int64_t)k * m;
    double nu2 = 0.0;
    for (int r = tid; r < m; r += blockDim.x) {
      zd z = far_entry(t, rules, lev, F.r0 + r, F.c0 + bj, F.cen);
      for (int l = 0; l < k; ++l) z -= U[(int64_t)l * m + r] * V[(int64_t)l * n + bj];
      Uk[r] = z;
      nu2 += norm2(z);
    }
    nv2 = block_sum(nv2, sv);
    nu2 = block_sum(nu2, sv);
    if (tid == 0) used_c[bj] = 1;
    // cross terms 2 sum_l |(u_k^H u_l)(v_k^H v_l)|, one warp per earlier term
    double cross = 0.0;
    if (k > 0) {
      const int lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
      for (int l = wid; l < k; l += nw) {
        zd d1, d2;
        for (int r = lane; r < m; r += 32) d1 += conj(Uk[r]) * U[(int64_t)l * m + r];
        for (int j = lane; j < n; j += 32) d2 += conj(Vk[j]) * V[(int64_t)l * n + j];
        d1 = warp_sum(d1);
        d2 = warp_sum(d2);
        if (lane == 0) cross += cabs(d1 * d2);
      }
      cross = block_sum(cross, sv);
    }
    fro2 += 2.0 * cross + nu2 * nv2;
    ++k;
    if (sqrt(nu2 * nv2) <= tol * sqrt(fro2)) {
      st = 0;
      break;
    }
    // next row: the largest entry of the new column among the unused rows
    double cb = -1.0;
    int ci = 0x7fffffff;
    for (int r = tid; r < m; r += blockDim.x) {
      const double a = used_r[r] ? 0.0 : cabs(Uk[r]);
      if (a > cb) {
        cb = a;
        ci = r;
      }
    }
    block_argmax(cb, ci, sv, si);
    if (!(cb > 0.0) || ci >= m) {
      st = 0;
      break;
    }
    i = ci;
  }
  if (tid == 0) {
    rank[blockIdx.x] = k;
    status[blockIdx.x] = st;
  }
}

// ------------------------------------------------------------------ matvec
// The matvec sums in double-float on the fp32 pipes (GB300 issues fp64 at
// 1/64 of the fp32 rate; the fp64 form of these sums kept the fp64 pipe 86 %
// busy): the operator and x are held as (hi, lo) fp32 pairs per real and
// imaginary part (float4: re h, re l, im h, im l), products are exact to
// fp32 x fp32 by FMA plus the low parts' cross terms, running sums by
// Knuth's two-sum (~2^-48 relative). Warp results are combined in fp64.
__device__ __forceinline__ float4 df_split(zd z) {
  const float rh = (float)z.re, ih = (float)z.im;
  return make_float4(rh, (float)(z.re - (double)rh), ih, (float)(z.im - (double)ih));
}

__global__ void df_split_kernel(const zd* __restrict__ src, float4* __restrict__ dst, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = df_split(src[i]);
}

struct DfAcc {
  float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
};

__device__ __forceinline__ void two_sum(float& h, float& l, float x) {
  const float s = __fadd_rn(h, x), z = __fsub_rn(s, h);
  l = __fadd_rn(l, __fadd_rn(__fsub_rn(h, __fsub_rn(s, z)), __fsub_rn(x, z)));
  h = s;
}

// p + e = a b for double-float reals a = (ah, al), b = (bh, bl)
__device__ __forceinline__ float two_prod(float ah, float al, float bh, float bl, float& e) {
  const float p = __fmul_rn(ah, bh);
  e = __fadd_rn(fmaf(ah, bh, -p), __fadd_rn(__fmul_rn(ah, bl), __fmul_rn(al, bh)));
  return p;
}

// acc += a b (complex, double-float)
__device__ __forceinline__ void df_cmac(DfAcc& acc, float4 a, float4 b) {
  float e1, e2, e3, e4;
  const float p1 = two_prod(a.x, a.y, b.x, b.y, e1);  // ar br
  const float p2 = two_prod(a.z, a.w, b.z, b.w, e2);  // ai bi
  const float p3 = two_prod(a.x, a.y, b.z, b.w, e3);  // ar bi
  const float p4 = two_prod(a.z, a.w, b.x, b.y, e4);  // ai br
  two_sum(acc.rh, acc.rl, p1);
  two_sum(acc.rh, acc.rl, -p2);
  acc.rl = __fadd_rn(acc.rl, __fsub_rn(e1, e2));
  two_sum(acc.ih, acc.il, p3);
  two_sum(acc.ih, acc.il, p4);
  acc.il = __fadd_rn(acc.il, __fadd_rn(e3, e4));
}

__device__ __forceinline__ zd df_value(const DfAcc& a) {
  return zd((double)a.rh + (double)a.rl, (double)a.ih + (double)a.il);
}

// per term l of a low-rank far block: V_l^T x[C] and U_l^T x[R], one warp per (block, term)
__global__ void far_t_kernel(const int2* __restrict__ terms, int nterm, const FarB* __restrict__ fb,
                             const float4* __restrict__ pool, const float4* __restrict__ x,
                             float4* __restrict__ tpool) {
  const int lane = threadIdx.x & 31;
  const int q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (q >= nterm) return;
  const int2 bt = terms[q];
  const FarB F = fb[bt.x];
  const int l = bt.y;
  const float4* U = pool + F.uv + (int64_t)l * F.m;
  const float4* V = pool + F.uv + (int64_t)F.kcap * F.m + (int64_t)l * F.n;
  DfAcc a1, a2;
  for (int j = lane; j < F.n; j += 32) df_cmac(a1, V[j], x[F.c0 + j]);
  for (int r = lane; r < F.m; r += 32) df_cmac(a2, U[r], x[F.r0 + r]);
  const zd d1 = warp_sum(df_value(a1)), d2 = warp_sum(df_value(a2));
  if (lane == 0) {
    tpool[F.t + l] = df_split(d1);
    tpool[F.t + F.kcap + l] = df_split(d2);
  }
}

// y (tree order, RWG rows), one warp per row: the items of the row's leaf
__global__ void __launch_bounds__(256) rows_kernel(const int32_t* __restrict__ row_leaf,
                                                   const int32_t* __restrict__ leaf_lo,
                                                   const int64_t* __restrict__ ent_off,
                                                   const int32_t* __restrict__ ent, const int32_t* __restrict__ near,
                                                   const int64_t* __restrict__ noff, const float4* __restrict__ Zn,
                                                   const FarB* __restrict__ fb, const float4* __restrict__ pool,
                                                   const float4* __restrict__ dpool, const float4* __restrict__ tpool,
                                                   const float4* __restrict__ ZxbT, int nb, int nv,
                                                   const float4* __restrict__ x, zd* __restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= nb) return;
  const int leaf = row_leaf[r];
  const int lo = leaf_lo[leaf];
  const int64_t e0 = ent_off[leaf], e1 = ent_off[leaf + 1];
  DfAcc acc;
  for (int64_t e = e0; e < e1; ++e) {
    const int type = ent[4 * e], id = ent[4 * e + 1], off = ent[4 * e + 2];
    if (type == 0) {
      const int a0 = near[4 * id], b0 = near[4 * id + 2], bn = near[4 * id + 3];
      const float4* row = Zn + noff[id] + (int64_t)(r - a0) * bn;
      for (int j = lane; j < bn; j += 32) df_cmac(acc, row[j], x[b0 + j]);
      continue;
    }
    const FarB F = fb[id];
    const int q = off + (r - lo);  // row of the block (type 1) or of its transpose (type 2)
    if (F.kind == 0) {
      const float4* U = pool + F.uv;
      const float4* V = U + (int64_t)F.kcap * F.m;
      if (type == 1)
        for (int l = lane; l < F.rank; l += 32) df_cmac(acc, U[(int64_t)l * F.m + q], tpool[F.t + l]);
      else
        for (int l = lane; l < F.rank; l += 32) df_cmac(acc, V[(int64_t)l * F.n + q], tpool[F.t + F.kcap + l]);
    } else {
      const float4* B = dpool + F.dense;
      if (type == 1) {
        const float4* row = B + (int64_t)q * F.n;
        for (int j = lane; j < F.n; j += 32) df_cmac(acc, row[j], x[F.c0 + j]);
      } else {
        const float4* row = B + (int64_t)F.m * F.n + (int64_t)q * F.m;
        for (int j = lane; j < F.m; j += 32) df_cmac(acc, row[j], x[F.r0 + j]);
      }
    }
  }
  for (int v = lane; v < nv; v += 32) df_cmac(acc, ZxbT[(int64_t)r * nv + v], x[nb + v]);
  const zd a = warp_sum(df_value(acc));
  if (lane == 0) y[r] = a;
}

// y of the via unknowns: Zvb x_b + Zvv x_v, one CTA per via row
__global__ void via_out_kernel(int nb, int nv, const zd* __restrict__ ZxbT, const zd* __restrict__ Zxx,
                               const zd* __restrict__ x, zd* __restrict__ y) {
  __shared__ double sv[32];
  const int v = blockIdx.x;
  zd acc;
  for (int r = threadIdx.x; r < nb; r += blockDim.x) acc += ZxbT[(int64_t)r * nv + v] * x[r];
  for (int u = threadIdx.x; u < nv; u += blockDim.x) acc += Zxx[(int64_t)v * nv + u] * x[nb + u];
  acc = block_sum(acc, sv);
  if (threadIdx.x == 0) y[nb + v] = acc;
}

__global__ void perm_in_kernel(int nb, int n, const int32_t* __restrict__ perm, const zd* __restrict__ x,
                               zd* __restrict__ xt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) xt[i] = i < nb ? x[perm[i]] : x[i];
}

__global__ void perm_out_kernel(int nb, int n, const int32_t* __restrict__ perm, const zd* __restrict__ yt,
                                zd* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i < nb ? perm[i] : i] = yt[i];
}

// ---------------------------------------------------------- preconditioner
// Block k (restricted additive Schwarz) holds S_k unknowns, pc_gidx[pc_off[k]
// ..]: whole leaves (tree positions) then vias (nb + via); it writes those
// with pc_own set. Its matrix is the compressed operator on those unknowns.

// block k's matrix (complex64, row-major S x S): per (row leaf, column leaf)
// pair the near block or the far block (as rows or as its transpose), then
// the via rows / columns
__global__ void diag_kernel(const int64_t* __restrict__ pc_off, const int32_t* __restrict__ gidx,
                            const int64_t* __restrict__ item_off, const int32_t* __restrict__ items,
                            const int64_t* __restrict__ doff, int nb, int nv, int nnear,
                            const int32_t* __restrict__ leaf_lo, const int64_t* __restrict__ noff,
                            const zd* __restrict__ Zn, const FarB* __restrict__ fb, const zd* __restrict__ pool,
                            const zd* __restrict__ dpool, const zd* __restrict__ ZxbT, const zd* __restrict__ Zxx,
                            zf* __restrict__ D) {
  __shared__ int nr;
  const int k = blockIdx.x;
  const int64_t g0 = pc_off[k];
  const int S = (int)(pc_off[k + 1] - g0);
  zf* Dk = D + doff[k];
  if (threadIdx.x == 0) nr = 0;
  __syncthreads();
  int mine = 0;
  for (int t = threadIdx.x; t < S; t += blockDim.x) mine += gidx[g0 + t] < nb;
  atomicAdd(&nr, mine);
  for (int64_t e = threadIdx.x; e < (int64_t)S * S; e += blockDim.x) Dk[e] = zf(0.f, 0.f);
  __syncthreads();
  const int R = nr;  // RWG unknowns first, then the vias
  for (int64_t it = item_off[k]; it < item_off[k + 1]; ++it) {
    const int src = items[5 * it], li = items[5 * it + 1], lj = items[5 * it + 2];
    const int lr0 = items[5 * it + 3], lc0 = items[5 * it + 4];
    const int a0 = leaf_lo[li], am = leaf_lo[li + 1] - a0, b0 = leaf_lo[lj], bn = leaf_lo[lj + 1] - b0;
    if (src < nnear) {
      const zd* blk = Zn + noff[src];
      for (int e = threadIdx.x; e < am * bn; e += blockDim.x) {
        const int ii = e / bn, jj = e - ii * bn;
        Dk[(int64_t)(lr0 + ii) * S + lc0 + jj] = zf(blk[e]);
      }
      continue;
    }
    const int f = (src - nnear) >> 1, o = (src - nnear) & 1;
    const FarB F = fb[f];
    const zd* U = F.kind == 0 ? pool + F.uv : nullptr;
    const zd* V = F.kind == 0 ? U + (int64_t)F.kcap * F.m : nullptr;
    for (int e = threadIdx.x; e < am * bn; e += blockDim.x) {
      const int ii = e / bn, jj = e - ii * bn;
      zf z(0.f, 0.f);
      if (o == 0) {  // rows in R, columns in C
        const int ir = a0 - F.r0 + ii, jc = b0 - F.c0 + jj;
        if (F.kind == 0)
          for (int l = 0; l < F.rank; ++l) z += zf(U[(int64_t)l * F.m + ir]) * zf(V[(int64_t)l * F.n + jc]);
        else
          z = zf(dpool[F.dense + (int64_t)ir * F.n + jc]);
      } else {  // rows in C, columns in R: the transpose
        const int ic = a0 - F.c0 + ii, jr = b0 - F.r0 + jj;
        if (F.kind == 0)
          for (int l = 0; l < F.rank; ++l) z += zf(V[(int64_t)l * F.n + ic]) * zf(U[(int64_t)l * F.m + jr]);
        else
          z = zf(dpool[F.dense + (int64_t)jr * F.n + ic]);
      }
      Dk[(int64_t)(lr0 + ii) * S + lc0 + jj] = z;
    }
  }
  const int nvk = S - R;
  for (int e = threadIdx.x; e < R * nvk; e += blockDim.x) {  // RWG x via (Z is symmetric)
    const int t = e / nvk, a = e - t * nvk;
    const zf z(ZxbT[(int64_t)gidx[g0 + t] * nv + (gidx[g0 + R + a] - nb)]);
    Dk[(int64_t)t * S + R + a] = z;
    Dk[(int64_t)(R + a) * S + t] = z;
  }
  for (int e = threadIdx.x; e < nvk * nvk; e += blockDim.x) {  // via x via
    const int a = e / nvk, b = e - a * nvk;
    Dk[(int64_t)(R + a) * S + R + b] = zf(Zxx[(int64_t)(gidx[g0 + R + a] - nb) * nv + (gidx[g0 + R + b] - nb)]);
  }
}

// In-place inversion of each diagonal block (one CTA per block, complex64:
// the flexible GMRES below keeps M^-1 v_j, so the preconditioner need not be
// exact). The block is first scaled symmetrically to a unit diagonal,
// D' = W D W with W = diag(|D_ii|^-1/2) (the via rows and the RWG rows
// differ by many orders of magnitude), then inverted by Gauss-Jordan
// elimination with partial pivoting (a zero pivot is replaced by 1: the
// block then preconditions less), the row interchanges undone on the
// columns, and D^-1 = W D'^-1 W stored in place.
__device__ __forceinline__ float fabs1(zf a) { return fabsf(a.re) + fabsf(a.im); }

__global__ void __launch_bounds__(1024) ginv_kernel(const int64_t* __restrict__ pc_off, const int64_t* __restrict__ doff,
                                                   zf* __restrict__ D) {
  __shared__ double sv[32];
  __shared__ int si[32];
  __shared__ int pv[1024];
  __shared__ float w[1024];
  __shared__ zf fcol[1024];
  const int k = blockIdx.x;
  const int S = (int)(pc_off[k + 1] - pc_off[k]);
  zf* A = D + doff[k];
  for (int i = threadIdx.x; i < S; i += blockDim.x) {
    const zf a = A[(int64_t)i * S + i];
    const float m = hypotf(a.re, a.im);
    w[i] = m > 0.f ? rsqrtf(m) : 1.f;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int r = wid; r < S; r += nw)
    for (int j = lane; j < S; j += 32) A[(int64_t)r * S + j] = A[(int64_t)r * S + j] * (w[r] * w[j]);
  __syncthreads();
  for (int c = 0; c < S; ++c) {
    double best = -1.0;
    int bi = 0x7fffffff;
    for (int r = c + threadIdx.x; r < S; r += blockDim.x) {
      const double a = fabs1(A[(int64_t)r * S + c]);
      if (a > best) {
        best = a;
        bi = r;
      }
    }
    block_argmax(best, bi, sv, si);
    if (bi < c || bi >= S) {
      bi = c;
      best = 0.0;
    }
    if (threadIdx.x == 0) pv[c] = bi;
    if (bi != c)
      for (int j = threadIdx.x; j < S; j += blockDim.x) {
        const zf t0 = A[(int64_t)c * S + j];
        A[(int64_t)c * S + j] = A[(int64_t)bi * S + j];
        A[(int64_t)bi * S + j] = t0;
      }
    __syncthreads();
    const zf d = best > 0.0 ? zf(1.f, 0.f) / A[(int64_t)c * S + c] : zf(1.f, 0.f);
    __syncthreads();
    for (int j = threadIdx.x; j < S; j += blockDim.x)
      A[(int64_t)c * S + j] = j == c ? d : A[(int64_t)c * S + j] * d;
    for (int r = threadIdx.x; r < S; r += blockDim.x) fcol[r] = A[(int64_t)r * S + c];
    __syncthreads();
    for (int r = wid; r < S; r += nw) {  // one warp per row, the lanes along it
      if (r == c) continue;
      const zf f = fcol[r];
      zf* Ar = A + (int64_t)r * S;
      const zf* Ac = A + (int64_t)c * S;
      for (int j = lane; j < S; j += 32) Ar[j] = j == c ? -(f * d) : Ar[j] - f * Ac[j];
    }
    __syncthreads();
  }
  for (int c = S - 1; c >= 0; --c) {
    const int p = pv[c];
    if (p != c)
      for (int r = threadIdx.x; r < S; r += blockDim.x) {
        const zf t0 = A[(int64_t)r * S + c];
        A[(int64_t)r * S + c] = A[(int64_t)r * S + p];
        A[(int64_t)r * S + p] = t0;
      }
    __syncthreads();
  }
  for (int r = wid; r < S; r += nw)
    for (int j = lane; j < S; j += 32) A[(int64_t)r * S + j] = A[(int64_t)r * S + j] * (w[r] * w[j]);
}

// out = D_k^-1 in on the unknowns block k owns (complex64 inverse, fp32 sums), one warp per row
__global__ void __launch_bounds__(256) psolve_kernel(const int64_t* __restrict__ pc_off, const int32_t* __restrict__ gidx,
                                                     const int8_t* __restrict__ own, const int64_t* __restrict__ doff,
                                                     const zf* __restrict__ D, const zd* __restrict__ in,
                                                     zd* __restrict__ out) {
  __shared__ zf xs[1024];
  const int k = blockIdx.x;
  const int64_t g0 = pc_off[k];
  const int S = (int)(pc_off[k + 1] - g0);
  const zf* A = D + doff[k];
  for (int i = threadIdx.x; i < S; i += blockDim.x) xs[i] = zf(in[gidx[g0 + i]]);
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int r = wid; r < S; r += nw) {
    if (!own[g0 + r]) continue;
    zf acc(0.f, 0.f);
    const zf* row = A + (int64_t)r * S;
    for (int j = lane; j < S; j += 32) acc += row[j] * xs[j];
    const zd a = warp_sum(zd(double(acc.re), double(acc.im)));
    if (lane == 0) out[gidx[g0 + r]] = a;
  }
}

// ------------------------------------------------------------------ GMRES
// h[l] = V_l^H w, one CTA per basis vector
__global__ void dots_kernel(const zd* __restrict__ V, int64_t ldv, int n, const zd* __restrict__ w, zd* __restrict__ h) {
  __shared__ double sv[32];
  const int l = blockIdx.x;
  zd acc;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += conj(V[(int64_t)l * ldv + i]) * w[i];
  acc = block_sum(acc, sv);
  if (threadIdx.x == 0) h[l] = acc;
}

// w += sign * sum_l V_l c[l]
__global__ void combine_kernel(zd* __restrict__ w, const zd* __restrict__ V, int64_t ldv, int nvec, int n,
                               const zd* __restrict__ c, double sign) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  zd acc;
  for (int l = 0; l < nvec; ++l) acc += V[(int64_t)l * ldv + i] * c[l];
  w[i] += acc * sign;
}

__global__ void norm_kernel(const zd* __restrict__ w, int n, double* __restrict__ out) {
  __shared__ double sv[32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += norm2(w[i]);
  acc = block_sum(acc, sv);
  if (threadIdx.x == 0) *out = sqrt(acc);
}

__global__ void scale_kernel(zd* __restrict__ dst, const zd* __restrict__ src, int n, double s) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i] * s;
}

// dst = a - b
__global__ void sub_kernel(zd* __restrict__ dst, const zd* __restrict__ a, const zd* __restrict__ b, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = a[i] - b[i];
}

template <class T>
int dalloc(std::vector<void*>& list, T** p, size_t count) {
  return alloc(list, reinterpret_cast<void**>(p), sizeof(T) * std::max<size_t>(count, 1));
}

Tabs make_tabs(m25_greens* gr) {
  Tabs t;
  t.coef = reinterpret_cast<const zd*>(gr->coef);
  t.rho = gr->rho;
  t.nrho = gr->nrho;
  t.L = gr->nlev;
  const int L = gr->nlev;
  for (int p = 0; p < L * L; ++p) {
    t.cA[p] = gr->lead_h[p];
    t.cV[p] = gr->lead_h[L * L + p];
    t.dz[p] = gr->dz_h[p];
  }
  t.jwmu = zd(0.0, gr->omega * kMu0);
  t.inv_jwe = zd(1.0) / zd(0.0, gr->omega * eps0());
  return t;
}

}  // namespace

// w_i = |Z_ii|^-1/2 from the leaves' own near blocks and the via block
__global__ void wscale_kernel(int nb, int n, int nv, const int32_t* __restrict__ row_leaf,
                              const int32_t* __restrict__ self_near, const int32_t* __restrict__ near,
                              const int64_t* __restrict__ noff, const zd* __restrict__ Zn, const zd* __restrict__ Zxx,
                              double* __restrict__ w) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  zd d;
  if (r < nb) {
    const int p = self_near[row_leaf[r]];
    const int a0 = near[4 * p], bn = near[4 * p + 3];
    d = Zn[noff[p] + (int64_t)(r - a0) * bn + (r - a0)];
  } else {
    d = Zxx[(int64_t)(r - nb) * nv + (r - nb)];
  }
  const double a = cabs(d);
  w[r] = a > 0.0 ? 1.0 / sqrt(a) : 1.0;
}

// dst = src w (inv: src / w)
__global__ void vscale_kernel(zd* __restrict__ dst, const zd* __restrict__ src, const double* __restrict__ w, int n,
                              int inv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = inv ? src[i] / w[i] : src[i] * w[i];
}

namespace {

// y = A x, tree order, device vectors
int apply(m25_hmat* h, const zd* x, zd* y) {
  cudaStream_t st = h->ctx->stream;
  df_split_kernel<<<(h->n + 255) / 256, 256, 0, st>>>(x, h->x_df, h->n);
  if (h->nterm) far_t_kernel<<<(h->nterm + 7) / 8, 256, 0, st>>>(h->terms, h->nterm, h->fb, h->pool_df, h->x_df, h->t_df);
  rows_kernel<<<(h->nb + 7) / 8, 256, 0, st>>>(h->row_leaf, h->leaf_lo, h->ent_off, h->ent, h->near, h->near_off,
                                               h->Zn_df, h->fb, h->pool_df, h->dense_df, h->t_df, h->ZxbT_df, h->nb,
                                               h->nv, h->x_df, y);
  if (h->nv) via_out_kernel<<<h->nv, 256, 0, st>>>(h->nb, h->nv, h->ZxbT, h->Zxx, x, y);
  M25_CHECK_LAUNCH();
  return M25_OK;
}

int precond(m25_hmat* h, const zd* in, zd* out) {
  psolve_kernel<<<h->npc, 256, 0, h->ctx->stream>>>(h->pc_off, h->pc_gidx, h->pc_own, h->pc_doff, h->D, in, out);
  M25_CHECK_LAUNCH();
  return M25_OK;
}

// the scaled system W A W: y = W A (W x)
int sapply(m25_hmat* h, const zd* x, zd* y) {
  cudaStream_t st = h->ctx->stream;
  const int g = (h->n + 255) / 256;
  vscale_kernel<<<g, 256, 0, st>>>(h->sx, x, h->wsc, h->n, 0);
  int rc = apply(h, h->sx, y);
  if (rc) return rc;
  vscale_kernel<<<g, 256, 0, st>>>(y, y, h->wsc, h->n, 0);
  M25_CHECK_LAUNCH();
  return M25_OK;
}

// its preconditioner W^-1 M^-1 W^-1
int sprecond(m25_hmat* h, const zd* in, zd* out) {
  cudaStream_t st = h->ctx->stream;
  const int g = (h->n + 255) / 256;
  vscale_kernel<<<g, 256, 0, st>>>(h->sx, in, h->wsc, h->n, 1);
  int rc = precond(h, h->sx, out);
  if (rc) return rc;
  vscale_kernel<<<g, 256, 0, st>>>(out, out, h->wsc, h->n, 1);
  M25_CHECK_LAUNCH();
  return M25_OK;
}

}  // namespace
}  // namespace m25

using namespace m25;

extern "C" int m25_hmat_create(m25_ctx* ctx, m25_geom* geom, const m25_hmat_desc* d, m25_hmat** out) {
  if (!ctx || !geom || !d || !out) {
    set_error("m25_hmat_create: null argument");
    return M25_ERR_VALUE;
  }
  if (d->nb != geom->nb || d->nv != geom->nv || d->nb < 2 || d->nleaf < 1 || d->nnear < 1 || d->npc < 1 ||
      d->nfar < 0 || d->nkeys < 1 || d->kcap < 2 || !(d->tol > 0.0)) {
    set_error("m25_hmat_create: bad sizes");
    return M25_ERR_VALUE;
  }
  if (d->nv > 1024) {
    set_error("m25_hmat_create: more than 1024 via unknowns");
    return M25_ERR_VALUE;
  }
  m25_hmat* h = new m25_hmat();
  h->ctx = ctx;
  h->geom = geom;
  h->nb = d->nb;
  h->nv = d->nv;
  h->n = d->nb + d->nv;
  h->nleaf = d->nleaf;
  h->nnear = d->nnear;
  h->nfar = d->nfar;
  h->npc = d->npc;
  h->npblk = d->npblk;
  h->nkeys = d->nkeys;
  h->tol = d->tol;
  h->kcap = d->kcap;
  cudaStream_t st = ctx->stream;
  int rc = M25_OK;
  auto fail = [&](int r) {
    free_all(h->allocs);
    delete h;
    return r;
  };
  // the near pairs' storage, both orders
  h->near_h.assign(d->near, d->near + 4 * (size_t)d->nnear);
  h->near_off_h.resize(d->nnear + 1);
  h->near_off_h[0] = 0;
  for (int p = 0; p < d->nnear; ++p) {
    const int a0 = h->near_h[4 * p], am = h->near_h[4 * p + 1], b0 = h->near_h[4 * p + 2], bn = h->near_h[4 * p + 3];
    if (am <= 0 || bn <= 0 || a0 < 0 || b0 < 0 || a0 + am > d->nb || b0 + bn > d->nb) return fail((set_error("m25_hmat_create: bad near pair"), M25_ERR_VALUE));
    h->near_off_h[p + 1] = h->near_off_h[p] + (int64_t)am * bn;
  }
  h->near_entries = h->near_off_h[d->nnear];
  // far blocks: ACA storage for blocks with both sides > 64, else stored as they are
  h->fb_h.resize(d->nfar);
  int64_t uv = 0, tt = 0, fl = 0;
  for (int f = 0; f < d->nfar; ++f) {
    FarB& F = h->fb_h[f];
    F.r0 = d->far[4 * f];
    F.m = d->far[4 * f + 1];
    F.c0 = d->far[4 * f + 2];
    F.n = d->far[4 * f + 3];
    if (F.m <= 0 || F.n <= 0 || F.r0 < 0 || F.c0 < 0 || F.r0 + F.m > d->nb || F.c0 + F.n > d->nb)
      return fail((set_error("m25_hmat_create: bad far block"), M25_ERR_VALUE));
    F.cen = d->far_cen[f];
    F.rank = 0;
    F.dense = -1;
    if (std::min(F.m, F.n) > 64) {
      F.kind = 0;
      F.kcap = std::min(std::max(2, std::min(F.m, F.n) / 3), d->kcap);
      F.uv = uv;
      uv += (int64_t)F.kcap * (F.m + F.n);
      F.t = tt;
      tt += 2 * (int64_t)F.kcap;
      F.flag = fl;
      fl += F.m + F.n;
      ++h->naca;
    } else {
      F.kind = 1;
      F.kcap = 0;
      F.uv = -1;
      F.t = -1;
      F.flag = -1;
    }
  }
  h->uv_entries = uv;
  h->t_entries = tt;
  h->flag_bytes = fl;
  // preconditioner blocks
  std::vector<int64_t> doff(d->npc + 1, 0);
  {
    if (d->pc_off[0] != 0 || d->pc_item_off[0] != 0)
      return fail((set_error("m25_hmat_create: bad preconditioner offsets"), M25_ERR_VALUE));
    std::vector<int> owned(h->n, 0);
    std::vector<int32_t> lsz(d->nleaf);
    for (int l = 0; l < d->nleaf; ++l) lsz[l] = d->leaf_lo[l + 1] - d->leaf_lo[l];
    for (int k = 0; k < d->npc; ++k) {
      const int64_t S = d->pc_off[k + 1] - d->pc_off[k];
      if (S <= 0 || S > 1024 || d->pc_item_off[k + 1] < d->pc_item_off[k])
        return fail((set_error("m25_hmat_create: bad preconditioner block"), M25_ERR_VALUE));
      bool vias = false;
      for (int64_t t = d->pc_off[k]; t < d->pc_off[k + 1]; ++t) {
        const int g = d->pc_gidx[t];
        if (g < 0 || g >= h->n || (vias && g < d->nb))
          return fail((set_error("m25_hmat_create: bad preconditioner unknown"), M25_ERR_VALUE));
        vias = vias || g >= d->nb;
        if (d->pc_own[t]) ++owned[g];
      }
      for (int64_t e = d->pc_item_off[k]; e < d->pc_item_off[k + 1]; ++e) {
        const int32_t* it = d->pc_items + 5 * e;
        const int src = it[0], li = it[1], lj = it[2], lr0 = it[3], lc0 = it[4];
        if (li < 0 || li >= d->nleaf || lj < 0 || lj >= d->nleaf || src < 0 || src >= d->nnear + 2 * d->nfar ||
            lr0 < 0 || lc0 < 0 || lr0 + lsz[li] > S || lc0 + lsz[lj] > S)
          return fail((set_error("m25_hmat_create: bad preconditioner item"), M25_ERR_VALUE));
        const int a0 = d->leaf_lo[li], b0 = d->leaf_lo[lj];
        bool ok;
        if (src < d->nnear) {
          const int32_t* q = d->near + 4 * src;
          ok = q[0] == a0 && q[1] == lsz[li] && q[2] == b0 && q[3] == lsz[lj];
        } else {
          const int f = (src - d->nnear) >> 1, o = (src - d->nnear) & 1;
          const int32_t* q = d->far + 4 * f;
          const int rr0 = o ? q[2] : q[0], rm = o ? q[3] : q[1], cc0 = o ? q[0] : q[2], cn = o ? q[1] : q[3];
          ok = a0 >= rr0 && a0 + lsz[li] <= rr0 + rm && b0 >= cc0 && b0 + lsz[lj] <= cc0 + cn;
        }
        if (!ok) return fail((set_error("m25_hmat_create: a preconditioner item outside its source block"), M25_ERR_VALUE));
      }
      doff[k + 1] = doff[k] + S * S;
    }
    for (int g = 0; g < h->n; ++g)
      if (owned[g] != 1) return fail((set_error("m25_hmat_create: an unknown not owned by exactly one block"), M25_ERR_VALUE));
  }
  h->d_entries = doff[d->npc];
  const int64_t nent = d->ent_off[d->nleaf];
  const int64_t nitems = d->pc_item_off[d->npc];
  const int64_t npcu = d->pc_off[d->npc];
#define TRY(x)                 \
  do {                         \
    if ((rc = (x))) return fail(rc); \
  } while (0)
  TRY(dalloc(h->allocs, &h->perm, d->nb));
  TRY(dalloc(h->allocs, &h->rules, (size_t)d->nb * kRule));
  TRY(dalloc(h->allocs, &h->lev, d->nb));
  TRY(dalloc(h->allocs, &h->leaf_lo, d->nleaf + 1));
  TRY(dalloc(h->allocs, &h->row_leaf, d->nb));
  TRY(dalloc(h->allocs, &h->self_near, d->nleaf));
  TRY(dalloc(h->allocs, &h->wsc, h->n));
  TRY(dalloc(h->allocs, &h->Zn_df, h->near_entries));
  TRY(dalloc(h->allocs, &h->pool_df, uv));
  TRY(dalloc(h->allocs, &h->ZxbT_df, (size_t)d->nb * std::max(d->nv, 1)));
  TRY(dalloc(h->allocs, &h->x_df, h->n));
  TRY(dalloc(h->allocs, &h->t_df, tt));
  TRY(dalloc(h->allocs, &h->sx, h->n));
  TRY(dalloc(h->allocs, &h->near, 4 * (size_t)d->nnear));
  TRY(dalloc(h->allocs, &h->near_off, d->nnear + 1));
  TRY(dalloc(h->allocs, &h->ent_off, d->nleaf + 1));
  TRY(dalloc(h->allocs, &h->ent, 4 * (size_t)nent));
  TRY(dalloc(h->allocs, &h->keys, d->nkeys));
  TRY(dalloc(h->allocs, &h->pblk, d->npblk));
  TRY(dalloc(h->allocs, &h->pc_off, d->npc + 1));
  TRY(dalloc(h->allocs, &h->pc_gidx, npcu));
  TRY(dalloc(h->allocs, &h->pc_own, npcu));
  TRY(dalloc(h->allocs, &h->pc_item_off, d->npc + 1));
  TRY(dalloc(h->allocs, &h->pc_items, 5 * (size_t)nitems));
  TRY(dalloc(h->allocs, &h->pc_doff, d->npc + 1));
  TRY(dalloc(h->allocs, &h->fb, d->nfar));
  TRY(dalloc(h->allocs, &h->Zn, h->near_entries));
  TRY(dalloc(h->allocs, &h->pool, uv));
  TRY(dalloc(h->allocs, &h->terms, std::max<int64_t>(tt / 2, 1)));
  TRY(dalloc(h->allocs, &h->flags, fl));
  TRY(dalloc(h->allocs, &h->ZxbT, (size_t)d->nb * std::max(d->nv, 1)));
  TRY(dalloc(h->allocs, &h->Zxx, (size_t)std::max(d->nv, 1) * std::max(d->nv, 1)));
  TRY(dalloc(h->allocs, &h->D, h->d_entries));
  TRY(dalloc(h->allocs, &h->aca_ids, std::max(h->naca, 1)));
  TRY(dalloc(h->allocs, &h->rank, std::max(h->naca, 1)));
  TRY(dalloc(h->allocs, &h->status, std::max(h->naca, 1)));
  TRY(dalloc(h->allocs, &h->dense_ids, std::max(d->nfar, 1)));
#undef TRY
  auto up = [&](void* dst, const void* src, size_t bytes) -> int {
    if (bytes) M25_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
    return M25_OK;
  };
  std::vector<int32_t> row_leaf(d->nb);
  for (int k = 0; k < d->nleaf; ++k) {
    if (d->leaf_lo[k + 1] <= d->leaf_lo[k]) return fail((set_error("m25_hmat_create: empty leaf"), M25_ERR_VALUE));
    for (int r = d->leaf_lo[k]; r < d->leaf_lo[k + 1] && r < d->nb; ++r) row_leaf[r] = k;
  }
  std::vector<int32_t> self_near(d->nleaf, -1);
  for (int p = 0; p < d->nnear; ++p)
    if (d->near[4 * p] == d->near[4 * p + 2]) {
      const int k = row_leaf[d->near[4 * p]];
      if (d->leaf_lo[k] == d->near[4 * p]) self_near[k] = p;
    }
  for (int k = 0; k < d->nleaf; ++k)
    if (self_near[k] < 0) return fail((set_error("m25_hmat_create: a leaf without its own near block"), M25_ERR_VALUE));
  std::vector<int32_t> aca;
  for (int f = 0; f < d->nfar; ++f)
    if (h->fb_h[f].kind == 0) aca.push_back(f);
  if ((rc = up(h->perm, d->perm, sizeof(int32_t) * d->nb)) || (rc = up(h->rules, d->rules, sizeof(double) * d->nb * kRule)) ||
      (rc = up(h->lev, d->lev, sizeof(int32_t) * d->nb)) ||
      (rc = up(h->leaf_lo, d->leaf_lo, sizeof(int32_t) * (d->nleaf + 1))) ||
      (rc = up(h->row_leaf, row_leaf.data(), sizeof(int32_t) * d->nb)) ||
      (rc = up(h->self_near, self_near.data(), sizeof(int32_t) * d->nleaf)) ||
      (rc = up(h->near, d->near, sizeof(int32_t) * 4 * d->nnear)) ||
      (rc = up(h->near_off, h->near_off_h.data(), sizeof(int64_t) * (d->nnear + 1))) ||
      (rc = up(h->ent_off, d->ent_off, sizeof(int64_t) * (d->nleaf + 1))) ||
      (rc = up(h->ent, d->ent, sizeof(int32_t) * 4 * nent)) ||
      (rc = up(h->keys, d->keys, sizeof(int64_t) * d->nkeys)) ||
      (rc = up(h->pblk, d->pblk, sizeof(int32_t) * d->npblk)) ||
      (rc = up(h->pc_off, d->pc_off, sizeof(int64_t) * (d->npc + 1))) ||
      (rc = up(h->pc_gidx, d->pc_gidx, sizeof(int32_t) * npcu)) ||
      (rc = up(h->pc_own, d->pc_own, sizeof(int8_t) * npcu)) ||
      (rc = up(h->pc_item_off, d->pc_item_off, sizeof(int64_t) * (d->npc + 1))) ||
      (rc = up(h->pc_items, d->pc_items, sizeof(int32_t) * 5 * nitems)) ||
      (rc = up(h->pc_doff, doff.data(), sizeof(int64_t) * (d->npc + 1))) ||
      (rc = up(h->aca_ids, aca.data(), sizeof(int32_t) * aca.size())))
    return fail(rc);
  // index checks of the lists the kernels follow
  for (int64_t e = 0; e < nent; ++e) {
    const int type = d->ent[4 * e], id = d->ent[4 * e + 1];
    if (type < 0 || type > 2 || id < 0 || id >= (type == 0 ? d->nnear : d->nfar))
      return fail((set_error("m25_hmat_create: bad leaf entry"), M25_ERR_VALUE));
  }
  const int64_t cells = (int64_t)geom->nblocks * geom->nt;
  for (int64_t q = 0; q < d->nkeys; ++q)
    if (d->keys[q] < 0 || d->keys[q] >= cells || (q && d->keys[q] <= d->keys[q - 1]))
      return fail((set_error("m25_hmat_create: near-field keys not sorted or out of range"), M25_ERR_VALUE));
  for (int b = 0; b < d->npblk; ++b)
    if (d->pblk[b] < 0 || d->pblk[b] >= geom->nblocks)
      return fail((set_error("m25_hmat_create: bad pad block"), M25_ERR_VALUE));
  for (int i = 0; i < d->nb; ++i)
    if (d->perm[i] < 0 || d->perm[i] >= d->nb || d->lev[i] < 0 || d->lev[i] >= geom->nlev)
      return fail((set_error("m25_hmat_create: bad permutation or level"), M25_ERR_VALUE));
  if (d->leaf_lo[0] != 0 || d->leaf_lo[d->nleaf] != d->nb)
    return fail((set_error("m25_hmat_create: leaves do not cover the unknowns"), M25_ERR_VALUE));
  M25_CUDA(cudaStreamSynchronize(st));
  *out = h;
  return M25_OK;
}

extern "C" int m25_hmat_destroy(m25_hmat* h) {
  if (!h) return M25_OK;
  cudaStreamSynchronize(h->ctx->stream);
  free_all(h->gm_allocs);
  free_all(h->dense_allocs);
  free_all(h->allocs);
  delete h;
  return M25_OK;
}

extern "C" int m25_hmat_assemble(m25_hmat* h, m25_greens* gr, double zs_re, double zs_im, double zsv_re,
                                 double zsv_im, int64_t* stats) {
  if (!h || !gr) {
    set_error("m25_hmat_assemble: null argument");
    return M25_ERR_VALUE;
  }
  if (gr->nlev != h->geom->nlev) {
    set_error("m25_hmat_assemble: tables of another level count");
    return M25_ERR_VALUE;
  }
  m25_ctx* ctx = h->ctx;
  m25_geom* g = h->geom;
  cudaStream_t st = ctx->stream;
  int rc;
  // near field: the listed pairs' values, then the leaf pairs' blocks
  std::vector<void*> tmp;
  int32_t* cidx = nullptr;
  zd* Hc = nullptr;
  int* err = nullptr;
  const int64_t cells = (int64_t)g->nblocks * g->nt;
  if ((rc = alloc_async(tmp, reinterpret_cast<void**>(&cidx), sizeof(int32_t) * cells, st)) ||
      (rc = alloc_async(tmp, reinterpret_cast<void**>(&Hc), sizeof(zd) * 288 * (size_t)h->nkeys, st)) ||
      (rc = alloc_async(tmp, reinterpret_cast<void**>(&err), sizeof(int) * 4, st))) {
    free_all_async(tmp, st);
    return rc;
  }
  auto done = [&](int r) {
    free_all_async(tmp, st);
    return r;
  };
  if (cudaMemsetAsync(cidx, 0xFF, sizeof(int32_t) * cells, st) != cudaSuccess ||
      cudaMemsetAsync(err, 0, sizeof(int) * 4, st) != cudaSuccess) {
    set_error("m25_hmat_assemble: memset failed");
    return done(M25_ERR_CUDA);
  }
  if (h->npblk) cidx_pad_kernel<<<dim3((g->nt + 255) / 256, h->npblk), 256, 0, st>>>(h->pblk, h->npblk, g->nt, cidx);
  cidx_keys_kernel<<<(unsigned)((h->nkeys + 255) / 256), 256, 0, st>>>(h->keys, h->nkeys, cidx);
  if (cudaGetLastError() != cudaSuccess) {
    set_error("m25_hmat_assemble: launch failed");
    return done(M25_ERR_CUDA);
  }
  const zd zs(zs_re, zs_im), zsv(zsv_re, zsv_im);
  if ((rc = fill_listed(ctx, g, gr, zs, zsv, cidx, Hc, h->perm, h->ZxbT, h->Zxx))) return done(rc);
  near_kernel<<<h->nnear, 256, 0, st>>>(h->near, h->near_off, h->perm, g->edge_tri, g->edge_loc, g->tpos, cidx, g->nt,
                                        Hc, h->Zn, err);
  if (cudaGetLastError() != cudaSuccess) {
    set_error("m25_hmat_assemble: near-field launch failed");
    return done(M25_ERR_CUDA);
  }
  // far field: ACA, then the blocks kept as they are
  const Tabs t = make_tabs(gr);
  std::vector<int32_t> rk(std::max(h->naca, 1)), stt(std::max(h->naca, 1));
  for (auto& F : h->fb_h) {
    F.rank = 0;
    if (F.kcap > 0) F.kind = 0;
  }
  if (h->naca) {
    if (cudaMemcpyAsync(h->fb, h->fb_h.data(), sizeof(FarB) * h->nfar, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(h->flags, 0, std::max<int64_t>(h->flag_bytes, 1), st) != cudaSuccess) {
      set_error("m25_hmat_assemble: copy failed");
      return done(M25_ERR_CUDA);
    }
    aca_kernel<<<h->naca, 256, 0, st>>>(t, h->rules, h->lev, h->fb, h->aca_ids, h->pool, h->flags, h->tol, h->rank,
                                        h->status);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(rk.data(), h->rank, sizeof(int32_t) * h->naca, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(stt.data(), h->status, sizeof(int32_t) * h->naca, cudaMemcpyDeviceToHost, st) != cudaSuccess) {
      set_error("m25_hmat_assemble: ACA launch failed");
      return done(M25_ERR_CUDA);
    }
  }
  int nerr = 0;
  if (cudaMemcpyAsync(&nerr, err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    set_error(std::string("m25_hmat_assemble: ") + cudaGetErrorString(cudaGetLastError()));
    return done(M25_ERR_CUDA);
  }
  if (nerr) {
    set_error("m25_hmat_assemble: a near block needs a triangle pair the near-field list does not hold");
    return done(M25_ERR_VALUE);
  }
  int64_t max_rank = 0, rank_sum = 0, not_low = 0, nlow = 0, far_entries = 0;
  {
    int a = 0;
    for (int f = 0; f < h->nfar; ++f) {
      FarB& F = h->fb_h[f];
      if (F.kcap == 0) continue;
      F.rank = rk[a];
      if (stt[a]) {
        F.kind = 1;
        ++not_low;
      } else {
        ++nlow;
        max_rank = std::max<int64_t>(max_rank, F.rank);
        rank_sum += F.rank;
        far_entries += (int64_t)F.rank * (F.m + F.n);
      }
      ++a;
    }
  }
  // the low-rank terms the matvec projects on, one warp each
  std::vector<int2> terms;
  for (int f = 0; f < h->nfar; ++f) {
    const FarB& F = h->fb_h[f];
    if (F.kind == 0)
      for (int l = 0; l < F.rank; ++l) terms.push_back(make_int2(f, l));
  }
  h->nterm = (int)terms.size();
  if (h->nterm && cudaMemcpyAsync(h->terms, terms.data(), sizeof(int2) * terms.size(), cudaMemcpyHostToDevice, st) !=
                      cudaSuccess) {
    set_error("m25_hmat_assemble: copy failed");
    return done(M25_ERR_CUDA);
  }
  // storage of the blocks kept as they are (B and B^T)
  std::vector<int32_t> dense;
  int64_t doff = 0;
  for (int f = 0; f < h->nfar; ++f) {
    FarB& F = h->fb_h[f];
    if (F.kind == 1) {
      F.dense = doff;
      doff += 2 * (int64_t)F.m * F.n;
      far_entries += (int64_t)F.m * F.n;
      dense.push_back(f);
    }
  }
  if ((size_t)doff * sizeof(zd) > h->dense_bytes) {
    free_all(h->dense_allocs);
    h->dense_pool = nullptr;
    h->dense_df = nullptr;
    h->dense_bytes = 0;
    if ((rc = dalloc(h->dense_allocs, &h->dense_pool, (size_t)doff)) ||
        (rc = dalloc(h->dense_allocs, &h->dense_df, (size_t)doff)))
      return done(rc);
    h->dense_bytes = (size_t)std::max<int64_t>(doff, 1) * sizeof(zd);
  }
  if ((h->nfar && cudaMemcpyAsync(h->fb, h->fb_h.data(), sizeof(FarB) * h->nfar, cudaMemcpyHostToDevice, st) !=
                     cudaSuccess) ||
      (dense.size() && cudaMemcpyAsync(h->dense_ids, dense.data(), sizeof(int32_t) * dense.size(),
                                       cudaMemcpyHostToDevice, st) != cudaSuccess)) {
    set_error("m25_hmat_assemble: copy failed");
    return done(M25_ERR_CUDA);
  }
  if (!dense.empty())
    far_dense_kernel<<<(unsigned)dense.size(), 256, 0, st>>>(t, h->rules, h->lev, h->fb, h->dense_ids, h->dense_pool);
  // preconditioner: the diagonal blocks and their LU
  {  // the matvec's double-float copies of the operator
    auto split = [&](const zd* src, float4* dst, int64_t n) {
      if (n > 0) df_split_kernel<<<(unsigned)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, st>>>(src, dst, n);
    };
    split(h->Zn, h->Zn_df, h->near_entries);
    split(h->pool, h->pool_df, h->uv_entries);
    split(h->ZxbT, h->ZxbT_df, (int64_t)h->nb * h->nv);
    split(h->dense_pool, h->dense_df, doff);
  }
  wscale_kernel<<<(h->n + 255) / 256, 256, 0, st>>>(h->nb, h->n, h->nv, h->row_leaf, h->self_near, h->near,
                                                    h->near_off, h->Zn, h->Zxx, h->wsc);
  diag_kernel<<<h->npc, 256, 0, st>>>(h->pc_off, h->pc_gidx, h->pc_item_off, h->pc_items, h->pc_doff, h->nb, h->nv,
                                      h->nnear, h->leaf_lo, h->near_off, h->Zn, h->fb, h->pool, h->dense_pool, h->ZxbT,
                                      h->Zxx, h->D);
  ginv_kernel<<<h->npc, 1024, 0, st>>>(h->pc_off, h->pc_doff, h->D);  // 32 warps: the sweeps wait on L2
  if (cudaGetLastError() != cudaSuccess) {
    set_error("m25_hmat_assemble: launch failed");
    return done(M25_ERR_CUDA);
  }
  rc = done(M25_OK);
  M25_CUDA(cudaStreamSynchronize(st));
  if (rc) return rc;
  h->assembled = true;
  if (stats) {
    stats[0] = h->near_entries;
    stats[1] = nlow;
    stats[2] = (int64_t)dense.size();
    stats[3] = far_entries;
    stats[4] = max_rank;
    stats[5] = rank_sum;
    stats[6] = not_low;
    stats[7] = h->nkeys;
  }
  return M25_OK;
}

namespace {
int ensure_gmres(m25_hmat* h, int restart) {
  if (h->restart_cap >= restart && h->Vb) return M25_OK;
  free_all(h->gm_allocs);
  h->Vb = h->Zb = h->w = h->xv = h->zv = h->bv = h->hv = nullptr;
  h->nrm = nullptr;
  int rc;
  const size_t n = h->n;
  if ((rc = dalloc(h->gm_allocs, &h->Vb, (size_t)(restart + 1) * n)) ||
      (rc = dalloc(h->gm_allocs, &h->Zb, (size_t)restart * n)) || (rc = dalloc(h->gm_allocs, &h->w, n)) ||
      (rc = dalloc(h->gm_allocs, &h->xv, n)) || (rc = dalloc(h->gm_allocs, &h->zv, n)) ||
      (rc = dalloc(h->gm_allocs, &h->bv, n)) || (rc = dalloc(h->gm_allocs, &h->hv, 2 * (size_t)(restart + 2))) ||
      (rc = dalloc(h->gm_allocs, &h->nrm, 4)))
    return rc;
  h->restart_cap = restart;
  return M25_OK;
}
}  // namespace

extern "C" int m25_hmat_matvec(m25_hmat* h, const double* x, double* y) {
  if (!h || !x || !y) {
    set_error("m25_hmat_matvec: null argument");
    return M25_ERR_VALUE;
  }
  if (!h->assembled) {
    set_error("m25_hmat_matvec: the operator is not assembled");
    return M25_ERR_VALUE;
  }
  int rc;
  if ((rc = ensure_gmres(h, 1))) return rc;
  cudaStream_t st = h->ctx->stream;
  const int n = h->n, g = (n + 255) / 256;
  M25_CUDA(cudaMemcpyAsync(h->bv, x, sizeof(zd) * n, cudaMemcpyHostToDevice, st));
  perm_in_kernel<<<g, 256, 0, st>>>(h->nb, n, h->perm, h->bv, h->xv);
  if ((rc = apply(h, h->xv, h->w))) return rc;
  perm_out_kernel<<<g, 256, 0, st>>>(h->nb, n, h->perm, h->w, h->zv);
  M25_CHECK_LAUNCH();
  M25_CUDA(cudaMemcpyAsync(y, h->zv, sizeof(zd) * n, cudaMemcpyDeviceToHost, st));
  M25_CUDA(cudaStreamSynchronize(st));
  return M25_OK;
}

extern "C" int m25_hmat_solve(m25_hmat* h, int32_t nrhs, const double* B, double* X, double rtol, int32_t restart,
                              int32_t maxiter, int32_t* iters, double* resid) {
  if (!h || !B || !X || nrhs < 1 || restart < 1 || restart > 2000 || maxiter < 1 || !(rtol > 0.0)) {
    set_error("m25_hmat_solve: bad argument");
    return M25_ERR_VALUE;
  }
  if (!h->assembled) {
    set_error("m25_hmat_solve: the operator is not assembled");
    return M25_ERR_VALUE;
  }
  int rc;
  if ((rc = ensure_gmres(h, restart))) return rc;
  cudaStream_t st = h->ctx->stream;
  const int n = h->n, g = (n + 255) / 256;
  const int64_t ldv = n;
  std::vector<std::complex<double>> col(n), hh(2 * (restart + 2));
  using cplx = std::complex<double>;
  for (int c = 0; c < nrhs; ++c) {
    for (int i = 0; i < n; ++i) col[i] = cplx(B[2 * ((int64_t)i * nrhs + c)], B[2 * ((int64_t)i * nrhs + c) + 1]);
    M25_CUDA(cudaMemcpyAsync(h->w, col.data(), sizeof(zd) * n, cudaMemcpyHostToDevice, st));
    perm_in_kernel<<<g, 256, 0, st>>>(h->nb, n, h->perm, h->w, h->zv);
    vscale_kernel<<<g, 256, 0, st>>>(h->bv, h->zv, h->wsc, n, 0);  // the scaled system's right-hand side W b
    M25_CUDA(cudaMemsetAsync(h->xv, 0, sizeof(zd) * n, st));
    norm_kernel<<<1, 1024, 0, st>>>(h->bv, n, h->nrm);
    double bnorm = 0.0;
    M25_CUDA(cudaMemcpyAsync(&bnorm, h->nrm, sizeof(double), cudaMemcpyDeviceToHost, st));
    M25_CUDA(cudaStreamSynchronize(st));
    int total = 0;
    double rel = 0.0;
    if (bnorm > 0.0) {
      bool conv = false;
      for (int cyc = 0; cyc < maxiter && !conv; ++cyc) {
        // r = b - A x (x = 0 on the first cycle)
        if (cyc == 0) {
          M25_CUDA(cudaMemcpyAsync(h->w, h->bv, sizeof(zd) * n, cudaMemcpyDeviceToDevice, st));
        } else {
          if ((rc = sapply(h, h->xv, h->zv))) return rc;
          sub_kernel<<<g, 256, 0, st>>>(h->w, h->bv, h->zv, n);
        }
        norm_kernel<<<1, 1024, 0, st>>>(h->w, n, h->nrm);
        double beta = 0.0;
        M25_CUDA(cudaMemcpyAsync(&beta, h->nrm, sizeof(double), cudaMemcpyDeviceToHost, st));
        M25_CUDA(cudaStreamSynchronize(st));
        rel = beta / bnorm;
        if (rel <= rtol) {
          conv = true;
          break;
        }
        scale_kernel<<<g, 256, 0, st>>>(h->Vb, h->w, n, 1.0 / beta);
        std::vector<cplx> H((size_t)(restart + 1) * restart), cs(restart), sn(restart), gv(restart + 1);
        gv[0] = beta;
        int j = 0;
        for (; j < restart; ++j) {
          // z_j = M^-1 v_j (kept: flexible GMRES), w = A z_j orthogonalised twice against v_0 .. v_j
          if ((rc = sprecond(h, h->Vb + (int64_t)j * ldv, h->Zb + (int64_t)j * ldv))) return rc;
          if ((rc = sapply(h, h->Zb + (int64_t)j * ldv, h->w))) return rc;
          for (int pass = 0; pass < 2; ++pass) {
            dots_kernel<<<j + 1, 256, 0, st>>>(h->Vb, ldv, n, h->w, h->hv + pass * (restart + 2));
            combine_kernel<<<g, 256, 0, st>>>(h->w, h->Vb, ldv, j + 1, n, h->hv + pass * (restart + 2), -1.0);
          }
          norm_kernel<<<1, 1024, 0, st>>>(h->w, n, h->nrm);
          M25_CHECK_LAUNCH();
          double hn = 0.0;
          M25_CUDA(cudaMemcpyAsync(hh.data(), h->hv, sizeof(zd) * 2 * (restart + 2), cudaMemcpyDeviceToHost, st));
          M25_CUDA(cudaMemcpyAsync(&hn, h->nrm, sizeof(double), cudaMemcpyDeviceToHost, st));
          M25_CUDA(cudaStreamSynchronize(st));
          cplx* Hj = H.data() + (size_t)j * (restart + 1);  // column j
          for (int l = 0; l <= j; ++l) Hj[l] = hh[l] + hh[(restart + 2) + l];
          Hj[j + 1] = hn;
          for (int l = 0; l < j; ++l) {  // earlier rotations
            const cplx a = Hj[l], b = Hj[l + 1];
            Hj[l] = std::conj(cs[l]) * a + std::conj(sn[l]) * b;
            Hj[l + 1] = -sn[l] * a + cs[l] * b;
          }
          const double den = std::sqrt(std::norm(Hj[j]) + hn * hn);
          if (den == 0.0) {
            cs[j] = 1.0;
            sn[j] = 0.0;
          } else {
            cs[j] = Hj[j] / den;
            sn[j] = cplx(hn, 0.0) / den;
          }
          Hj[j] = std::conj(cs[j]) * Hj[j] + std::conj(sn[j]) * cplx(hn, 0.0);
          Hj[j + 1] = 0.0;
          gv[j + 1] = -sn[j] * gv[j];
          gv[j] = std::conj(cs[j]) * gv[j];
          ++total;
          rel = std::abs(gv[j + 1]) / bnorm;
          if (hn > 0.0) scale_kernel<<<g, 256, 0, st>>>(h->Vb + (int64_t)(j + 1) * ldv, h->w, n, 1.0 / hn);
          if (rel <= rtol || hn == 0.0) {
            ++j;
            break;
          }
        }
        const int k = std::min(j, restart);
        // y from the triangle, x += Z y
        std::vector<cplx> y(k);
        for (int r = k - 1; r >= 0; --r) {
          cplx s = gv[r];
          for (int l = r + 1; l < k; ++l) s -= H[(size_t)l * (restart + 1) + r] * y[l];
          y[r] = s / H[(size_t)r * (restart + 1) + r];
        }
        M25_CUDA(cudaMemcpyAsync(h->hv, y.data(), sizeof(zd) * k, cudaMemcpyHostToDevice, st));
        combine_kernel<<<g, 256, 0, st>>>(h->xv, h->Zb, ldv, k, n, h->hv, 1.0);
        M25_CHECK_LAUNCH();
      }
      // the true residual (of the scaled system)
      if ((rc = sapply(h, h->xv, h->zv))) return rc;
      sub_kernel<<<g, 256, 0, st>>>(h->w, h->bv, h->zv, n);
      norm_kernel<<<1, 1024, 0, st>>>(h->w, n, h->nrm);
      double rn = 0.0;
      M25_CUDA(cudaMemcpyAsync(&rn, h->nrm, sizeof(double), cudaMemcpyDeviceToHost, st));
      M25_CUDA(cudaStreamSynchronize(st));
      rel = rn / bnorm;
    }
    vscale_kernel<<<g, 256, 0, st>>>(h->w, h->xv, h->wsc, n, 0);  // x = W x~
    perm_out_kernel<<<g, 256, 0, st>>>(h->nb, n, h->perm, h->w, h->zv);
    M25_CHECK_LAUNCH();
    M25_CUDA(cudaMemcpyAsync(col.data(), h->zv, sizeof(zd) * n, cudaMemcpyDeviceToHost, st));
    M25_CUDA(cudaStreamSynchronize(st));
    for (int i = 0; i < n; ++i) {
      X[2 * ((int64_t)i * nrhs + c)] = col[i].real();
      X[2 * ((int64_t)i * nrhs + c) + 1] = col[i].imag();
    }
    if (iters) iters[c] = total;
    if (resid) resid[c] = rel;
  }
  return M25_OK;
}
