// Dense complex LU with partial pivoting and the triangular solves, the
// GPU replacement of mom25d's _dense_solve (Engine/mom25d/solver.py:11-23,
// LAPACK zgetrf / zgetrs through scipy).
//
// Right-looking blocked factorisation of a row-major matrix, per panel of
// nb columns:
//   panel_kernel   cooperative grid: each CTA keeps a slice of the panel
//                  rows in shared memory; one bounded grid barrier per
//                  column (pivot search |re| + |im| as izamax, swap, scale,
//                  rank-1 update of the panel)
//   swap_trsm_kernel  the panel's row interchanges on the other columns,
//                  composed into one gather, fused with U12 = L11^-1 A12
//   gemm_kernel    A22 -= L21 U12 (SIMT)
// The complex64 factorisation with tensor cores (lu_tc.cu) goes in blocks of
// 128 columns, each two panels of 64: the first panel's interchanges and
// U12 on the second panel's columns, their rank-64 update, the second panel,
// then both panels' interchanges with U12 = L11^-1 A12 (L11 128 x 128) on
// the trailing columns and one rank-128 update of the trailing matrix. The
// update is bound by its read-modify-write of the trailing matrix, which
// this does once per 128 columns.
// Solve: permutation, blocked forward / backward substitution. The mixed
// path refines in fp64: r = B - Z X, X += LU32^-1 r.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "m25_internal.h"

namespace m25 {

constexpr long long kBarrierSpinLimit = 1LL << 25;  // ~1 s of polling, then give up

// Grid-wide barrier for a cooperative launch. Every wait is bounded: on
// timeout the CTA raises *err and the caller returns.
__device__ inline bool grid_sync(unsigned* count, unsigned* gen, unsigned nblocks, int* err) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vgen = gen;
    unsigned g0 = *vgen;
    __threadfence();
    unsigned arrived = atomicAdd(count, 1u);
    if (arrived == nblocks - 1) {
      atomicExch(count, 0u);
      __threadfence();
      atomicAdd(gen, 1u);
    } else {
      long long it = 0;
      while (*vgen == g0) {
        if (++it > kBarrierSpinLimit || *(volatile int*)err) {
          atomicExch(err, 1);
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *(volatile int*)err == 0;
}

template <class T>
struct PanelArgs {
  cx<T>* A;
  int64_t lda;
  int n, k0, nb, rows_per_cta;
  int32_t* ipiv;      // absolute pivot row per factored row
  cx<T>* cand;        // (2, G, nb) candidate pivot rows
  T* candval;         // (2, G)
  int* candidx;       // (2, G)
  cx<T>* rowj;        // (2, nb) row k0+j before the swap
  unsigned* bar;      // count, generation
  int* err;           // barrier timeout
  int* info;          // first zero pivot (1-based), 0 if none
};

template <class T>
__global__ void __launch_bounds__(256) panel_kernel(PanelArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int G = gridDim.x, g = blockIdx.x, nb = a.nb;
  const int r0 = a.k0 + g * a.rows_per_cta;
  const int r1 = min(a.n, r0 + a.rows_per_cta);
  const int R = max(0, r1 - r0);
  cx<T>* P = reinterpret_cast<cx<T>*>(smem_raw);      // (rows_per_cta, nb)
  cx<T>* urow = P + (size_t)a.rows_per_cta * nb;        // (nb)
  __shared__ T red_v[8];
  __shared__ int red_i[8];
  __shared__ int red_g[8];
  __shared__ int piv_sh;
  for (int e = threadIdx.x; e < R * nb; e += blockDim.x) {
    int r = e / nb, c = e % nb;
    P[e] = a.A[(int64_t)(r0 + r) * a.lda + a.k0 + c];
  }
  __syncthreads();
  for (int j = 0; j < nb; ++j) {
    const int row_j = a.k0 + j;
    const int par = j & 1;
    // local pivot candidate: max |re|+|im|, first index on ties
    T best = T(-1);
    int bi = -1;
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
      if (r0 + r < row_j) continue;
      T v = cabs1(P[r * nb + j]);
      if (v > best) {
        best = v;
        bi = r0 + r;
      }
    }
    for (int o = 16; o; o >>= 1) {
      T ov = __shfl_down_sync(0xffffffffu, best, o);
      int oi = __shfl_down_sync(0xffffffffu, bi, o);
      if (oi >= 0 && (ov > best || (ov == best && (bi < 0 || oi < bi)))) {
        best = ov;
        bi = oi;
      }
    }
    if ((threadIdx.x & 31) == 0) {
      red_v[threadIdx.x >> 5] = best;
      red_i[threadIdx.x >> 5] = bi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      T bv = T(-1);
      int bidx = -1;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        int oi = red_i[w];
        T ov = red_v[w];
        if (oi >= 0 && (ov > bv || (ov == bv && (bidx < 0 || oi < bidx)))) {
          bv = ov;
          bidx = oi;
        }
      }
      a.candval[par * G + g] = bv;
      a.candidx[par * G + g] = bidx;
      piv_sh = bidx;
    }
    __syncthreads();
    {
      int bidx = piv_sh;
      if (bidx >= 0)
        for (int c = threadIdx.x; c < nb; c += blockDim.x)
          a.cand[((size_t)par * G + g) * nb + c] = P[(bidx - r0) * nb + c];
      if (row_j >= r0 && row_j < r1)
        for (int c = threadIdx.x; c < nb; c += blockDim.x) a.rowj[par * nb + c] = P[(row_j - r0) * nb + c];
    }
    if (!grid_sync(a.bar, a.bar + 1, G, a.err)) return;
    // global pivot: all threads read the G candidates, then a block reduction
    {
      T bv = T(-1);
      int bidx = -1, bg = -1;
      for (int q = threadIdx.x; q < G; q += blockDim.x) {
        int oi = *(volatile int*)&a.candidx[par * G + q];
        T ov = *(volatile T*)&a.candval[par * G + q];
        if (oi >= 0 && (ov > bv || (ov == bv && (bidx < 0 || oi < bidx)))) {
          bv = ov;
          bidx = oi;
          bg = q;
        }
      }
      for (int o = 16; o; o >>= 1) {
        T ov = __shfl_down_sync(0xffffffffu, bv, o);
        int oi = __shfl_down_sync(0xffffffffu, bidx, o);
        int og = __shfl_down_sync(0xffffffffu, bg, o);
        if (oi >= 0 && (ov > bv || (ov == bv && (bidx < 0 || oi < bidx)))) {
          bv = ov;
          bidx = oi;
          bg = og;
        }
      }
      if ((threadIdx.x & 31) == 0) {
        red_v[threadIdx.x >> 5] = bv;
        red_i[threadIdx.x >> 5] = bidx;
        red_g[threadIdx.x >> 5] = bg;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      T bv = T(-1);
      int bidx = -1, bg = -1;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        int oi = red_i[w];
        T ov = red_v[w];
        if (oi >= 0 && (ov > bv || (ov == bv && (bidx < 0 || oi < bidx)))) {
          bv = ov;
          bidx = oi;
          bg = red_g[w];
        }
      }
      if (bidx < 0 || bv == T(0)) {
        if (g == 0 && *a.info == 0) *a.info = row_j + 1;
        bidx = row_j;
        bg = -1;
      }
      piv_sh = bidx;
      red_i[0] = bg;
      if (g == 0) a.ipiv[row_j] = bidx;
    }
    __syncthreads();
    const int p = piv_sh, pg = red_i[0];
    for (int c = threadIdx.x; c < nb; c += blockDim.x) {
      if (pg >= 0) {
        volatile cx<T>* src = &a.cand[((size_t)par * G + pg) * nb + c];
        urow[c] = cx<T>(src->re, src->im);
      } else if (row_j >= r0 && row_j < r1) {
        urow[c] = P[(row_j - r0) * nb + c];
      }
    }
    __syncthreads();
    if (pg < 0 && !(row_j >= r0 && row_j < r1)) {
      // zero pivot owned elsewhere: take the row from the published copy
      for (int c = threadIdx.x; c < nb; c += blockDim.x) {
        volatile cx<T>* src = &a.rowj[par * nb + c];
        urow[c] = cx<T>(src->re, src->im);
      }
      __syncthreads();
    }
    if (p != row_j) {
      if (p >= r0 && p < r1)
        for (int c = threadIdx.x; c < nb; c += blockDim.x) {
          volatile cx<T>* src = &a.rowj[par * nb + c];
          P[(p - r0) * nb + c] = cx<T>(src->re, src->im);
        }
      if (row_j >= r0 && row_j < r1)
        for (int c = threadIdx.x; c < nb; c += blockDim.x) P[(row_j - r0) * nb + c] = urow[c];
    }
    __syncthreads();
    const cx<T> piv = urow[j];
    const bool zero = piv.re == T(0) && piv.im == T(0);
    // multipliers, then the rank-1 update of the panel's remaining columns
    if (!zero)
      for (int r = threadIdx.x; r < R; r += blockDim.x)
        if (r0 + r > row_j) P[r * nb + j] = P[r * nb + j] / piv;
    __syncthreads();
    const int w = nb - j - 1;
    if (w > 0)
      for (int e = threadIdx.x; e < R * w; e += blockDim.x) {
        int r = e / w, c = j + 1 + e % w;
        if (r0 + r > row_j) P[r * nb + c] -= P[r * nb + j] * urow[c];
      }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < R * nb; e += blockDim.x) {
    int r = e / nb, c = e % nb;
    a.A[(int64_t)(r0 + r) * a.lda + a.k0 + c] = P[e];
  }
}

// ------------------------------------------------ panel on one CTA cluster
// For trailing sizes whose panel fits in the shared memory of one cluster of
// CL CTAs (16, the largest cluster size: about 6500 rows of
// 64 complex64 columns), the panel is factored without global barriers. CTA q
// of the cluster keeps rows k0 + q R .. + R - 1 in shared memory. Per column
// j, every CTA pushes its pivot candidate (value, row index and the whole
// row) into the shared memory of all 16 CTAs, and the owner of row j pushes
// row j as well; one hardware cluster barrier later every CTA holds all it
// needs locally: it picks the pivot (max |re| + |im|, first index on ties,
// as panel_kernel), the two owners swap rows p and j in place, and every CTA
// scales and updates its own rows, finding the next column's candidate while
// it updates. The pushed data is double-buffered by column parity: a CTA can
// only write column j + 2's buffers after every CTA has passed column j + 1's
// barrier, that is, after all reads of column j's buffers.
constexpr int kPanelCluster = 16;  // the largest cluster; smaller trailing blocks take 8 or 4 CTAs
constexpr int kPanelLd = 65;  // padded row of the panel in shared memory

template <class T>
struct ClusterPanelArgs {
  cx<T>* A;
  int64_t lda;
  int n, k0, nb, rows_per_cta;
  int32_t* ipiv;
  int* info;
  int* err;  // a wait for pushed data ran out
  float* A2; // tensor-core update: tf32 [hi | lo] planes of conj(L21) (rows of 2 P floats), or null
  int P;
};

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

template <class T>
struct alignas(16) PivCand {
  T val;
  int idx;
};

template <class T, int CL>
constexpr size_t cluster_panel_smem(int R) {
  // rows + candidate rows (2 x CL x 64) + row j (2 x 64)
  return sizeof(cx<T>) * ((size_t)R * kPanelLd + 2 * CL * 64 + 2 * 64);
}

__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;\n" : "=r"(r));
  return r;
}
// the address of a shared variable of this CTA in the shared memory of cluster CTA rank
__device__ __forceinline__ uint32_t dsmem(const void* p, uint32_t rank) {
  uint32_t a = (uint32_t)__cvta_generic_to_shared(p), r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
// remote store that completes its bytes on the destination CTA's mbarrier
__device__ __forceinline__ void st_async(uint32_t a, cx<float> v, uint32_t bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f32 [%0], {%1, %2}, [%3];\n" ::"r"(a),
               "f"(v.re), "f"(v.im), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void st_async(uint32_t a, cx<double> v, uint32_t bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f64 [%0], {%1, %2}, [%3];\n" ::"r"(a),
               "d"(v.re), "d"(v.im), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void st_async(uint32_t a, PivCand<float> v, uint32_t bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.b32 [%0], {%1, %2}, [%3];\n" ::"r"(a),
               "r"(__float_as_uint(v.val)), "r"(v.idx), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void st_async(uint32_t a, PivCand<double> v, uint32_t bar) {
  asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.b64 [%0], {%1, %2}, [%3];\n" ::"r"(a),
               "l"(__double_as_longlong(v.val)), "l"((long long)v.idx), "r"(bar)
               : "memory");
}
// bytes of one pushed candidate record
template <class T>
constexpr int cand_push_bytes() {
  return sizeof(T) == 4 ? 8 : 16;
}
__device__ __forceinline__ void cl_mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"((uint32_t)__cvta_generic_to_shared(bar)), "r"(count));
}
__device__ __forceinline__ void cl_mbar_expect(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(bar)),
               "r"(bytes)
               : "memory");
}
// bounded wait (iterations and wall clock) for the phase of the given parity
// of a barrier completed by remote transactions; false on a timeout
__device__ __forceinline__ bool cl_mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t addr = (uint32_t)__cvta_generic_to_shared(bar);
  unsigned long long t0;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t0));
  for (long long it = 0; it < kBarrierSpinLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    if (t - t0 > 500ull * 1000 * 1000) return false;
  }
  return false;
}

// better candidate: larger value, first index on ties
template <class T>
__device__ __forceinline__ bool piv_better(T ov, int oi, T v, int i) {
  return oi >= 0 && (ov > v || (ov == v && (i < 0 || oi < i)));
}

constexpr int kPanelThreads = 512;
constexpr int kPanelGroups = kPanelThreads / 64;  // row groups of the update's 2-D map

template <class T, int CL>
__global__ void __launch_bounds__(kPanelThreads, 1) panel_cluster_kernel(ClusterPanelArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int q = (int)cluster_rank(), nb = a.nb, R = a.rows_per_cta, tid = threadIdx.x;
  const int r0 = a.k0 + q * R;
  const int r1 = min(a.n, r0 + R);
  const int Rq = max(0, r1 - r0);
  cx<T>* P = reinterpret_cast<cx<T>*>(smem_raw);          // (R, kPanelLd) this CTA's rows
  cx<T>* crow = P + (size_t)R * kPanelLd;                   // (2, 16, 64) pushed candidate rows
  cx<T>* jrow = crow + 2 * CL * 64;              // (2, 64) pushed row k0 + j
  __shared__ PivCand<T> cand[2][CL];             // pushed candidates
  __shared__ T gmax_v[kPanelGroups];
  __shared__ int gmax_i[kPanelGroups];
  __shared__ __align__(8) uint64_t colbar[2];  // per column parity: completed by the 16 CTAs' pushes
  if (tid == 0) {
    cl_mbar_init(&colbar[0], 1);
    cl_mbar_init(&colbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  for (int e = tid; e < Rq * 64; e += blockDim.x) {
    const int r = e >> 6, c = e & 63;
    if (c < nb) P[r * kPanelLd + c] = a.A[(int64_t)(r0 + r) * a.lda + a.k0 + c];
  }
  // 2-D map of the update: column uc, rows ug, ug + kPanelGroups, ...
  const int uc = tid & 63, ug = tid >> 6;
  __syncthreads();
  // candidate of column 0 (afterwards found during each update)
  if (uc == 0) {
    T bv = T(-1);
    int bi = -1;
    for (int r = ug; r < Rq; r += kPanelGroups) {
      const T v = cabs1(P[r * kPanelLd]);
      if (v > bv) {
        bv = v;
        bi = r0 + r;
      }
    }
    gmax_v[ug] = bv;
    gmax_i[ug] = bi;
  }
  __syncthreads();
  cluster_sync_all();  // every CTA runs, with its barriers set up, before the first push
  // bytes pushed into each CTA per column: 16 candidates, 16 rows, row j
  const uint32_t expect = CL * (cand_push_bytes<T>() + nb * (int)sizeof(cx<T>)) + nb * sizeof(cx<T>);
  for (int j = 0; j < nb; ++j) {
    const int row_j = a.k0 + j, par = j & 1;
    const int qj = j / R;
    // this CTA's candidate for column j (rows >= row_j)
    T bv = T(-1);
    int bi = -1;
#pragma unroll
    for (int g = 0; g < kPanelGroups; ++g)
      if (piv_better(gmax_v[g], gmax_i[g], bv, bi)) {
        bv = gmax_v[g];
        bi = gmax_i[g];
      }
    // push: candidate, candidate row (zeros without a candidate), and row j
    // from its owner, into all 16 CTAs; each store completes its bytes on
    // the destination's barrier of this column's parity
    if (tid == 0) cl_mbar_expect(&colbar[par], expect);
    if (tid < CL) st_async(dsmem(&cand[par][q], tid), PivCand<T>{bv, bi}, dsmem(&colbar[par], tid));
    for (int e = tid; e < CL * 64; e += blockDim.x) {
      const int dst = e >> 6, c = e & 63;
      if (c < nb)
        st_async(dsmem(&crow[(par * CL + q) * 64 + c], dst),
                 bi >= 0 ? P[(bi - r0) * kPanelLd + c] : cx<T>(), dsmem(&colbar[par], dst));
    }
    if (q == qj)
      for (int e = tid; e < CL * 64; e += blockDim.x) {
        const int dst = e >> 6, c = e & 63;
        if (c < nb)
          st_async(dsmem(&jrow[par * 64 + c], dst), P[(row_j - r0) * kPanelLd + c], dsmem(&colbar[par], dst));
      }
    // wait until all of column j's pushes have landed here
    const bool got = cl_mbar_wait(&colbar[par], (j >> 1) & 1);
    if (__syncthreads_or(!got)) {
      if (tid == 0) atomicExch(a.err, 1);
      break;
    }
    // every thread picks the pivot from the 16 local candidates
    T v = T(-1);
    int p = -1, src = -1;
#pragma unroll
    for (int k = 0; k < CL; ++k) {
      const PivCand<T> c = cand[par][k];
      if (piv_better(c.val, c.idx, v, p)) {
        v = c.val;
        p = c.idx;
        src = k;
      }
    }
    if (p < 0 || v == T(0)) {  // zero column: no interchange, no scaling
      if (tid == 0 && q == 0 && *a.info == 0) *a.info = row_j + 1;
      p = row_j;
      src = -1;
    }
    if (tid == 0 && q == 0) a.ipiv[row_j] = p;
    const cx<T>* urow = src >= 0 ? crow + (par * CL + src) * 64 : jrow + par * 64;
    if (p != row_j) {
      if (p >= r0 && p < r1)
        for (int c = tid; c < nb; c += blockDim.x) P[(p - r0) * kPanelLd + c] = jrow[par * 64 + c];
      if (q == qj)
        for (int c = tid; c < nb; c += blockDim.x) P[(row_j - r0) * kPanelLd + c] = urow[c];
    }
    __syncthreads();
    // multipliers (rows below row j), by the reciprocal pivot
    if (src >= 0) {
      const cx<T> pv = urow[j];
      const T m2 = pv.re * pv.re + pv.im * pv.im;
      const cx<T> rp(pv.re / m2, -pv.im / m2);
      for (int r = tid; r < Rq; r += blockDim.x)
        if (r0 + r > row_j) P[r * kPanelLd + j] = P[r * kPanelLd + j] * rp;
    }
    __syncthreads();
    // rank-1 update of the columns right of j, four rows at a time (loads
    // first); the threads of column j + 1 track the next candidate
    {
      T gv = T(-1);
      int gi = -1;
      if (uc > j && uc < nb) {
        const cx<T> u = urow[uc];
        // first row below row j in this group
        int r = ug;
        const int rlo = row_j + 1 - r0;
        if (r < rlo) r += (rlo - r + kPanelGroups - 1) / kPanelGroups * kPanelGroups;
        for (; r + 3 * kPanelGroups < Rq; r += 4 * kPanelGroups) {
          cx<T> x[4], m[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            x[i] = P[(r + i * kPanelGroups) * kPanelLd + uc];
            m[i] = P[(r + i * kPanelGroups) * kPanelLd + j];
          }
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            x[i] -= m[i] * u;
            P[(r + i * kPanelGroups) * kPanelLd + uc] = x[i];
          }
          if (uc == j + 1)
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              const T cv = cabs1(x[i]);
              if (cv > gv) {
                gv = cv;
                gi = r0 + r + i * kPanelGroups;
              }
            }
        }
        for (; r < Rq; r += kPanelGroups) {
          const cx<T> x = P[r * kPanelLd + uc] - P[r * kPanelLd + j] * u;
          P[r * kPanelLd + uc] = x;
          if (uc == j + 1) {
            const T cv = cabs1(x);
            if (cv > gv) {
              gv = cv;
              gi = r0 + r;
            }
          }
        }
      }
      if (uc == j + 1) {
        gmax_v[ug] = gv;
        gmax_i[ug] = gi;
      }
    }
    __syncthreads();
  }
  for (int e = tid; e < Rq * 64; e += blockDim.x) {
    const int r = e >> 6, c = e & 63;
    if (c < nb) a.A[(int64_t)(r0 + r) * a.lda + a.k0 + c] = P[r * kPanelLd + c];
  }
  if (a.A2) {
    // the trailing rows as the tensor-core update's A operand: real and minus
    // imaginary parts of L21 interleaved (j = 2 t + f), split into tf32 hi
    // and lo planes P floats apart, zero beyond the panel's 2 nb columns
    for (int e = tid; e < Rq * a.P; e += blockDim.x) {
      const int r = e / a.P, j = e - r * a.P, t = j >> 1;
      const int row = r0 + r - (a.k0 + nb);
      if (row < 0) continue;
      float hi = 0.f, lo = 0.f;
      if (t < nb) {
        const cx<T> L = P[r * kPanelLd + t];
        const float v = (j & 1) ? -(float)L.im : (float)L.re;
        hi = tf32_rna(v);
        lo = tf32_rna(v - hi);
      }
      a.A2[(int64_t)row * 2 * a.P + j] = hi;
      a.A2[(int64_t)row * 2 * a.P + a.P + j] = lo;
    }
  }
  // no CTA leaves while a peer may still store into its shared memory
  cluster_sync_all();
}

// The panel's row interchanges applied to the columns outside it, fused with
// U12 = L11^-1 A12 on the columns to its right (L11 unit lower). A CTA owns
// 32 columns: it gathers the rows the interchanges touch into shared memory
// (lane = column), writes them to their final rows, and on the right-hand
// columns runs the forward substitution with 8 lanes per column, each lane
// holding W / 8 of the w <= W panel rows (rows l, l + 8, ...): at step t the
// lane of row t passes x[t] to the other 7 by a shuffle. Every element
// takes its subtractions in the order t = 0, 1, ... as in LAPACK's ztrsm.
// The interchanges are composed, not replayed: the rows touched are the w
// panel rows and the pivot rows below the panel, and the original row that
// ends in position x is found by applying the swaps to x in reverse order.
// (LAPACK zgetrf applies the same swaps one by one through zlaswp.)
// The CTAs cover the columns vc_begin <= vc < vc_end counted without the
// panel's (vc < k0: column vc, else column vc + w). W = 128 serves a block
// of two 64-column panels whose interchanges and L11 are taken together.
constexpr int kSwapMaxW = 64;
constexpr int kSwapLd = 33;  // row stride of the gathered rows (complex elements)

constexpr int kLsLd = 65;  // row stride of a 64 x 64 block of L11 in shared memory (complex elements)

// shared memory: W / 64 blocks of L11 (64 x 64, transposed) and the W gathered rows
template <class T, int W = kSwapMaxW>
__host__ __device__ constexpr size_t swap_trsm_smem() {
  return sizeof(cx<T>) * ((size_t)(W / 64) * 64 * kLsLd + (size_t)W * kSwapLd);
}

// Lb[t * kLsLd + r] = L11[r0 + r][c0 + t] for r0 + r < w (strictly below the
// diagonal on a diagonal block), zero elsewhere; rows of A read coalesced
template <class T>
__device__ __forceinline__ void load_l_block(cx<T>* Lb, const cx<T>* A, int64_t lda, int k0, int w, int r0, int c0) {
  cx<T> v[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const int e = threadIdx.x + 256 * k, t = e & 63, r = e >> 6;
    const bool keep = r0 + r < w && (r0 != c0 || t < r);
    v[k] = keep ? A[(int64_t)(k0 + r0 + r) * lda + k0 + c0 + t] : cx<T>();
  }
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const int e = threadIdx.x + 256 * k, t = e & 63, r = e >> 6;
    Lb[t * kLsLd + r] = v[k];
  }
}

// ipiv null: no interchanges (the rows are in place already); solve false:
// the interchanges alone, no U12 (and no B2). B2 rows are 2 P floats long
// ([hi | lo] planes of width P); this call writes K positions koff ..
// koff + 2 W - 1 of each plane.
template <class T, int W = kSwapMaxW>
__global__ void __launch_bounds__(256) swap_trsm_kernel(cx<T>* A, int64_t lda, int n, int k0, int w,
                                                        const int32_t* __restrict__ ipiv, float* __restrict__ B2,
                                                        int P, int vc_begin, int vc_end, int koff = 0,
                                                        bool solve = true) {
  static_assert(W == 64 || W == 128, "panel blocks of 64 or 128 columns");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // L11 in 64 x 64 blocks, transposed: for W = 128 first [L11 of rows and
  // columns 0..63 | rows 64..127 x columns 0..63], then rows and columns 64..127
  // in the first buffer
  cx<T>* Ls = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* Ls1 = Ls + (W / 64 - 1) * 64 * kLsLd;
  cx<T>* V = Ls + (W / 64) * 64 * kLsLd;  // the w panel rows of the CTA's columns [W][kSwapLd]
  __shared__ int piv[W], dst[2 * W], src[2 * W];
  __shared__ int nd_s;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int kend = k0 + w;
  const int vc0 = vc_begin + blockIdx.x * 32;  // first column of the CTA, counted without the panel's
  // positions touched: the panel rows, then each pivot row below the panel
  // once (its first occurrence among the panel's pivots, in order); one
  // pivot per thread of the first W / 32 warps
  __shared__ int wcnt[W / 32];
  int pj = -1;
  if (threadIdx.x < W) {
    pj = (int)threadIdx.x < w ? (ipiv ? ipiv[k0 + threadIdx.x] : k0 + (int)threadIdx.x) : -1;
    piv[threadIdx.x] = pj;
  }
  __syncthreads();
  bool fst = false;
  if (threadIdx.x < W && pj >= kend) {
    fst = true;
    for (int q = 0; q < (int)threadIdx.x; ++q)
      if (piv[q] == pj) {
        fst = false;
        break;
      }
  }
  const unsigned fb = __ballot_sync(~0u, fst);
  if (warp < W / 32 && lane == 0) wcnt[warp] = __popc(fb);
  for (int i = threadIdx.x; i < w; i += blockDim.x) dst[i] = k0 + i;
  __syncthreads();
  if (fst) {
    int off = 0;
    for (int u = 0; u < warp; ++u) off += wcnt[u];
    dst[w + off + __popc(fb & ((1u << lane) - 1u))] = pj;
  }
  if (threadIdx.x == 0) {
    int nx = 0;
#pragma unroll
    for (int u = 0; u < W / 32; ++u) nx += wcnt[u];
    nd_s = w + nx;
  }
  // the CTA's columns vc0 .. vc0 + 31 map to vc (< k0) or vc + w (right of the panel)
  const bool any_right = solve && kend < n && min(vc0 + 31, vc_end - 1) >= k0;
  if (any_right) {
    load_l_block(Ls, A, lda, k0, w, 0, 0);
    if (W == 128) load_l_block(Ls1, A, lda, k0, w, 64, 0);
  }
  __syncthreads();
  const int nd = nd_s;
  // the original row of each touched position: the swaps applied to it in
  // reverse order, one position per thread (nd <= 2 W <= the CTA's threads)
  for (int i = threadIdx.x; i < nd; i += blockDim.x) {
    int y = dst[i];
#pragma unroll 4
    for (int j = w - 1; j >= 0; --j) {
      const int r = k0 + j, p = piv[j];
      y = y == r ? p : (y == p ? r : y);
    }
    src[i] = y;
  }
  __syncthreads();
  const int vc = vc0 + lane;
  const bool valid = vc < vc_end;
  const int c = vc < k0 ? vc : vc + w;
  const bool right = solve && c >= kend;
  {
    // warp q gathers rows q, q + 8, ...; every row of the CTA's columns is
    // read before any is written (the barrier), as rows move between warps
    cx<T> v[2 * W / 8];
#pragma unroll
    for (int j = 0; j < 2 * W / 8; ++j) {
      const int i = warp + 8 * j;
      v[j] = valid && i < nd ? A[(int64_t)src[i] * lda + c] : cx<T>();
    }
    if (any_right)
#pragma unroll
      for (int j = 0; j < 2 * W / 8; ++j) {
        const int i = warp + 8 * j;
        if (i < w) V[i * kSwapLd + lane] = v[j];
      }
    __syncthreads();
    // rows that are not solved go straight to their final rows
#pragma unroll
    for (int j = 0; j < 2 * W / 8; ++j) {
      const int i = warp + 8 * j;
      if (valid && i < nd && (i >= w || !right) && src[i] != dst[i]) A[(int64_t)dst[i] * lda + c] = v[j];
    }
  }
  if (!any_right) return;
  {
    constexpr int R = W / 8;  // rows per lane
    const int l8 = lane & 7, col = 4 * warp + (lane >> 3);
    cx<T> x[R];
#pragma unroll
    for (int k = 0; k < R; ++k) x[k] = l8 + 8 * k < w ? V[(l8 + 8 * k) * kSwapLd + col] : cx<T>();
    // rows 0..63 (and, for W = 128, rows 64..127 take their products with
    // them); the loops over a lane's registers are unrolled, the 8 steps
    // within a group of rows are not (a fully unrolled substitution is
    // thousands of instructions, and the warps then wait on instruction fetch)
#pragma unroll
    for (int kb = 0; kb < 8; ++kb)
#pragma unroll 1
      for (int j = 0; j < 8; ++j) {
        const int t = 8 * kb + j;
        cx<T> xt;
        xt.re = __shfl_sync(~0u, x[kb].re, (lane & ~7) | j);
        xt.im = __shfl_sync(~0u, x[kb].im, (lane & ~7) | j);
        // L11 rows >= w and on / above the diagonal are zero in Ls
#pragma unroll
        for (int k = kb; k < 8; ++k)
          if (k > kb || l8 > j) x[k] -= Ls[t * kLsLd + l8 + 8 * k] * xt;
#pragma unroll
        for (int k = 8; k < R; ++k) x[k] -= Ls1[t * kLsLd + l8 + 8 * (k - 8)] * xt;
      }
    if (W == 128) {
      // rows 64..127 with their own diagonal block, loaded over the first one
      __syncthreads();
      load_l_block(Ls, A, lda, k0, w, 64, 64);
      __syncthreads();
#pragma unroll
      for (int kb = 8; kb < R; ++kb)
#pragma unroll 1
        for (int j = 0; j < 8; ++j) {
          const int t = 8 * (kb - 8) + j;
          cx<T> xt;
          xt.re = __shfl_sync(~0u, x[kb].re, (lane & ~7) | j);
          xt.im = __shfl_sync(~0u, x[kb].im, (lane & ~7) | j);
#pragma unroll
          for (int k = kb; k < R; ++k)
            if (k > kb || l8 > j) x[k] -= Ls[t * kLsLd + l8 + 8 * (k - 8)] * xt;
        }
    }
#pragma unroll
    for (int k = 0; k < R; ++k)
      if (l8 + 8 * k < w) V[(l8 + 8 * k) * kSwapLd + col] = x[k];
  }
  __syncthreads();
  if (valid && right)
#pragma unroll
    for (int j = 0; j < W / 8; ++j) {
      const int i = warp + 8 * j;
      if (i < w) A[(int64_t)(k0 + i) * lda + c] = V[i * kSwapLd + lane];
    }
  if (B2) {
    // U12 as the tensor-core update's B operand: for trailing column cc the
    // rows 2 cc (re, im) and 2 cc + 1 (im, -re) of (U, -iU), K-major, split
    // into tf32 hi and lo planes P floats apart, zero beyond 2 w
    for (int row = warp; row < 64; row += 8) {  // row = 2 x (column of the CTA) + part
      const int cl = row >> 1, part = row & 1;
      const int vcl = vc0 + cl;
      if (vcl >= vc_end || vcl < k0) continue;  // not a trailing column
      const int cc = vcl - k0;                  // = (vcl + w) - kend
      for (int jj = lane; jj < 2 * W; jj += 32) {
      const int t = jj >> 1, f = jj & 1;
      float hi = 0.f, lo = 0.f;
      if (t < w) {
        const cx<T> U = V[t * kSwapLd + cl];
        const float v = part == 0 ? (f == 0 ? (float)U.re : (float)U.im) : (f == 0 ? (float)U.im : -(float)U.re);
        hi = tf32_rna(v);
        lo = tf32_rna(v - hi);
      }
      B2[(int64_t)(2 * cc + part) * 2 * P + koff + jj] = hi;
      B2[(int64_t)(2 * cc + part) * 2 * P + P + koff + jj] = lo;
      }
    }
  }
}

// C[r][c] -= sum_t Lp[r][t] Up[t][c] over rows / cols >= off, t < nb:
// 64 x 64 tile per CTA, 4 x 4 complex outputs per thread.
template <class T>
__global__ void __launch_bounds__(256) gemm_kernel(cx<T>* A, int64_t lda, int n, int k0, int nb) {
  const int off = k0 + nb;
  const int row0 = off + blockIdx.y * 64, col0 = off + blockIdx.x * 64;
  __shared__ cx<T> As[16][64 + 1];
  __shared__ cx<T> Bs[16][64];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  cx<T> acc[4][4];
  for (int t0 = 0; t0 < nb; t0 += 16) {
    for (int e = threadIdx.x; e < 16 * 64; e += 256) {
      int r = e >> 4, t = e & 15;  // As[t][r] = L[row0 + r][k0 + t0 + t]
      int gr = row0 + r, gt = t0 + t;
      As[t][r] = (gr < n && gt < nb) ? A[(int64_t)gr * lda + k0 + gt] : cx<T>();
      int t2 = e >> 6, c = e & 63;  // Bs[t][c] = U[k0 + t0 + t][col0 + c]
      int gc = col0 + c, gt2 = t0 + t2;
      Bs[t2][c] = (gc < n && gt2 < nb) ? A[(int64_t)(k0 + gt2) * lda + gc] : cx<T>();
    }
    __syncthreads();
#pragma unroll 4
    for (int t = 0; t < 16; ++t) {
      cx<T> a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[t][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[t][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          acc[i][j].re += a[i].re * b[j].re - a[i].im * b[j].im;
          acc[i][j].im += a[i].re * b[j].im + a[i].im * b[j].re;
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int r = row0 + ty + 16 * i, c = col0 + tx + 16 * j;
      if (r < n && c < n) A[(int64_t)r * lda + c] -= acc[i][j];
    }
}

// perm from the interchange list: perm[i] = the original row that ends in
// row i after the interchanges (sequential in shared memory, one thread;
// built once per factorisation)
// STAGE: ipiv is first copied to shared memory, so that the serial loop of
// swaps reads no global memory (n <= 25600)
template <bool STAGE>
__global__ void perm_kernel(int n, const int32_t* __restrict__ ipiv, int32_t* __restrict__ perm_out) {
  extern __shared__ int perm[];
  int* piv = perm + n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    perm[i] = i;
    if (STAGE) piv[i] = ipiv[i];
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int i = 0; i < n; ++i) {
      int p = STAGE ? piv[i] : ipiv[i];
      if (p != i && p >= 0 && p < n) {
        int t = perm[i];
        perm[i] = perm[p];
        perm[p] = t;
      }
    }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) perm_out[i] = perm[i];
}

// Bp[i] = B[perm[i]] for every right-hand side
template <class T>
__global__ void gather_rows_kernel(int n, int nrhs, const int32_t* __restrict__ perm, const cx<T>* __restrict__ B,
                                   cx<T>* __restrict__ Bp) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)n * nrhs) return;
  int i = int(e / nrhs), c = int(e % nrhs);
  Bp[e] = B[(int64_t)perm[i] * nrhs + c];
}

// ----------------------------------------------------------------- drivers
// lu_tc.cu
int lu_tc_prepare(m25_ctx* ctx, int n);
int lu_tc_buffers(m25_ctx* ctx, int n, float** A3, float** B3, float** Ai, float** Bi);
int lu_tc_pack_a(m25_ctx* ctx, const zf* A, int64_t lda, int k0, int w, int row0, int m, int P, int pw, int koff,
                 float* A3);
int lu_tc_update(m25_ctx* ctx, zf* A, int64_t lda, int r0, int c0, int m, int nc, int P, int pw, const float* A3,
                 const float* B3, int slot);
int lu_tc_error(m25_ctx* ctx, int* flag);
bool lu_tc_available();

template <class T>
int lu_factor(m25_ctx* ctx, cx<T>* A, int64_t lda, int n, int32_t* ipiv, int nb, bool use_tc, int* info_host) {
  cudaStream_t st = ctx->stream;
  // the tensor-core update reduces into C through a TMA tensor map: rows of
  // a multiple of 16 bytes and a 16-byte aligned matrix (else SIMT updates)
  use_tc = use_tc && std::is_same<T, float>::value && lda % 2 == 0 && reinterpret_cast<uintptr_t>(A) % 16 == 0 &&
           nb == kSwapMaxW;
  // panel workspace
  int bps_max = 0;
  size_t panel_smem = 0;
  int G = 0, rows = 0;
  const size_t extra = (size_t)nb * sizeof(cx<T>);
  // pick the widest grid whose slices fit: rows_per_cta = ceil(m / G)
  auto fits = [&](int g, int m, size_t& smem) {
    int rpc = (m + g - 1) / g;
    smem = (size_t)rpc * nb * sizeof(cx<T>) + extra;
    return smem <= 200 * 1024;
  };
  M25_CUDA(cudaFuncSetAttribute(panel_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
  if (nb > kSwapMaxW) {
    set_error("dense LU: panel width above 64");
    return M25_ERR_VALUE;
  }
  M25_CUDA(cudaFuncSetAttribute(swap_trsm_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)swap_trsm_smem<T>()));
  if constexpr (std::is_same<T, float>::value)
    M25_CUDA(cudaFuncSetAttribute(swap_trsm_kernel<T, 128>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)swap_trsm_smem<T, 128>()));
  (void)bps_max;
  (void)rows;
  int Gmax = ctx->ext_scratch ? ctx->ext_gmax : 4 * ctx->num_sms;
  char* base = ctx->ext_scratch;
  if (!base) {
    int rc = ctx->scratch.ensure(sizeof(cx<T>) * 2 * (size_t)Gmax * nb + sizeof(T) * 2 * Gmax +
                                 sizeof(int) * 2 * Gmax + sizeof(cx<T>) * 2 * nb + 64);
    if (rc) return rc;
    base = ctx->scratch.as<char>();
  }
  unsigned* bar = reinterpret_cast<unsigned*>(base);
  int* err = reinterpret_cast<int*>(base + 8);
  int* info = reinterpret_cast<int*>(base + 12);
  cx<T>* cand = reinterpret_cast<cx<T>*>(base + 64);
  T* candval = reinterpret_cast<T*>(cand + 2 * (size_t)Gmax * nb);
  int* candidx = reinterpret_cast<int*>(candval + 2 * Gmax);
  cx<T>* rowj = reinterpret_cast<cx<T>*>(candidx + 2 * Gmax);
  M25_CUDA(cudaMemsetAsync(base, 0, 64, st));
  if (use_tc) {
    int rc = lu_tc_prepare(ctx, n);
    if (rc) return rc;
  }
  // the cluster panel: the smallest cluster (4, 8 or 16 CTAs) whose shared
  // memory holds the trailing rows; the exchange per column grows with the
  // square of the cluster size, and small clusters are easier to place next
  // to the kernels of concurrent sweeps
  int cl_rows[3] = {0, 0, 0};  // rows that fit in clusters of 4, 8, 16
  {
    int optin = 0;
    M25_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
    const size_t avail = (size_t)optin - 1024;  // static shared variables
    auto rows_of = [&](size_t smem0) {
      return nb > 64 ? 0 : (int)((avail - smem0) / ((size_t)kPanelLd * sizeof(cx<T>)));
    };
    // decided once (thread-safe initialisation: sweeps on several threads)
    static const bool ok = [avail] {
      bool yes = false;
      const char* off = getenv("M25_NO_CLUSTER_PANEL");
      if (!(off && *off == '1') &&
          cudaFuncSetAttribute(panel_cluster_kernel<T, 16>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
              cudaSuccess &&
          cudaFuncSetAttribute(panel_cluster_kernel<T, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)avail) ==
              cudaSuccess &&
          cudaFuncSetAttribute(panel_cluster_kernel<T, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)avail) ==
              cudaSuccess &&
          cudaFuncSetAttribute(panel_cluster_kernel<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)avail) ==
              cudaSuccess) {
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = 16;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(16);
        cfg.blockDim = dim3(kPanelThreads);
        cfg.dynamicSmemBytes = avail;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nclusters = 0;
        yes = cudaOccupancyMaxActiveClusters(&nclusters, panel_cluster_kernel<T, 16>, &cfg) == cudaSuccess &&
              nclusters > 0;
      }
      cudaGetLastError();  // a refused attribute only means: no cluster panel
      return yes;
    }();
    // M25_PANEL_CLUSTER_MIN: the smallest cluster size used (4, 8 or 16; a tuning knob)
    static const int cl_min_env = [] {
      const char* e = getenv("M25_PANEL_CLUSTER_MIN");
      const int v = e ? atoi(e) : 4;
      return v >= 16 ? 16 : v >= 8 ? 8 : 4;
    }();
    // the context's setting (m25_ctx_set_tuning) over the process default
    const int cl_min = ctx->tune_cluster_min >= 16 ? 16
                       : ctx->tune_cluster_min >= 8 ? 8
                       : ctx->tune_cluster_min > 0  ? 4
                                                    : cl_min_env;
    if (ok) {
      cl_rows[0] = cl_min <= 4 ? 4 * rows_of(cluster_panel_smem<T, 4>(0)) : 0;
      cl_rows[1] = cl_min <= 8 ? 8 * rows_of(cluster_panel_smem<T, 8>(0)) : 0;
      cl_rows[2] = 16 * rows_of(cluster_panel_smem<T, 16>(0));
    }
  }
  // one panel of w <= nb columns at k0 over the rows k0 .. n - 1; A2 / P2:
  // the tensor-core operand planes of its trailing rows (cluster panel only),
  // *packed tells whether they were written
  auto run_panel = [&](int k0, int w, float* A2, int P2, bool* packed) -> int {
    const int m = n - k0;
    const int CL = m <= cl_rows[0] ? 4 : m <= cl_rows[1] ? 8 : m <= cl_rows[2] ? 16 : 0;
    if (packed) *packed = CL > 0 && A2;
    if (CL > 0) {
      ClusterPanelArgs<T> ca{A, lda, n, k0, w, (m + CL - 1) / CL, ipiv, info, err, A2, P2};
      const size_t smem = CL == 4    ? cluster_panel_smem<T, 4>(ca.rows_per_cta)
                          : CL == 8 ? cluster_panel_smem<T, 8>(ca.rows_per_cta)
                                    : cluster_panel_smem<T, 16>(ca.rows_per_cta);
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = CL;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.gridDim = dim3(CL);
      cfg.blockDim = dim3(kPanelThreads);
      cfg.dynamicSmemBytes = smem;
      cfg.stream = st;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      StageTimer tm(ctx, ST_PANEL);
      if (CL == 4) M25_CUDA(cudaLaunchKernelEx(&cfg, panel_cluster_kernel<T, 4>, ca));
      else if (CL == 8) M25_CUDA(cudaLaunchKernelEx(&cfg, panel_cluster_kernel<T, 8>, ca));
      else M25_CUDA(cudaLaunchKernelEx(&cfg, panel_cluster_kernel<T, 16>, ca));
      return M25_OK;
    }
    // grid size: as many CTAs as can be co-resident, each with >= 1 row
    int occ = 0;
    G = std::min(std::min(m, ctx->num_sms), Gmax);
    // M25_PANEL_CTAS: fixed panel grid (a tuning knob; 0 or unset = automatic)
    static const int forced = getenv("M25_PANEL_CTAS") ? atoi(getenv("M25_PANEL_CTAS")) : 0;
    if (forced > 0) G = std::min(std::min(m, forced), Gmax);
    fits(G, m, panel_smem);
    // fewest CTAs (one per SM) whose row slices fit: the per-column barrier
    // and pivot reduction cost grow with the grid
    for (int bps = 1; bps <= 4 && forced <= 0; ++bps) {
      int g = std::min(m, bps * ctx->num_sms);
      size_t smem;
      if (g > Gmax || !fits(g, m, smem)) continue;
      M25_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, panel_kernel<T>, 256, smem));
      if (occ * ctx->num_sms >= g) {
        G = g;
        panel_smem = smem;
        break;
      }
    }
    if (!fits(G, m, panel_smem)) {
      set_error("dense LU: matrix too large for the panel slices in shared memory");
      return M25_ERR_VALUE;
    }
    M25_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, panel_kernel<T>, 256, panel_smem));
    if (occ * ctx->num_sms < G) {
      set_error("dense LU: cooperative panel grid does not fit on the device");
      return M25_ERR_VALUE;
    }
    PanelArgs<T> pa;
    pa.A = A;
    pa.lda = lda;
    pa.n = n;
    pa.k0 = k0;
    pa.nb = w;
    pa.rows_per_cta = (m + G - 1) / G;
    pa.ipiv = ipiv;
    pa.cand = cand;
    pa.candval = candval;
    pa.candidx = candidx;
    pa.rowj = rowj;
    pa.bar = bar;
    pa.err = err;
    pa.info = info;
    void* args[] = {&pa};
    StageTimer tm(ctx, ST_PANEL);
    M25_CUDA(cudaLaunchCooperativeKernel((void*)panel_kernel<T>, dim3(G), dim3(256), args, panel_smem, st));
    return M25_OK;
  };
  // interchanges of the panel at k0 (width w) on the columns vc_begin <= vc <
  // vc_end (counted without the panel's), U12 on those right of it
  auto swap_trsm = [&](int k0, int w, int vc_begin, int vc_end, float* B2, int P2) -> int {
    if (vc_end <= vc_begin) return M25_OK;
    StageTimer tm(ctx, ST_TRSM);
    swap_trsm_kernel<T><<<(vc_end - vc_begin + 31) / 32, 256, swap_trsm_smem<T>(), st>>>(A, lda, n, k0, w, ipiv, B2,
                                                                                         P2, vc_begin, vc_end, 0, true);
    M25_CHECK_LAUNCH();
    return M25_OK;
  };
  // the same for a block of w <= 128 columns (two panels' interchanges and a
  // 128-row L11 at once): piv null skips the interchanges, solve false skips
  // U12; B planes of width P at K offset koff
  auto swap_trsm128 = [&](int k0, int w, int vc_begin, int vc_end, float* B2, int P, int koff, const int32_t* piv,
                          bool solve) -> int {
    if (vc_end <= vc_begin) return M25_OK;
    StageTimer tm(ctx, ST_TRSM);
    swap_trsm_kernel<T, 128><<<(vc_end - vc_begin + 31) / 32, 256, swap_trsm_smem<T, 128>(), st>>>(
        A, lda, n, k0, w, piv, B2, P, vc_begin, vc_end, koff, solve);
    M25_CHECK_LAUNCH();
    return M25_OK;
  };
  int rc = M25_OK;
  if (!use_tc) {
    // right-looking: panel, interchanges and U12, SIMT update of the trailing matrix
    for (int k0 = 0; k0 < n; k0 += nb) {
      const int w = std::min(nb, n - k0);
      if ((rc = run_panel(k0, w, nullptr, 0, nullptr))) return rc;
      if ((rc = swap_trsm(k0, w, 0, n - w, nullptr, 0))) return rc;
      if (k0 + w < n) {
        const int ncol = n - k0 - w;
        StageTimer tm(ctx, ST_GEMM);
        dim3 grid((ncol + 63) / 64, (ncol + 63) / 64);
        gemm_kernel<T><<<grid, 256, 0, st>>>(A, lda, n, k0, w);
        M25_CHECK_LAUNCH();
      }
    }
  } else if constexpr (std::is_same<T, float>::value) {
    // super-blocks of 256 columns: two blocks a, b of 128, each factored as
    // two panels of 64 (the first panel's rank-64 update of the second's
    // columns). Block a's interchanges and U_a = L_aa^-1 A_a go to every
    // column right of it, its rank-128 update only to block b's columns;
    // block b is factored; on the trailing columns then block b's
    // interchanges, its rows minus L_ba U_a, U_b = L_bb^-1 of those rows, and
    // one rank-256 update of the trailing matrix: its read-modify-write of C,
    // the bound of the update, once per 256 columns. B3 holds U_a at K
    // 0..255 and U_b at K 256..511 of planes 512 floats wide, for the columns
    // from the first right of block a (block b's, then the trailing ones).
    float *A3, *B3, *Ai, *Bi;
    if ((rc = lu_tc_buffers(ctx, n, &A3, &B3, &Ai, &Bi))) return rc;
    constexpr int kHalf = kSwapMaxW, kBlock = 2 * kSwapMaxW, kSuper = 2 * kBlock, kPW = 2 * kSuper;
    int slot = 0;
    // one block of W <= 128 columns at c0: both panels, the first one's U12
    // and rank-64 update on the second one's columns, each panel's
    // interchanges on every column left of it (none on columns right of the block)
    auto factor_block = [&](int c0, int W) -> int {
      const int w1 = std::min(kHalf, W), w2 = W - w1;
      bool packed = false;
      int r;
      if ((r = run_panel(c0, w1, w2 > 0 ? Ai : nullptr, 128, &packed))) return r;
      if (w2 == 0) return swap_trsm(c0, w1, 0, c0, nullptr, 0);
      if ((r = swap_trsm(c0, w1, 0, c0 + w2, Bi, 128))) return r;
      const int m1 = n - c0 - w1;
      if (!packed && (r = lu_tc_pack_a(ctx, A, lda, c0, w1, c0 + w1, m1, 128, 128, 0, Ai))) return r;
      if ((r = lu_tc_update(ctx, A, lda, c0 + w1, c0 + w1, m1, w2, 128, 128, Ai, Bi, slot++))) return r;
      if ((r = run_panel(c0 + w1, w2, nullptr, 0, nullptr))) return r;
      return swap_trsm(c0 + w1, w2, 0, c0 + w1, nullptr, 0);
    };
    for (int k0 = 0; k0 < n; k0 += kSuper) {
      const int SW = std::min(kSuper, n - k0), wa = std::min(kBlock, SW), wb = SW - wa;
      if ((rc = factor_block(k0, wa))) return rc;
      const int ra = k0 + wa;  // first column (and row) right of block a
      if (ra >= n) break;      // (then wb = 0)
      // block a's interchanges and U_a on every column right of it
      if ((rc = swap_trsm128(k0, wa, k0, n - wa, B3, kPW, 0, ipiv, true))) return rc;
      // block a's rank-128 update of block b's columns
      if ((rc = lu_tc_pack_a(ctx, A, lda, k0, wa, ra, n - ra, 2 * kBlock, kPW, 0, A3))) return rc;
      if ((rc = lu_tc_update(ctx, A, lda, ra, ra, n - ra, wb, 2 * kBlock, kPW, A3, B3, slot++))) return rc;
      if ((rc = factor_block(ra, wb))) return rc;
      const int t0 = k0 + SW, nt = n - t0;  // the trailing columns
      if (nt <= 0) continue;
      float* Bt = B3 + (size_t)2 * wb * 2 * kPW;  // B rows of the trailing columns
      // block b's interchanges on the trailing columns
      if ((rc = swap_trsm128(ra, wb, ra, ra + nt, nullptr, 0, 0, ipiv, false))) return rc;
      // block b's rows of the trailing columns minus L_ba U_a
      if ((rc = lu_tc_pack_a(ctx, A, lda, k0, wa, ra, wb, 2 * kBlock, kPW, 0, A3))) return rc;
      if ((rc = lu_tc_update(ctx, A, lda, ra, t0, wb, nt, 2 * kBlock, kPW, A3, Bt, slot++))) return rc;
      // U_b = L_bb^-1 of those rows, its B planes at K 256..511
      if ((rc = swap_trsm128(ra, wb, ra, ra + nt, Bt, kPW, 2 * kBlock, nullptr, true))) return rc;
      // the rank-256 update of the trailing matrix
      if ((rc = lu_tc_pack_a(ctx, A, lda, k0, SW, t0, nt, kPW, kPW, 0, A3))) return rc;
      if ((rc = lu_tc_update(ctx, A, lda, t0, t0, nt, nt, kPW, kPW, A3, Bt, slot++))) return rc;
    }
  }
  int hflags[3];
  M25_CUDA(cudaMemcpyAsync(hflags, base + 8, 8, cudaMemcpyDeviceToHost, st));
  M25_CUDA(cudaStreamSynchronize(st));
  if (hflags[0]) {
    set_error("dense LU: a wait of the panel factorisation ran out");
    return M25_ERR_CUDA;
  }
  if (use_tc) {
    int tcerr = 0;
    int rc = lu_tc_error(ctx, &tcerr);
    if (rc) return rc;
    if (tcerr) {
      set_error("dense LU: a wait of the tensor-core update ran out");
      return M25_ERR_CUDA;
    }
  }
  *info_host = hflags[1];
  return M25_OK;
}

constexpr long long kFlagSpinLimit = 1LL << 24;  // bounded wait on a block's ready flag

template <class TF, class TV>
struct WaveArgs {
  const cx<TF>* A;
  int64_t lda;
  int n, nrhs, upper;
  cx<TV>* X;       // in: permuted right-hand sides; out: the solution of this sweep
  int* flags;      // (nblk) == epoch once block k of X is final (complex128 vectors)
  int epoch;
  int* err;        // a wait ran out
  long long spins; // polls per wait before it gives up
  // complex64 vectors: the solved values published with the sweep's epoch in
  // every 8-byte word, (epoch << 32) | bits of re, then the same for im, so
  // a reader can poll the data itself (aligned 8-byte accesses are single-copy
  // atomic); replaces the ready flags and their fences
  unsigned long long* Yt;
};

// asynchronous global -> shared copy of one element (8 or 16 bytes); a
// column outside the matrix is zero-filled without reading global memory
template <int BYTES>
__device__ __forceinline__ void cp_async_elem(void* dst, const void* src, bool valid) {
  unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  int n = valid ? BYTES : 0;
  if (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(n));
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(n));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

constexpr int kTileLd = 65;  // padded row of a 64-wide tile in shared memory

// fetch the w x 64 tile at (r0, c0) (columns >= wc zero) into a (64, 65) shared buffer; one commit group
template <class TF>
__device__ __forceinline__ void fetch_tile(cx<TF>* dst, const cx<TF>* A, int64_t lda, int r0, int c0, int w, int wc) {
  for (int e = threadIdx.x; e < w * 64; e += blockDim.x) {
    int r = e >> 6, c = e & 63;
    const cx<TF>* src = A + (int64_t)(r0 + r) * lda + c0 + (c < wc ? c : 0);
    cp_async_elem<sizeof(cx<TF>)>(&dst[r * kTileLd + c], src, c < wc);
  }
  cp_async_commit();
}

// the diagonal w x w tile at (r0, r0), transposed: DgT[c * 65 + r] = A[r0 + r][r0 + c]; one commit group
template <class TF>
__device__ __forceinline__ void fetch_diag_t(cx<TF>* DgT, const cx<TF>* A, int64_t lda, int r0, int w) {
  for (int e = threadIdx.x; e < w * 64; e += blockDim.x) {
    int r = e >> 6, c = e & 63;
    const cx<TF>* src = A + (int64_t)(r0 + r) * lda + r0 + (c < w ? c : 0);
    cp_async_elem<sizeof(cx<TF>)>(&DgT[c * kTileLd + r], src, c < w);
  }
  cp_async_commit();
}

// Substitution on the diagonal block by one warp for one right-hand side c,
// in registers: lane l owns the rows 2l and 2l + 1, so each round the owner of
// a pair of rows solves both locally and broadcasts them with one round of
// shuffles (32 rounds for 64 rows). DgT is the transposed diagonal tile
// already masked to the triangle of this sweep (zeros elsewhere and outside
// the block), dinv the reciprocal diagonal (zero outside the block), so the
// rounds load factors without any test. Lower: unit diagonal, forward; upper:
// backward. acc (rows x P) in and out, column c.
template <class TF, class TV>
__device__ __forceinline__ void diag_solve1(int lane, int w, int P, int c, int upper, const cx<TF>* DgT,
                                            const cx<TV>* dinv, cx<TV>* acc) {
  const int ra = 2 * lane, rb = ra + 1;
  cx<TV> va = ra < w ? acc[ra * P + c] : cx<TV>();
  cx<TV> vb = rb < w ? acc[rb * P + c] : cx<TV>();
  const int npair = (w + 1) >> 1;
  struct Fac {
    cx<TV> aA, aB, bA, bB, da, db;  // row ra / rb at column 2k / 2k + 1; reciprocal diagonals of the pair
  };
  auto load = [&](int k) {
    Fac f;
    const cx<TF>* ca = DgT + (2 * k) * kTileLd;
    const cx<TF>* cb = ca + kTileLd;
    f.aA = cx<TV>(ca[ra]);
    f.bA = cx<TV>(ca[rb]);
    f.aB = cx<TV>(cb[ra]);
    f.bB = cx<TV>(cb[rb]);
    if (upper) {
      f.da = dinv[2 * k];
      f.db = dinv[2 * k + 1];
    }
    return f;
  };
  if (!upper) {
    Fac nx = load(0);
    for (int k = 0; k < npair; ++k) {
      const Fac f = nx;
      nx = load(min(k + 1, npair - 1));
      const bool mine = lane == k;
      // owner (lane k): x_2k is final, x_2k+1 = v_2k+1 - L[2k+1][2k] x_2k
      const cx<TV> xb_own = vb - f.bA * va;
      const cx<TV> xa(__shfl_sync(0xffffffffu, va.re, k), __shfl_sync(0xffffffffu, va.im, k));
      const cx<TV> xb(__shfl_sync(0xffffffffu, xb_own.re, k), __shfl_sync(0xffffffffu, xb_own.im, k));
      // rows below the pair; the owner keeps the two values it broadcast
      va = mine ? xa : va - (f.aA * xa + f.aB * xb);
      vb = mine ? xb : vb - (f.bA * xa + f.bB * xb);
    }
  } else {
    Fac nx = load(npair - 1);
    for (int k = npair - 1; k >= 0; --k) {
      const Fac f = nx;
      nx = load(max(k - 1, 0));
      const bool mine = lane == k;
      // owner: x_2k+1 = v_2k+1 / d, then x_2k = (v_2k - U[2k][2k+1] x_2k+1) / d
      const cx<TV> xb_own = vb * f.db;
      const cx<TV> xa_own = (va - f.aB * xb_own) * f.da;
      const cx<TV> xa(__shfl_sync(0xffffffffu, xa_own.re, k), __shfl_sync(0xffffffffu, xa_own.im, k));
      const cx<TV> xb(__shfl_sync(0xffffffffu, xb_own.re, k), __shfl_sync(0xffffffffu, xb_own.im, k));
      va = mine ? xa : va - (f.aA * xa + f.aB * xb);
      vb = mine ? xb : vb - (f.bA * xa + f.bB * xb);
    }
  }
  if (ra < w) acc[ra * P + c] = va;
  if (rb < w) acc[rb * P + c] = vb;
}

// tiles in flight per CTA: 4 complex64 or 2 complex128 tiles
template <class TF>
constexpr int wave_stages() {
  return sizeof(cx<TF>) == 8 ? 4 : 2;
}
constexpr int kYtWords = 64 * 8 * 2;  // tagged words of one block of y (64 rows, up to 8 right-hand sides)
template <class TF, class TV>
constexpr size_t wave_smem() {
  return sizeof(cx<TF>) * 64 * kTileLd * (1 + wave_stages<TF>()) + sizeof(cx<TV>) * (64 * 8 * 2 + 64) +
         (sizeof(TV) == 4 ? sizeof(unsigned long long) * kYtWords * wave_stages<TF>() : 0);
}

// One triangular sweep as a dependency wavefront (no grid barriers): CTA g
// owns the 64-row blocks g, g + G, ... For its block i it subtracts the
// tile products A_ij y_j of the blocks j it depends on (j < i for the unit
// lower factor, j > i for the upper one, in the order they become final) as
// soon as block j is flagged final, solves the diagonal block by
// substitution, publishes y_i and raises flag i. The off-diagonal tiles
// stream through a ring of cp.async stages so that a CTA's backlog of tiles
// never holds up the chain; the chain step itself is the flag round trip,
// one 64 x 64 tile product and the substitution, which one warp runs in
// registers (lane l owns rows l and l + 32; each solved row is broadcast with
// shuffles; the upper sweep multiplies by the reciprocal diagonal). Every
// wait is bounded; blocks only wait on blocks solved earlier, and the
// cooperative launch keeps all CTAs resident, so the order cannot deadlock.
template <class TF, class TV>
__global__ void __launch_bounds__(256, 1) trsv_wave_kernel(WaveArgs<TF, TV> a) {
  constexpr int S = wave_stages<TF>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<TF>* Dg = reinterpret_cast<cx<TF>*>(smem_raw);  // (64, 65) diagonal tile, transposed
  cx<TF>* ring = Dg + 64 * kTileLd;                   // S x (64, 65) off-diagonal tiles
  cx<TV>* acc = reinterpret_cast<cx<TV>*>(ring + S * 64 * kTileLd);  // (64, P)
  cx<TV>* y = acc + 64 * 8;                                            // (64, P)
  cx<TV>* dinv = y + 64 * 8;                                           // (64) reciprocal diagonal
  constexpr bool kTagged = sizeof(TV) == 4;
  unsigned long long* yring = reinterpret_cast<unsigned long long*>(dinv + 64);  // S x kYtWords (tagged)
  const unsigned tag = (unsigned)a.epoch;
  __shared__ int fail;
  const int G = gridDim.x, P = a.nrhs, tid = threadIdx.x;
  const int nblk = (a.n + 63) / 64;
  if (tid == 0) fail = 0;
  __syncthreads();
  for (int q = blockIdx.x; q < nblk; q += G) {
    const int i = a.upper ? nblk - 1 - q : q;
    const int r0 = i * 64, w = min(64, a.n - r0);
    // dependencies in the order they become final: j = 0 .. i-1 (lower) or nblk-1 .. i+1 (upper)
    const int ndep = a.upper ? nblk - 1 - i : i;
    auto dep = [&](int d) { return a.upper ? nblk - 1 - d : d; };
    // the tile of dependency d (and, for tagged vectors, the published y_j as
    // it stands now) into ring slot d % S; one commit group per dependency
    auto fetch_dep = [&](int d) {
      const int j = dep(d), wj = min(64, a.n - j * 64);
      if constexpr (kTagged) {
        unsigned long long* ys = yring + (d % S) * kYtWords;
        for (int e = threadIdx.x; e < wj * P; e += blockDim.x)  // 16 bytes = one complex value, L2 only
          cp_async_elem<16>(ys + 2 * e, a.Yt + ((int64_t)j * 64 * P + e) * 2, true);
      }
      fetch_tile(ring + (d % S) * 64 * kTileLd, a.A, a.lda, r0, j * 64, w, wj);
    };
    // commit groups: the diagonal tile, then one per dependency (dependency d is group d + 1)
    fetch_diag_t(Dg, a.A, a.lda, r0, w);
    for (int d = 0; d < S; ++d) {
      if (d < ndep) fetch_dep(d);
      else cp_async_commit();
    }
    for (int e = tid; e < w * P; e += blockDim.x) acc[e] = a.X[(int64_t)r0 * P + e];
    // reciprocal diagonal (zero outside the block), then the tile masked to
    // this sweep's triangle (zero elsewhere); the first step's barrier
    // separates the two, the next barrier publishes the result
    auto prep_diag = [&]() {
      if (tid < 64) {
        cx<TV> di;
        if (a.upper && tid < w) {
          const cx<TV> dd(Dg[tid * kTileLd + tid]);
          const TV m2 = dd.re * dd.re + dd.im * dd.im;
          di = cx<TV>(dd.re / m2, -dd.im / m2);
        }
        dinv[tid] = di;
      }
      __syncthreads();
      for (int e = tid; e < 64 * 64; e += blockDim.x) {
        const int col = e >> 6, r = e & 63;
        const bool keep = r < w && col < w && (a.upper ? r < col : r > col);
        if (!keep) Dg[col * kTileLd + r] = cx<TF>();
      }
    };
    for (int d = 0; d < ndep; ++d) {
      const int j = dep(d), c0 = j * 64, wj = min(64, a.n - c0);
      const cx<TF>* T = ring + (d % S) * 64 * kTileLd;
      if constexpr (kTagged) {
        cp_async_wait<S - 1>();  // tile d and the prefetched y_j have landed
        __syncthreads();
        if (d == 0) prep_diag();  // the diagonal tile (group 0) is in: mask it while the chain runs
        // words of y_j not yet final when prefetched are polled until they carry this sweep's tag
        const unsigned long long* ys = yring + (d % S) * kYtWords;
        bool bad = false;
        for (int e = tid; e < 64 * P * 2; e += blockDim.x) {
          float f = 0.f;
          if (e < wj * P * 2) {
            unsigned long long v = ys[e];
            if ((unsigned)(v >> 32) != tag) {
              const volatile unsigned long long* g = a.Yt + (int64_t)j * 64 * P * 2 + e;
              long long it = 0;
              while (true) {
                v = *g;
                if ((unsigned)(v >> 32) == tag) break;
                if (++it > a.spins || *(volatile int*)a.err) {
                  bad = true;
                  break;
                }
                __nanosleep(20);
              }
            }
            f = __uint_as_float((unsigned)v);
          }
          if (e & 1) y[e >> 1].im = f;
          else y[e >> 1].re = f;
        }
        if (__syncthreads_or(bad)) {
          if (tid == 0) atomicExch(a.err, 1);
          cp_async_wait<0>();
          return;
        }
      } else {
        if (tid == 0) {
          long long it = 0;
          while (*(volatile int*)&a.flags[j] != a.epoch) {
            if (++it > a.spins || *(volatile int*)a.err) {
              atomicExch(a.err, 1);
              fail = 1;
              break;
            }
            __nanosleep(32);
          }
          __threadfence();
        }
        cp_async_wait<S - 1>();  // tile d has landed
        __syncthreads();
        if (d == 0) prep_diag();
        if (fail) {
          cp_async_wait<0>();
          return;
        }
        for (int e = tid; e < 64 * P; e += blockDim.x) {
          if (e < wj * P) {
            volatile cx<TV>* src = &a.X[(int64_t)c0 * P + e];
            y[e] = cx<TV>(src->re, src->im);
          } else {
            y[e] = cx<TV>();
          }
        }
        __syncthreads();
      }
      for (int e = tid; e < w * P; e += blockDim.x) {
        const int r = e / P, c = e % P;
        const cx<TF>* Tr = T + r * kTileLd;
        cx<TV> s0, s1, s2, s3;
#pragma unroll 4
        for (int t = 0; t < 64; t += 4) {
          s0 += cx<TV>(Tr[t]) * y[t * P + c];
          s1 += cx<TV>(Tr[t + 1]) * y[(t + 1) * P + c];
          s2 += cx<TV>(Tr[t + 2]) * y[(t + 2) * P + c];
          s3 += cx<TV>(Tr[t + 3]) * y[(t + 3) * P + c];
        }
        acc[e] -= (s0 + s1) + (s2 + s3);
      }
      __syncthreads();  // the stage of tile d is free again
      if (d + S < ndep) fetch_dep(d + S);
      else cp_async_commit();
    }
    cp_async_wait<0>();
    __syncthreads();
    if (ndep == 0) {
      prep_diag();
      __syncthreads();
    }
    // diagonal block: warp c solves right-hand side c (P <= 8 warps in parallel)
    const int warp = tid >> 5, lane = tid & 31;
    if (warp < P) diag_solve1<TF, TV>(lane, w, P, warp, a.upper, Dg, dinv, acc);
    __syncthreads();
    // publish y_i (warp 0)
    if (tid < 32) {
      if constexpr (kTagged) {
        // publish first (the chain waits on it), then the plain copy for the next sweep
        const unsigned long long hi = (unsigned long long)tag << 32;
        volatile unsigned long long* yt = a.Yt + (int64_t)r0 * P * 2;
        for (int e = lane; e < w * P; e += 32) {
          const cx<TV> v = acc[e];
          yt[2 * e] = hi | __float_as_uint((float)v.re);
          yt[2 * e + 1] = hi | __float_as_uint((float)v.im);
        }
      }
      for (int e = lane; e < w * P; e += 32) a.X[(int64_t)r0 * P + e] = acc[e];
      if constexpr (!kTagged) __threadfence();
    }
    __syncthreads();
    if constexpr (!kTagged) {
      if (tid == 0) atomicExch(&a.flags[i], a.epoch);
    }
  }
}

// perm (n ints, device) of the interchanges in ipiv; once per factorisation
int lu_make_perm(m25_ctx* ctx, int n, const int32_t* ipiv, int32_t* perm) {
  if ((size_t)n * sizeof(int) > 200 * 1024) {
    set_error("dense solve: n <= 51200");
    return M25_ERR_VALUE;
  }
  static const bool attr =
      cudaFuncSetAttribute(perm_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) ==
          cudaSuccess &&
      cudaFuncSetAttribute(perm_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) ==
          cudaSuccess;
  if (!attr) {
    set_error("dense solve: the permutation kernel's shared memory could not be reserved");
    return M25_ERR_CUDA;
  }
  if ((size_t)n * 2 * sizeof(int) <= 200 * 1024)
    perm_kernel<true><<<1, 1024, 2 * n * sizeof(int), ctx->stream>>>(n, ipiv, perm);
  else
    perm_kernel<false><<<1, 1024, n * sizeof(int), ctx->stream>>>(n, ipiv, perm);
  M25_CHECK_LAUNCH();
  return M25_OK;
}

// X = (LU)^-1 P B: the permutation (from ipiv, or the precomputed perm when
// given), then one wavefront launch per factor.
template <class TF, class TV>
int lu_solve_wave(m25_ctx* ctx, const cx<TF>* A, int64_t lda, int n, const int32_t* ipiv, const cx<TV>* B, int nrhs,
                  cx<TV>* X, const int32_t* perm) {
  cudaStream_t st = ctx->stream;
  if (nrhs > 8 || (size_t)n * sizeof(int) > 200 * 1024) {
    set_error("dense solve: at most 8 right-hand sides and n <= 51200");
    return M25_ERR_VALUE;
  }
  const int nblk = (n + 63) / 64;
  // layout: [0] wait error, [16 ..] ready flag per block, then the
  // permutation when it is built here; zeroed whenever the buffer is
  // (re)allocated (a caller-provided buffer comes zeroed)
  // then (complex64 vectors) the tagged copy of y, 16 bytes per value
  const bool tagged = sizeof(TV) == 4;
  const size_t yt_off = ((sizeof(int) * (nblk + 16 + n)) + 255) / 256 * 256;
  int* err = ctx->ext_flags;
  if (tagged && err) {
    set_error("dense solve: complex64 vectors need the context's flag buffer");
    return M25_ERR_VALUE;
  }
  if (!err) {
    void* before = ctx->flags.p;
    int rc = ctx->flags.ensure(yt_off + (tagged ? sizeof(unsigned long long) * 2 * (size_t)n * 8 : 0));
    if (rc) return rc;
    if (ctx->flags_fresh || ctx->flags.p != before) {
      M25_CUDA(cudaMemsetAsync(ctx->flags.p, 0, ctx->flags.bytes, st));
      ctx->flags_fresh = false;
      ctx->epoch = 0;
    }
    err = ctx->flags.as<int>();
  }
  int* flags = err + 16;
  unsigned long long* Yt =
      tagged ? reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(err) + yt_off) : nullptr;
  if (!Yt && ctx->yt_off && sizeof(int) * (nblk + 16 + n) > ctx->yt_off)
    ctx->yt_off = 0;  // this call's permutation reaches into the tagged copy of an earlier one
  if (Yt && ctx->yt_off != yt_off) {
    // the tagged copy moved (another n): what the buffer held there before
    // (permutations, flags) must not pass for a tag of this sweep
    M25_CUDA(cudaMemsetAsync(Yt, 0, sizeof(unsigned long long) * 2 * (size_t)n * 8, st));
    ctx->yt_off = yt_off;
  }
  const size_t sm = wave_smem<TF, TV>();
  M25_CUDA(cudaFuncSetAttribute(trsv_wave_kernel<TF, TV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  int occ = 0;
  M25_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, trsv_wave_kernel<TF, TV>, 256, sm));
  if (occ < 1) {
    set_error("dense solve: the triangular-solve kernel does not fit on an SM");
    return M25_ERR_CUDA;
  }
  // M25_WAVE_CTAS: at most this many CTAs (a tuning knob; 0 or unset = one per block up to the device's fill)
  static const int wave_cap_env = getenv("M25_WAVE_CTAS") ? atoi(getenv("M25_WAVE_CTAS")) : 0;
  const int wave_cap = ctx->tune_wave_ctas > 0 ? ctx->tune_wave_ctas : wave_cap_env;
  const int G = std::min(std::min(nblk, ctx->num_sms * occ), wave_cap > 0 ? wave_cap : nblk);
  StageTimer tm(ctx, ST_TRSV);
  if (!perm) {
    if (ctx->ext_flags) {  // no room for a permutation in a caller-provided flag buffer
      set_error("dense solve: a precomputed permutation is required here");
      return M25_ERR_VALUE;
    }
    int32_t* pbuf = flags + nblk;
    int rc = lu_make_perm(ctx, n, ipiv, pbuf);
    if (rc) return rc;
    perm = pbuf;
  }
  {
    const int64_t tot = (int64_t)n * nrhs;
    gather_rows_kernel<TV><<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(n, nrhs, perm, B, X);
  }
  for (int upper = 0; upper < 2; ++upper) {
    if (++ctx->epoch <= 0) {  // wrapped: start the flags (and tags) afresh
      M25_CUDA(cudaMemsetAsync(flags, 0, sizeof(int) * nblk, st));
      if (Yt) M25_CUDA(cudaMemsetAsync(Yt, 0, sizeof(unsigned long long) * 2 * (size_t)n * 8, st));
      ctx->epoch = 1;
    }
    WaveArgs<TF, TV> wa{A, lda, n, nrhs, upper, X, flags, ctx->epoch, err,
                        ctx->wave_spins > 0 ? ctx->wave_spins : kFlagSpinLimit, Yt};
    void* args[] = {&wa};
    M25_CUDA(cudaLaunchCooperativeKernel((void*)trsv_wave_kernel<TF, TV>, dim3(G), dim3(256), args, sm, st));
  }
  M25_CHECK_LAUNCH();
  return M25_OK;
}

// clear the wait flag of the triangular solves before a solve: a solve whose
// wait ran out left it set, and every later sweep would give up at once
int lu_wave_reset(m25_ctx* ctx) {
  if (ctx->ext_flags) return M25_OK;  // a caller-provided flag buffer is cleared by its owner
  if (ctx->flags.p) M25_CUDA(cudaMemsetAsync(ctx->flags.p, 0, sizeof(int), ctx->stream));
  return M25_OK;
}

// the wait flag of the last sweeps (0: every wait ended in time)
int lu_wave_error(m25_ctx* ctx, int n, int* flag) {
  *flag = 0;
  (void)n;
  const int* src = ctx->ext_flags ? ctx->ext_flags : ctx->flags.as<int>();
  if (!src) return M25_OK;
  M25_CUDA(cudaMemcpyAsync(flag, src, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  M25_CUDA(cudaStreamSynchronize(ctx->stream));
  return M25_OK;
}

template int lu_solve_wave<double, double>(m25_ctx*, const zd*, int64_t, int, const int32_t*, const zd*, int, zd*,
                                           const int32_t*);
template int lu_solve_wave<float, double>(m25_ctx*, const zf*, int64_t, int, const int32_t*, const zd*, int, zd*,
                                          const int32_t*);
template int lu_solve_wave<float, float>(m25_ctx*, const zf*, int64_t, int, const int32_t*, const zf*, int, zf*,
                                         const int32_t*);

template int lu_factor<double>(m25_ctx*, zd*, int64_t, int, int32_t*, int, bool, int*);
template int lu_factor<float>(m25_ctx*, zf*, int64_t, int, int32_t*, int, bool, int*);

// ------------------------------------------------ GMRES iterative refinement
// Right-hand sides are handled in lockstep (one column per rhs).

// ---- fp64-accurate products on the fp32 pipes. GB300's fp64 rate makes an
// fp64 matrix-vector product arithmetic-bound (~0.8 ms at N = 5943); here
// Z is held as two complex64 planes, Z = Zh + Zl (Zl = fp32(Z - Zh)), the
// vectors likewise, and the dot products use the error-free transforms of
// Ogita, Rump & Oishi ("Accurate sum and dot product", 2005): the FMA
// two-product and Knuth's two-sum, with the cross terms Zh Xl + Zl Xh and the
// rounding errors summed in fp32. The result is as accurate as a dot product
// in about 2^-48 relative precision, read from the same HBM bytes as the
// complex128 matrix.
__device__ __forceinline__ void dot2_acc(float& s, float& c, float ah, float al, float bh, float bl) {
  const float p = ah * bh;
  const float ep = fmaf(ah, bh, -p);
  const float t = s + p;
  const float z = t - s;
  const float es = (s - (t - z)) + (p - z);
  s = t;
  c += (ep + es) + fmaf(ah, bl, al * bh);
}

// Y = Z X for ROWS rows per warp; Zl may be absent (LO false: Z is exact in complex64)
template <int P, int ROWS, bool LO>
__global__ void __launch_bounds__(256) matvec_df_kernel(int n, const zf* __restrict__ Zh, const zf* __restrict__ Zl,
                                                        int64_t ldz, const zf* __restrict__ Xh,
                                                        const zf* __restrict__ Xl, zd* __restrict__ Y) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  const int r0 = warp * ROWS;
  if (r0 >= n) return;
  float s[ROWS][P][2], cc[ROWS][P][2];
#pragma unroll
  for (int r = 0; r < ROWS; ++r)
#pragma unroll
    for (int c = 0; c < P; ++c) s[r][c][0] = s[r][c][1] = cc[r][c][0] = cc[r][c][1] = 0.f;
  for (int t = lane; t < n; t += 32) {
    zf xh[P], xl[P];
#pragma unroll
    for (int c = 0; c < P; ++c) {
      xh[c] = Xh[(int64_t)t * P + c];
      xl[c] = Xl[(int64_t)t * P + c];
    }
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
      if (r0 + r >= n) break;
      const zf zh = Zh[(int64_t)(r0 + r) * ldz + t];
      const zf zl = LO ? Zl[(int64_t)(r0 + r) * ldz + t] : zf();
#pragma unroll
      for (int c = 0; c < P; ++c) {
        dot2_acc(s[r][c][0], cc[r][c][0], zh.re, zl.re, xh[c].re, xl[c].re);
        dot2_acc(s[r][c][0], cc[r][c][0], zh.im, zl.im, -xh[c].im, -xl[c].im);
        dot2_acc(s[r][c][1], cc[r][c][1], zh.re, zl.re, xh[c].im, xl[c].im);
        dot2_acc(s[r][c][1], cc[r][c][1], zh.im, zl.im, xh[c].re, xl[c].re);
      }
    }
  }
#pragma unroll
  for (int r = 0; r < ROWS; ++r) {
    if (r0 + r >= n) break;
#pragma unroll
    for (int c = 0; c < P; ++c) {
      double v[2];
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        float a = s[r][c][q], e = cc[r][c][q];
        for (int o = 16; o; o >>= 1) {
          const float b = __shfl_down_sync(0xffffffffu, a, o), f = __shfl_down_sync(0xffffffffu, e, o);
          const float t = a + b, z = t - a;
          e += f + ((a - (t - z)) + (b - z));
          a = t;
        }
        v[q] = (double)a + (double)e;
      }
      if (lane == 0) Y[(int64_t)(r0 + r) * P + c] = zd(v[0], v[1]);
    }
  }
}

// hi / lo complex64 planes of complex128 values: hi = fp32(x), lo = fp32(x - hi)
__global__ void split_z64_kernel(int64_t n, const zd* __restrict__ X, zf* __restrict__ Xh, zf* __restrict__ Xl) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const zd x = X[e];
  const float hr = (float)x.re, hi = (float)x.im;
  Xh[e] = zf(hr, hi);
  Xl[e] = zf((float)(x.re - (double)hr), (float)(x.im - (double)hi));
}

// the same for an n x m block of a matrix (leading dimensions lda / ldb),
// also writing the hi plane to a second destination (the LU's input, ldlu)
// Row equilibration of the mixed solve: rs[r] = 2^-e with max_c |Z[r][c]|
// (|re| + |im|) in [2^(e-1), 2^e): scaling by powers of two is exact, and
// rows of very different size (the via unknowns' rows next to the RWG rows)
// no longer hide the RWG rows' residuals in the normwise backward error.
__global__ void row_scale_kernel(int n, const zd* __restrict__ a, int64_t lda, double* __restrict__ rs) {
  const int r = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (r >= n) return;
  double mx = 0.0;
  for (int c = lane; c < n; c += 32) {
    const zd x = a[(int64_t)r * lda + c];
    mx = fmax(mx, fabs(x.re) + fabs(x.im));
  }
  for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) {
    int e = 0;
    frexp(mx, &e);
    rs[r] = mx > 0.0 && isfinite(mx) ? ldexp(1.0, -e) : 1.0;
  }
}

__global__ void scale_rows_kernel(int64_t n, int P, const double* __restrict__ rs, zd* __restrict__ B) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * P) return;
  const double s = rs[e / P];
  B[e] = zd(B[e].re * s, B[e].im * s);
}

__global__ void split_matrix_kernel(const zd* __restrict__ a, int64_t lda, zf* __restrict__ lu, int64_t ldlu,
                                    zf* __restrict__ h, zf* __restrict__ l, int64_t ldb, int n, int m,
                                    const double* __restrict__ rs) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)n * m) return;
  const int64_t r = e / m, c = e % m;
  zd x = a[r * lda + c];
  if (rs) x = zd(x.re * rs[r], x.im * rs[r]);
  const float hr = (float)x.re, hi = (float)x.im;
  const zf hv(hr, hi);
  lu[r * ldlu + c] = hv;
  h[r * ldb + c] = hv;
  l[r * ldb + c] = zf((float)(x.re - (double)hr), (float)(x.im - (double)hi));
}

// Y = (Zh + Zl) X in fp64-level accuracy; Xw holds the split X (2 n P complex64)
void matvec_df(int n, int P, const zf* Zh, const zf* Zl, int64_t ldz, const zd* X, zf* Xw, zd* Y, cudaStream_t st) {
  const int64_t np = (int64_t)n * P;
  split_z64_kernel<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(np, X, Xw, Xw + np);
  const zf* Xh = Xw;
  const zf* Xl = Xw + np;
#define M25_MVDF(PP, RR)                                                                                       \
  do {                                                                                                         \
    const unsigned g = (unsigned)(((size_t)(n + RR - 1) / RR * 32 + 255) / 256);                               \
    if (Zl)                                                                                                    \
      matvec_df_kernel<PP, RR, true><<<g, 256, 0, st>>>(n, Zh, Zl, ldz, Xh, Xl, Y);                            \
    else                                                                                                       \
      matvec_df_kernel<PP, RR, false><<<g, 256, 0, st>>>(n, Zh, Zl, ldz, Xh, Xl, Y);                           \
  } while (0)
  // one row per warp: enough warps in flight to cover the HBM latency of Z
  switch (P) {
    case 1: M25_MVDF(1, 1); break;
    case 2: M25_MVDF(2, 1); break;
    case 3: M25_MVDF(3, 1); break;
    case 4: M25_MVDF(4, 1); break;
    case 5: M25_MVDF(5, 1); break;
    case 6: M25_MVDF(6, 1); break;
    case 7: M25_MVDF(7, 1); break;
    case 8: M25_MVDF(8, 1); break;
    default: break;  // 1 <= P <= 8 is checked by the callers
  }
#undef M25_MVDF
}

// h[i][c] = sum_t conj(V_i[t][c]) W[t][c] for i < nvec: one CTA per i
__global__ void dots_kernel(int n, int P, const zd* __restrict__ V, int64_t vstride, const zd* __restrict__ W,
                            zd* __restrict__ h) {
  int i = blockIdx.x;
  const zd* Vi = V + (int64_t)i * vstride;
  zd acc[8];
  for (int t = threadIdx.x; t < n; t += blockDim.x)
    for (int c = 0; c < P; ++c) acc[c] += conj(Vi[(int64_t)t * P + c]) * W[(int64_t)t * P + c];
  __shared__ double red[32][2];
  for (int c = 0; c < P; ++c) {
    double re = acc[c].re, im = acc[c].im;
    for (int o = 16; o; o >>= 1) {
      re += __shfl_down_sync(0xffffffffu, re, o);
      im += __shfl_down_sync(0xffffffffu, im, o);
    }
    if ((threadIdx.x & 31) == 0) {
      red[threadIdx.x >> 5][0] = re;
      red[threadIdx.x >> 5][1] = im;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double a = 0, b = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        a += red[w][0];
        b += red[w][1];
      }
      h[i * P + c] = zd(a, b);
    }
    __syncthreads();
  }
}

// W[t][c] -= sum_{i < nvec} V_i[t][c] h[i][c]
__global__ void orth_update_kernel(int n, int P, int nvec, const zd* __restrict__ V, int64_t vstride,
                                   const zd* __restrict__ h, zd* __restrict__ W) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)n * P) return;
  int c = int(e % P);
  zd s = W[e];
  for (int i = 0; i < nvec; ++i) s -= V[(int64_t)i * vstride + e] * h[i * P + c];
  W[e] = s;
}

// per-column squared 2-norms: out[c] (one CTA)
__global__ void norms_kernel(int n, int P, const zd* __restrict__ W, double* __restrict__ out) {
  double acc[8] = {};
  for (int t = threadIdx.x; t < n; t += blockDim.x)
    for (int c = 0; c < P; ++c) acc[c] += norm2(W[(int64_t)t * P + c]);
  __shared__ double red[32];
  for (int c = 0; c < P; ++c) {
    double v = acc[c];
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
      out[c] = s;
    }
    __syncthreads();
  }
}

// out[t][c] = in[t][c] * s[c] (s complex per column)
__global__ void col_scale_kernel(int64_t n, int P, const zd* __restrict__ in, const zd* __restrict__ s,
                                 zd* __restrict__ out) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n * P) out[e] = in[e] * s[e % P];
}

// X[t][c] += sum_i V_i[t][c] y[i][c]
__global__ void combine_kernel(int n, int P, int nvec, const zd* __restrict__ V, int64_t vstride,
                               const zd* __restrict__ y, zd* __restrict__ X) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)n * P) return;
  int c = int(e % P);
  zd s(0.0);
  for (int i = 0; i < nvec; ++i) s += V[(int64_t)i * vstride + e] * y[i * P + c];
  X[e] += s;
}

// max over rows of sum |Z[t][k]| (infinity norm; it only scales the stopping
// test, so fp32 from the hi plane), one warp per row + atomicMax on the bits
__global__ void rownorm_kernel(int n, const zf* __restrict__ Z, int64_t ldz, unsigned long long* __restrict__ out) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n) return;
  float s = 0;
  for (int t = lane; t < n; t += 32) {
    const zf z = Z[(int64_t)warp * ldz + t];
    s += sqrtf(z.re * z.re + z.im * z.im);
  }
  for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if (lane == 0) atomicMax(out, (unsigned long long)__double_as_longlong((double)s));  // s >= 0: bit order = value order
}

// o = a / s and back, s = *sp (a device scalar; 1 when it is not positive)
__global__ void z64_to_z32_scaled(int64_t n, const zd* __restrict__ a, const double* __restrict__ sp,
                                  zf* __restrict__ o) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const double s = *sp > 0 ? 1.0 / *sp : 1.0;
  if (e < n) o[e] = zf(float(a[e].re * s), float(a[e].im * s));
}
__global__ void z32_to_z64_scaled(int64_t n, const zf* __restrict__ a, const double* __restrict__ sp,
                                  zd* __restrict__ o) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const double s = *sp > 0 ? *sp : 1.0;
  if (e < n) o[e] = zd(double(a[e].re) * s, double(a[e].im) * s);
}
__global__ void maxabs_kernel(int64_t n, const zd* __restrict__ a, double* __restrict__ out) {
  double m = 0;
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) m = fmax(m, cabs1(a[e]));
  __shared__ double red[32];
  for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmax(r, red[w]);
    *out = r;
  }
}

// Restarted flexible GMRES in fp64 on Z x = B, right-preconditioned by the
// complex64 LU applied in fp32 arithmetic (GMRES-based iterative refinement,
// Carson & Higham 2017, in its flexible form so that the rounding of the
// fp32 triangular solves does not break the Arnoldi relation: fp64 on this
// GPU is too slow for the serial substitution chains). Orthogonalisation and
// the iterate stay in fp64; the matrix-vector products use Z = Zh + Zl, two
// complex64 planes, with fp64-level accuracy on the fp32 pipes (matvec_df;
// Zl absent when Z is itself complex64). Stops when the normwise backward
// error |r| / (|Z| |x| + |b|) of every column <= tol; max_iter bounds the
// total number of GMRES steps.
int refine(m25_ctx* ctx, int n, int P, const zf* Zh, const zf* Zl, int64_t ldz, const zf* LU, int64_t ldlu,
           const int32_t* ipiv, const zd* B, zd* X, double tol, int max_iter, int* steps) {
  cudaStream_t st = ctx->stream;
  const int m = std::min(30, std::max(1, max_iter));
  const size_t np = (size_t)n * P;
  int rc = ctx->Rw.ensure(sizeof(zd) * np * (2 * m + 3) + sizeof(zf) * np * 4 + sizeof(double) * 64 +
                          sizeof(zd) * (size_t)(m + 2) * P * 2 + sizeof(int32_t) * n);
  if (rc) return rc;
  zd* V = ctx->Rw.as<zd>();           // (m+1) Arnoldi vectors
  zd* Zp = V + np * (m + 1);          // (m) preconditioned directions
  zd* W = Zp + np * m;                // work vector
  zd* R = W + np;                     // residual
  zf* r32 = reinterpret_cast<zf*>(R + np);
  zf* d32 = r32 + np;
  double* dsc = reinterpret_cast<double*>(d32 + np);  // scalars
  zd* hdev = reinterpret_cast<zd*>(dsc + 64);
  zd* ydev = hdev + (size_t)(m + 2) * P;
  zf* xsplit = reinterpret_cast<zf*>(ydev + (size_t)(m + 2) * P);  // (2 n P) hi / lo planes of a vector
  int32_t* perm = reinterpret_cast<int32_t*>(xsplit + 2 * np);       // row permutation of the LU
  const unsigned g1 = (unsigned)((np + 255) / 256);
  const unsigned gw = (unsigned)(((size_t)n * 32 + 255) / 256);
  StageTimer tm(ctx, ST_REFINE);
  // out = (LU32)^-1 in, in fp32 with the input scaled to O(1) by its
  // largest entry (kept on the device: no host round trip)
  double* pscale = dsc + 48;
  auto precond = [&](const zd* in, zd* out) -> int {
    maxabs_kernel<<<1, 1024, 0, st>>>((int64_t)np, in, pscale);
    z64_to_z32_scaled<<<g1, 256, 0, st>>>((int64_t)np, in, pscale, r32);
    int r = lu_solve_wave<float, float>(ctx, LU, ldlu, n, ipiv, r32, P, d32, perm);
    if (r) return r;
    z32_to_z64_scaled<<<g1, 256, 0, st>>>((int64_t)np, d32, pscale, out);
    return M25_OK;
  };
  auto col_norms = [&](const zd* v, std::vector<double>& out) -> int {
    norms_kernel<<<1, 1024, 0, st>>>(n, P, v, dsc);
    out.assign(P, 0.0);
    M25_CUDA(cudaMemcpyAsync(out.data(), dsc, sizeof(double) * P, cudaMemcpyDeviceToHost, st));
    M25_CUDA(cudaStreamSynchronize(st));
    for (auto& x : out) x = sqrt(x);
    return M25_OK;
  };
  auto set_col_scalars = [&](const std::vector<zd>& v) -> int {
    M25_CUDA(cudaMemcpyAsync(ydev, v.data(), sizeof(zd) * v.size(), cudaMemcpyHostToDevice, st));
    return M25_OK;
  };
  if ((rc = lu_make_perm(ctx, n, ipiv, perm))) return rc;
  std::vector<double> bn, rn, xn;
  if ((rc = col_norms(B, bn))) return rc;
  double znorm = 0;
  {
    unsigned long long* zb = reinterpret_cast<unsigned long long*>(dsc + 32);
    M25_CUDA(cudaMemsetAsync(zb, 0, sizeof(unsigned long long), st));
    rownorm_kernel<<<gw, 256, 0, st>>>(n, Zh, ldz, zb);
    M25_CUDA(cudaMemcpyAsync(&znorm, zb, sizeof(double), cudaMemcpyDeviceToHost, st));
    M25_CUDA(cudaStreamSynchronize(st));
  }
  // start from the fp32 solution x0 = M^-1 B
  if ((rc = precond(B, X))) return rc;
  int total = 0;
  double prev_worst = INFINITY;
  std::vector<zd> hh((size_t)(m + 2) * P), H((size_t)(m + 1) * m * P), g((size_t)(m + 1) * P), cs(m * P), sn(m * P);
  for (int outer = 0; outer < 50; ++outer) {
    // R = B - Z X
    matvec_df(n, P, Zh, Zl, ldz, X, xsplit, W, st);
    M25_CUDA(cudaMemcpyAsync(R, B, np * sizeof(zd), cudaMemcpyDeviceToDevice, st));
    if ((rc = set_col_scalars(std::vector<zd>(P, zd(-1.0))))) return rc;
    combine_kernel<<<g1, 256, 0, st>>>(n, P, 1, W, 0, ydev, R);
    if ((rc = col_norms(R, rn))) return rc;
    if ((rc = col_norms(X, xn))) return rc;
    double worst = 0;
    std::vector<double> target(P);
    bool finite = std::isfinite(znorm);
    for (int c = 0; c < P; ++c) {
      double den = znorm * xn[c] + bn[c];
      target[c] = tol * den;
      finite = finite && std::isfinite(rn[c]) && std::isfinite(xn[c]);
      worst = std::max(worst, den > 0 ? rn[c] / den : 0.0);
    }
    if (!finite) {  // an overflow in the complex64 factors or solves: never "converged"
      set_error("mixed solve: non-finite residual or solution (complex64 LU overflow?)");
      return M25_ERR_NUMERIC;
    }
    if (worst <= tol) break;
    const bool stalled = worst > 0.5 * prev_worst;
    if (total >= max_iter || stalled) {
      if (worst <= 1e3 * tol && outer > 0) break;  // at the fp64 floor
      char msg[160];
      snprintf(msg, sizeof msg,
               "mixed solve: GMRES refinement stopped at backward error %.3e (tolerance %.1e) after %d steps",
               worst, tol, total);
      set_error(msg);
      return M25_ERR_NUMERIC;
    }
    prev_worst = worst;
    // V0 = R / |R|
    {
      std::vector<zd> inv(P);
      for (int c = 0; c < P; ++c) inv[c] = zd(rn[c] > 0 ? 1.0 / rn[c] : 0.0);
      if ((rc = set_col_scalars(inv))) return rc;
      col_scale_kernel<<<g1, 256, 0, st>>>((int64_t)n, P, R, ydev, V);
    }
    std::fill(g.begin(), g.end(), zd(0.0));
    for (int c = 0; c < P; ++c) g[c] = zd(rn[c]);
    int k = 0;
    for (; k < m && total < max_iter; ++k, ++total) {
      zd* zk = Zp + np * k;
      if ((rc = precond(V + np * k, zk))) return rc;
      matvec_df(n, P, Zh, Zl, ldz, zk, xsplit, W, st);
      // classical Gram-Schmidt, twice
      std::fill(hh.begin(), hh.end(), zd(0.0));
      for (int pass = 0; pass < 2; ++pass) {
        dots_kernel<<<k + 1, 256, 0, st>>>(n, P, V, (int64_t)np, W, hdev);
        orth_update_kernel<<<g1, 256, 0, st>>>(n, P, k + 1, V, (int64_t)np, hdev, W);
        std::vector<zd> tmp((size_t)(k + 1) * P);
        M25_CUDA(cudaMemcpyAsync(tmp.data(), hdev, sizeof(zd) * tmp.size(), cudaMemcpyDeviceToHost, st));
        M25_CUDA(cudaStreamSynchronize(st));
        for (size_t i = 0; i < tmp.size(); ++i) hh[i] += tmp[i];
      }
      std::vector<double> wn;
      if ((rc = col_norms(W, wn))) return rc;
      {
        std::vector<zd> inv(P);
        for (int c = 0; c < P; ++c) inv[c] = zd(wn[c] > 0 ? 1.0 / wn[c] : 0.0);
        if ((rc = set_col_scalars(inv))) return rc;
        col_scale_kernel<<<g1, 256, 0, st>>>((int64_t)n, P, W, ydev, V + np * (k + 1));
      }
      bool done = true;
      for (int c = 0; c < P; ++c) {
        // column k of the Hessenberg matrix, rotated by the previous Givens rotations
        std::vector<zd> col(k + 2);
        for (int i = 0; i <= k; ++i) col[i] = hh[(size_t)i * P + c];
        col[k + 1] = zd(wn[c]);
        for (int i = 0; i < k; ++i) {
          zd x0 = col[i], x1 = col[i + 1];
          zd cI = cs[(size_t)i * P + c], sI = sn[(size_t)i * P + c];
          col[i] = conj(cI) * x0 + conj(sI) * x1;
          col[i + 1] = -sI * x0 + cI * x1;
        }
        double r = sqrt(norm2(col[k]) + norm2(col[k + 1]));
        zd cN = r > 0 ? col[k] / zd(r) : zd(1.0), sN = r > 0 ? col[k + 1] / zd(r) : zd(0.0);
        cs[(size_t)k * P + c] = cN;
        sn[(size_t)k * P + c] = sN;
        col[k] = zd(r);
        col[k + 1] = zd(0.0);
        for (int i = 0; i <= k; ++i) H[((size_t)i * m + k) * P + c] = col[i];
        zd gk = g[(size_t)k * P + c];
        g[(size_t)k * P + c] = conj(cN) * gk;
        g[(size_t)(k + 1) * P + c] = -sN * gk;
        // right preconditioning: |g_{k+1}| estimates the true residual
        if (cabs(g[(size_t)(k + 1) * P + c]) > 0.25 * target[c]) done = false;
      }
      if (done) {
        ++k;
        ++total;
        break;
      }
    }
    // y = H^-1 g (upper triangular), X += Zp y
    std::vector<zd> y((size_t)k * P, zd(0.0));
    for (int c = 0; c < P; ++c)
      for (int i = k - 1; i >= 0; --i) {
        zd sacc = g[(size_t)i * P + c];
        for (int j = i + 1; j < k; ++j) sacc -= H[((size_t)i * m + j) * P + c] * y[(size_t)j * P + c];
        zd d = H[((size_t)i * m + i) * P + c];
        y[(size_t)i * P + c] = (d.re != 0 || d.im != 0) ? sacc / d : zd(0.0);
      }
    if (k > 0) {
      if ((rc = set_col_scalars(y))) return rc;
      combine_kernel<<<g1, 256, 0, st>>>(n, P, k, Zp, (int64_t)np, ydev, X);
    }
  }
  *steps = total;
  M25_CHECK_LAUNCH();
  return M25_OK;
}



// rs (n doubles, device) or null: the rows are equilibrated by powers of two
// (row_scale_kernel), and the right-hand sides B (n x P) with them
void split_to_z32(m25_ctx* ctx, const zd* a, int64_t lda, zf* lu, int64_t ldlu, zf* h, zf* l, int64_t ldb, int n,
                  int m, double* rs, zd* B, int P) {
  int64_t tot = (int64_t)n * m;
  if (rs) {
    row_scale_kernel<<<(unsigned)(((int64_t)n * 32 + 255) / 256), 256, 0, ctx->stream>>>(n, a, lda, rs);
    scale_rows_kernel<<<(unsigned)(((int64_t)n * P + 255) / 256), 256, 0, ctx->stream>>>(n, P, rs, B);
  }
  split_matrix_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, ctx->stream>>>(a, lda, lu, ldlu, h, l, ldb, n, m, rs);
}

}  // namespace m25

// ------------------------------------------------- allocation-free solve
// Scratch of m25_dense_solve_noalloc: one file-scope device array that every
// GPU loading this library holds until the process exits. Layout: [0, 64)
// barrier words of the panel factorisation, then its candidate pivot rows for
// up to kNoAllocGmax CTAs of 64 columns, then the ready flags of the
// triangular solves, then the row permutation of the factorisation.
namespace {
constexpr int kNoAllocGmax = 192;
constexpr size_t kNoAllocPanelBytes = 64 + sizeof(m25::zd) * 2 * kNoAllocGmax * 64 + sizeof(double) * 2 * kNoAllocGmax +
                                      sizeof(int) * 2 * kNoAllocGmax + sizeof(m25::zd) * 2 * 64;
constexpr size_t kNoAllocFlagsOffset = (kNoAllocPanelBytes + 255) / 256 * 256;
constexpr size_t kNoAllocPermOffset =
    (kNoAllocFlagsOffset + sizeof(int) * (16 + M25_NOALLOC_MAX_N / 64 + 1) + 255) / 256 * 256;
static_assert(kNoAllocPermOffset + sizeof(int) * M25_NOALLOC_MAX_N <= M25_NOALLOC_SCRATCH_BYTES,
              "scratch too small for the declared maximum size");
std::mutex g_noalloc_mu;
constexpr int kMaxDevices = 64;
void* g_noalloc_addr[kMaxDevices] = {};
}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[M25_NOALLOC_SCRATCH_BYTES];

extern "C" int m25_dense_solve_noalloc(int32_t n, int32_t nrhs, void* Z, const void* B, void* X, int32_t* ipiv,
                                       void* stream, int32_t* info) {
  using namespace m25;
  if (!Z || !B || !X || !ipiv || n < 1 || nrhs < 1 || nrhs > 8) {
    set_error("m25_dense_solve_noalloc: null pointer, n < 1 or nrhs outside 1..8");
    return M25_ERR_VALUE;
  }
  if (n > M25_NOALLOC_MAX_N) {
    set_error("m25_dense_solve_noalloc: n = " + std::to_string(n) + " exceeds the maximum " +
              std::to_string(M25_NOALLOC_MAX_N) + " of the static scratch; use m25_dense_solve");
    return M25_ERR_VALUE;
  }
  int dev = 0;
  M25_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("m25_dense_solve_noalloc: device index out of range");
    return M25_ERR_VALUE;
  }
  void* addr = nullptr;
  {
    // once per device, with that device current: the device address of the
    // array (its host-side name is only a stand-in, not a device pointer)
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        set_error(std::string("m25_dense_solve_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        return M25_ERR_CUDA;
      }
      g_noalloc_addr[dev] = p;
    }
    addr = g_noalloc_addr[dev];
  }
  m25_ctx c;  // borrowed stream, no workspace of its own
  c.device = dev;
  c.stream = static_cast<cudaStream_t>(stream);
  M25_CUDA(cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, dev));
  if (c.num_sms > kNoAllocGmax) {
    set_error("m25_dense_solve_noalloc: more SMs than the static panel scratch covers");
    return M25_ERR_VALUE;
  }
  char* base = static_cast<char*>(addr);
  c.ext_scratch = base;
  c.ext_gmax = kNoAllocGmax;
  c.ext_flags = reinterpret_cast<int*>(base + kNoAllocFlagsOffset);
  // the array keeps the previous call's contents: clear the barrier words
  // (lu_factor clears its header) and the ready flags
  M25_CUDA(cudaMemsetAsync(c.ext_flags, 0, sizeof(int) * (16 + (n + 63) / 64), c.stream));
  int zinfo = 0;
  int rc = lu_factor<double>(&c, static_cast<zd*>(Z), n, n, ipiv, 64, false, &zinfo);
  if (rc) return rc;
  if (info) {
    info[0] = 0;
    info[1] = zinfo;
  }
  if (zinfo) {
    set_error("m25_dense_solve_noalloc: exactly singular matrix (zero pivot)");
    return M25_ERR_NUMERIC;
  }
  int32_t* perm = reinterpret_cast<int32_t*>(base + kNoAllocPermOffset);
  if ((rc = lu_make_perm(&c, n, ipiv, perm))) return rc;
  rc = lu_solve_wave<double, double>(&c, static_cast<const zd*>(Z), n, n, ipiv, static_cast<const zd*>(B), nrhs,
                                     static_cast<zd*>(X), perm);
  if (rc) return rc;
  int werr = 0;
  if ((rc = lu_wave_error(&c, n, &werr))) return rc;
  if (werr) {
    set_error("m25_dense_solve_noalloc: a wait of the triangular solve ran out");
    return M25_ERR_CUDA;
  }
  return M25_OK;
}
