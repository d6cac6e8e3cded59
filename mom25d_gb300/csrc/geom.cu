// Frequency-independent fill data on the device (the role of mom25d's
// AssemblyGeometry, Engine/mom25d/solver.py:321-426): per-triangle quadrature
// data, near/mid/far class of every (test block, source triangle) pair and
// the closed-form 1/R integrals of the near pairs.
#include <algorithm>
#include <cstring>
#include <vector>

#include "m25_integrals.cuh"
#include "m25_internal.h"

namespace m25 {

int alloc(std::vector<void*>& list, void** p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    set_error(std::string("cudaMalloc(") + std::to_string(bytes) + " B): " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? M25_ERR_MEMORY : M25_ERR_CUDA;
  }
  list.push_back(*p);
  return M25_OK;
}

void free_all(std::vector<void*>& list) {
  for (void* p : list) cudaFree(p);
  list.clear();
}

int alloc_async(std::vector<void*>& list, void** p, size_t bytes, cudaStream_t st) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMallocAsync(p, bytes, st);
  if (e != cudaSuccess) {
    set_error(std::string("cudaMallocAsync(") + std::to_string(bytes) + " B): " + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? M25_ERR_MEMORY : M25_ERR_CUDA;
  }
  list.push_back(*p);
  return M25_OK;
}

void free_all_async(std::vector<void*>& list, cudaStream_t st) {
  for (void* p : list) cudaFreeAsync(p, st);
  list.clear();
}

// Products and sums written out so that nvcc does not contract them into
// FMAs: the near/mid/far thresholds compare the same rounded values as numpy.
__device__ inline double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ inline double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ inline double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ inline double hyp_rn(double x, double y) { return sqrt(add_rn(mul_rn(x, x), mul_rn(y, y))); }

__global__ void tri_data_kernel(int nt, const double* __restrict__ verts, const int32_t* __restrict__ tri_basis,
                                const double* __restrict__ tri_sign, const double* __restrict__ edge_len,
                                double* __restrict__ cen, TriData<double>* __restrict__ td64,
                                TriData<float>* __restrict__ td32, TriDF* __restrict__ tddf,
                                float4* __restrict__ cen_df) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  double V[3][2];
  for (int v = 0; v < 3; ++v)
    for (int d = 0; d < 2; ++d) V[v][d] = verts[(t * 3 + v) * 2 + d];
  double cx = add_rn(add_rn(V[0][0], V[1][0]), V[2][0]) / 3.0;
  double cy = add_rn(add_rn(V[0][1], V[1][1]), V[2][1]) / 3.0;
  cen[2 * t] = cx;
  cen[2 * t + 1] = cy;
  {
    const float xh = (float)cx, yh = (float)cy;
    cen_df[t] = make_float4(xh, (float)(cx - (double)xh), yh, (float)(cy - (double)yh));
  }
  double e1x = sub_rn(V[1][0], V[0][0]), e1y = sub_rn(V[1][1], V[0][1]);
  double e2x = sub_rn(V[2][0], V[0][0]), e2y = sub_rn(V[2][1], V[0][1]);
  double area = 0.5 * fabs(sub_rn(mul_rn(e1x, e2y), mul_rn(e1y, e2x)));
  // longest edge, |V - roll(V, 1)| per vertex
  double size = 0.0;
  for (int v = 0; v < 3; ++v) {
    int u = (v + 2) % 3;
    size = fmax(size, hyp_rn(sub_rn(V[v][0], V[u][0]), sub_rn(V[v][1], V[u][1])));
  }
  TriData<double> a;
  double rel[3][2];
  for (int v = 0; v < 3; ++v) {
    rel[v][0] = V[v][0] - cx;
    rel[v][1] = V[v][1] - cy;
    a.v[v][0] = rel[v][0];
    a.v[v][1] = rel[v][1];
  }
  for (int k = 0; k < 7; ++k) {
    for (int d = 0; d < 2; ++d) {
      double s = 0.0;
      for (int v = 0; v < 3; ++v) s += tri7_bary(k, v) * rel[v][d];
      a.q7[k][d] = s;
    }
    a.w7[k] = tri7_w(k) * area;
  }
  for (int k = 0; k < 3; ++k) {
    for (int d = 0; d < 2; ++d) {
      double s = 0.0;
      for (int v = 0; v < 3; ++v) s += tri3_bary(k, v) * rel[v][d];
      a.q3[k][d] = s;
    }
    a.w3[k] = (1.0 / 3.0) * area;
  }
  for (int i = 0; i < 3; ++i) {
    int b = tri_basis[3 * t + i];
    double l = b >= 0 ? edge_len[b] : 0.0;
    a.cA[i] = tri_sign[3 * t + i] * l / (2.0 * area);
    a.cV[i] = tri_sign[3 * t + i] * l / area;
  }
  a.area = area;
  a.size = size;
  td64[t] = a;
  TriData<float> f;
  const double* src = reinterpret_cast<const double*>(&a);
  float* dst = reinterpret_cast<float*>(&f);
  for (int i = 0; i < int(sizeof(TriData<double>) / sizeof(double)); ++i) dst[i] = float(src[i]);
  td32[t] = f;
  TriDF g;
  auto split = [](double x, float& h, float& l) {
    h = (float)x;
    l = (float)(x - (double)h);
  };
  for (int v = 0; v < 3; ++v)
    for (int d = 0; d < 2; ++d) split(a.v[v][d], g.vh[v][d], g.vl[v][d]);
  for (int i = 0; i < 3; ++i) {
    split(a.cA[i], g.cAh[i], g.cAl[i]);
    split(a.cV[i], g.cVh[i], g.cVl[i]);
  }
  // the conductor-loss factor of the self pair (frequency-independent; the
  // fill multiplies it by the surface impedance), as the fp64 fill forms it
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double gsum = 0.0;
      for (int k = 0; k < 7; ++k)
        gsum += a.w7[k] * ((a.q7[k][0] - a.v[i][0]) * (a.q7[k][0] - a.v[j][0]) +
                           (a.q7[k][1] - a.v[i][1]) * (a.q7[k][1] - a.v[j][1]));
      split(gsum * a.cA[i] * a.cA[j], g.gzh[i][j], g.gzl[i][j]);
    }
  tddf[t] = g;
}

// class of (test block b, source triangle s): 0 near (< near_factor), 1 mid
// (< far_factor), 2 far, from min over the block of the 3-D centroid distance
// over max(size_test, size_source); counts the near pairs of each block.
__global__ void classify_kernel(int nt, int nblocks, const int32_t* __restrict__ block_tris,
                                const int32_t* __restrict__ tri_layer, const double* __restrict__ level_z,
                                const double* __restrict__ cen, const TriData<double>* __restrict__ td,
                                double near_f, double far_f, int32_t* __restrict__ cls,
                                int32_t* __restrict__ near_count) {
  int b = blockIdx.y;
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  __shared__ double tc[32][3];
  __shared__ int tl_sh;
  __shared__ int cnt;
  if (threadIdx.x < 32) {
    int t = block_tris[b * 32 + threadIdx.x];
    tc[threadIdx.x][0] = t >= 0 ? cen[2 * t] : 0.0;
    tc[threadIdx.x][1] = t >= 0 ? cen[2 * t + 1] : 0.0;
    tc[threadIdx.x][2] = t >= 0 ? td[t].size : -1.0;
    if (threadIdx.x == 0) {
      tl_sh = tri_layer[block_tris[b * 32]];
      cnt = 0;
    }
  }
  __syncthreads();
  if (s < nt) {
    double dz = fabs(level_z[tl_sh] - level_z[tri_layer[s]]);
    double sx = cen[2 * s], sy = cen[2 * s + 1], ss = td[s].size;
    double rel = INFINITY;
    for (int p = 0; p < 32; ++p) {
      if (tc[p][2] < 0) continue;
      double nrm = hyp_rn(sub_rn(tc[p][0], sx), sub_rn(tc[p][1], sy));
      double dist = sqrt(add_rn(mul_rn(nrm, nrm), mul_rn(dz, dz)));
      rel = fmin(rel, dist / fmax(tc[p][2], ss));
    }
    int c = rel < near_f ? 0 : (rel < far_f ? 1 : 2);
    cls[(int64_t)b * nt + s] = -1 - c;  // provisional: -1 near, -2 mid, -3 far
    if (c == 0) atomicAdd(&cnt, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0 && cnt) atomicAdd(&near_count[b], cnt);
}

// Final codes: near pairs get their index into the static-integral store
// (block order, source order within a block), mid -1, far -2.
__global__ void near_index_kernel(int nt, const int64_t* __restrict__ block_off, int32_t* __restrict__ cls,
                                  int2* __restrict__ near_list) {
  int b = blockIdx.x;
  __shared__ int warp_sum[32];
  __shared__ int64_t base;
  if (threadIdx.x == 0) base = block_off[b];
  __syncthreads();
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int s0 = 0; s0 < nt; s0 += blockDim.x) {
    int s = s0 + threadIdx.x;
    int code = s < nt ? cls[(int64_t)b * nt + s] : -3;
    int flag = code == -1;
    unsigned m = __ballot_sync(0xffffffffu, flag);
    int pre = __popc(m & ((1u << lane) - 1));
    if (lane == 0) warp_sum[warp] = __popc(m);
    __syncthreads();
    int off = 0, tot = 0;
    for (int w = 0; w < nw; ++w) {
      if (w < warp) off += warp_sum[w];
      tot += warp_sum[w];
    }
    if (s < nt) {
      if (flag) {
        int64_t idx = base + off + pre;
        cls[(int64_t)b * nt + s] = (int32_t)idx;
        near_list[idx] = make_int2(b, s);
      } else {
        cls[(int64_t)b * nt + s] = code + 1;  // -2 -> -1 mid, -3 -> -2 far
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) base += tot;
    __syncthreads();
  }
}

// Closed-form 1/R parts of the near pairs at the 7 test points of every
// slot of the block: S0 = I0 / 4pi and S1 = ((r - c_s) I0 + I1) / 4pi, the
// first moment taken about the source centroid c_s.
__global__ void static_kernel(int64_t nnear, const int2* __restrict__ near_list,
                              const int32_t* __restrict__ block_tris, const int32_t* __restrict__ tri_layer,
                              const double* __restrict__ level_z, const double* __restrict__ cen,
                              const TriData<double>* __restrict__ td, double* __restrict__ st64,
                              float* __restrict__ st32) {
  int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= nnear * 224) return;
  int64_t idx = gid / 224;
  int m = int(gid % 224);
  int lane = m / 7, k = m % 7;
  int2 bs = near_list[idx];
  int t = block_tris[bs.x * 32 + lane];
  int s = bs.y;
  double S0 = 0, S1x = 0, S1y = 0;
  if (t >= 0) {
    const TriData<double>& A = td[t];
    const TriData<double>& B = td[s];
    double rx = (cen[2 * t] - cen[2 * s]) + A.q7[k][0];
    double ry = (cen[2 * t + 1] - cen[2 * s + 1]) + A.q7[k][1];
    double dz = fabs(level_z[tri_layer[t]] - level_z[tri_layer[s]]);
    double I0, I1x, I1y;
    potential_integrals(B.v, rx, ry, dz, I0, I1x, I1y);
    const double f = 1.0 / (4.0 * kPi);
    S0 = I0 * f;
    S1x = (rx * I0 + I1x) * f;
    S1y = (ry * I0 + I1y) * f;
  }
  int64_t base = idx * 3 * 7 * 32;
  int64_t o0 = base + (0 * 7 + k) * 32 + lane, o1 = base + (1 * 7 + k) * 32 + lane, o2 = base + (2 * 7 + k) * 32 + lane;
  st64[o0] = S0;
  st64[o1] = S1x;
  st64[o2] = S1y;
  st32[o0] = float(S0);
  st32[o1] = float(S1x);
  st32[o2] = float(S1y);
}

// The test-point sums of the closed-form parts, per near pair and slot:
// [sum w S0, sum w x S0, sum w y S0, sum w S1x, sum w S1y, sum w (x S1x +
// y S1y)] (w, x, y: the test triangle's 7-point weights and points about its
// centroid). They are frequency independent; the mixed fill multiplies them
// by the leading coefficients cA, cV of the frequency.
__global__ void stat_sums_kernel(int64_t nnear, const int2* __restrict__ near_list,
                                 const int32_t* __restrict__ block_tris, const TriData<double>* __restrict__ td,
                                 const double* __restrict__ st64, float2* __restrict__ st6) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= nnear * 32) return;
  const int64_t idx = gid >> 5;
  const int lane = (int)(gid & 31);
  const int t = block_tris[near_list[idx].x * 32 + lane];
  double v[6] = {0, 0, 0, 0, 0, 0};
  if (t >= 0) {
    const TriData<double>& A = td[t];
    const double* st = st64 + idx * 672;
    for (int k = 0; k < 7; ++k) {
      const double s0 = st[(0 * 7 + k) * 32 + lane], s1x = st[(1 * 7 + k) * 32 + lane], s1y = st[(2 * 7 + k) * 32 + lane];
      const double w = A.w7[k], wx = w * A.q7[k][0], wy = w * A.q7[k][1];
      v[0] += w * s0;
      v[1] += wx * s0;
      v[2] += wy * s0;
      v[3] += w * s1x;
      v[4] += w * s1y;
      v[5] += wx * s1x + wy * s1y;
    }
  }
  for (int q = 0; q < 6; ++q) {  // double-float: the fp32 rounding and its remainder
    const float h = (float)v[q];
    st6[(idx * 6 + q) * 32 + lane] = make_float2(h, (float)(v[q] - (double)h));
  }
}

__global__ void fill_i32(int32_t* p, int64_t n, int32_t v) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

__global__ void tpos_kernel(int nblocks, const int32_t* __restrict__ block_tris, const int32_t* __restrict__ tri_layer,
                            int32_t* __restrict__ tpos, int32_t* __restrict__ block_level) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nblocks * 32) return;
  int t = block_tris[i];
  if (t >= 0) tpos[t] = i;
  if ((i & 31) == 0) block_level[i >> 5] = tri_layer[t];
}

}  // namespace m25

using namespace m25;

template <class T>
static int upload(m25_geom* g, T** dst, const T* src, size_t n) {
  int rc = alloc(g->allocs, (void**)dst, n * sizeof(T));
  if (rc) return rc;
  if (n) M25_CUDA(cudaMemcpyAsync(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice, g->ctx->stream));
  return M25_OK;
}

extern "C" int m25_geometry_create(m25_ctx* ctx, const m25_mesh_desc* d, m25_geom** out) {
  if (!ctx || !d || !out) {
    set_error("m25_geometry_create: null argument");
    return M25_ERR_VALUE;
  }
  if (d->nt <= 0 || d->nb < 0 || d->nlev <= 0 || d->nblocks <= 0 || d->nv < 0 || d->npad < 0) {
    set_error("m25_geometry_create: bad sizes");
    return M25_ERR_VALUE;
  }
  // host-side validation of every index the kernels follow
  for (int64_t i = 0; i < (int64_t)d->nt * 3; ++i)
    if (d->tri_basis[i] < -1 || d->tri_basis[i] >= d->nb) {
      set_error("m25_geometry_create: tri_basis out of range");
      return M25_ERR_VALUE;
    }
  for (int i = 0; i < d->nt; ++i)
    if (d->tri_layer[i] < 0 || d->tri_layer[i] >= d->nlev) {
      set_error("m25_geometry_create: tri_layer out of range");
      return M25_ERR_VALUE;
    }
  for (int64_t i = 0; i < (int64_t)d->nb * 2; ++i)
    if (d->edge_tri[i] < 0 || d->edge_tri[i] >= d->nt || d->edge_loc[i] < 0 || d->edge_loc[i] > 2) {
      set_error("m25_geometry_create: edge_tri / edge_loc out of range (every basis needs two triangles)");
      return M25_ERR_VALUE;
    }
  {
    std::vector<int> seen(d->nt, 0);
    for (int b = 0; b < d->nblocks; ++b) {
      int t0 = d->block_tris[b * 32];
      if (t0 < 0) {
        set_error("m25_geometry_create: empty test block");
        return M25_ERR_VALUE;
      }
      for (int l = 0; l < 32; ++l) {
        int t = d->block_tris[b * 32 + l];
        if (t < -1 || t >= d->nt || (t >= 0 && d->tri_layer[t] != d->tri_layer[t0])) {
          set_error("m25_geometry_create: block_tris out of range or mixing levels");
          return M25_ERR_VALUE;
        }
        if (t >= 0) seen[t]++;
      }
    }
    for (int t = 0; t < d->nt; ++t)
      if (seen[t] != 1) {
        set_error("m25_geometry_create: every triangle must sit in exactly one block slot");
        return M25_ERR_VALUE;
      }
  }
  if (d->nv) {
    int npe = d->seg_pad_off[d->nv];
    for (int i = 0; i < npe; ++i)
      if (d->seg_pad[i] < 0 || d->seg_pad[i] >= d->npad) {
        set_error("m25_geometry_create: seg_pad out of range");
        return M25_ERR_VALUE;
      }
    for (int i = 0; i < d->npad; ++i)
      if (d->pad_tris[i] < 0 || d->pad_tris[i] >= d->nt) {
        set_error("m25_geometry_create: pad_tris out of range");
        return M25_ERR_VALUE;
      }
    for (int i = 0; i < 2 * d->nv; ++i)
      if (d->seg_end_lev[i] < -1 || d->seg_end_lev[i] >= d->nlev) {
        set_error("m25_geometry_create: seg_end_lev out of range");
        return M25_ERR_VALUE;
      }
  }
  M25_CUDA(cudaSetDevice(ctx->device));
  m25_geom* g = new m25_geom();
  g->ctx = ctx;
  g->nt = d->nt;
  g->nb = d->nb;
  g->nlev = d->nlev;
  g->nblocks = d->nblocks;
  g->nv = d->nv;
  g->npad = d->npad;
  g->near_factor = d->near_factor;
  g->far_factor = d->far_factor;
  int nt = d->nt;
  cudaStream_t st = ctx->stream;
  int rc = M25_OK;
  double* verts = nullptr;
  double* sign = nullptr;
  double* elen = nullptr;
  int64_t* block_off = nullptr;
  int32_t* counts = nullptr;
  int2* near_list = nullptr;
  std::vector<void*> tmp;
#define TRY(x)            \
  do {                    \
    rc = (x);             \
    if (rc) goto fail;    \
  } while (0)
  TRY(upload(g, &verts, d->verts, (size_t)nt * 6));
  TRY(upload(g, &g->tri_basis, d->tri_basis, (size_t)nt * 3));
  TRY(upload(g, &sign, d->tri_sign, (size_t)nt * 3));
  TRY(upload(g, &elen, d->edge_len, (size_t)std::max(d->nb, 1)));
  TRY(upload(g, &g->tri_layer, d->tri_layer, (size_t)nt));
  TRY(upload(g, &g->level_z, d->level_z, (size_t)d->nlev));
  TRY(upload(g, &g->edge_tri, d->edge_tri, (size_t)d->nb * 2));
  TRY(upload(g, &g->edge_loc, d->edge_loc, (size_t)d->nb * 2));
  TRY(upload(g, &g->block_tris, d->block_tris, (size_t)d->nblocks * 32));
  TRY(alloc(g->allocs, (void**)&g->cen, sizeof(double) * 2 * nt));
  TRY(alloc(g->allocs, (void**)&g->td64, sizeof(TriData<double>) * nt));
  TRY(alloc(g->allocs, (void**)&g->td32, sizeof(TriData<float>) * nt));
  TRY(alloc(g->allocs, (void**)&g->tddf, sizeof(TriDF) * nt));
  TRY(alloc(g->allocs, (void**)&g->cen_df, sizeof(float4) * nt));
  TRY(alloc(g->allocs, (void**)&g->tpos, sizeof(int32_t) * nt));
  TRY(alloc(g->allocs, (void**)&g->block_level, sizeof(int32_t) * d->nblocks));
  TRY(alloc(g->allocs, (void**)&g->cls, sizeof(int32_t) * (size_t)d->nblocks * nt));
  TRY(alloc(g->allocs, (void**)&g->pad_pos, sizeof(int32_t) * nt));
  tri_data_kernel<<<(nt + 127) / 128, 128, 0, st>>>(nt, verts, g->tri_basis, sign, elen, g->cen, g->td64, g->td32,
                                                   g->tddf, g->cen_df);
  tpos_kernel<<<(d->nblocks * 32 + 255) / 256, 256, 0, st>>>(d->nblocks, g->block_tris, g->tri_layer, g->tpos,
                                                             g->block_level);
  TRY(alloc(tmp, (void**)&counts, sizeof(int32_t) * d->nblocks));
  M25_CUDA(cudaMemsetAsync(counts, 0, sizeof(int32_t) * d->nblocks, st));
  {
    dim3 grid((nt + 255) / 256, d->nblocks);
    classify_kernel<<<grid, 256, 0, st>>>(nt, d->nblocks, g->block_tris, g->tri_layer, g->level_z, g->cen, g->td64,
                                          d->near_factor, d->far_factor, g->cls, counts);
    M25_CHECK_LAUNCH();
  }
  {
    std::vector<int32_t> hc(d->nblocks);
    std::vector<int64_t> off(d->nblocks + 1, 0);
    M25_CUDA(cudaMemcpyAsync(hc.data(), counts, sizeof(int32_t) * d->nblocks, cudaMemcpyDeviceToHost, st));
    M25_CUDA(cudaStreamSynchronize(st));
    for (int b = 0; b < d->nblocks; ++b) off[b + 1] = off[b] + hc[b];
    g->nnear = off[d->nblocks];
    TRY(alloc(tmp, (void**)&block_off, sizeof(int64_t) * (d->nblocks + 1)));
    M25_CUDA(cudaMemcpyAsync(block_off, off.data(), sizeof(int64_t) * (d->nblocks + 1), cudaMemcpyHostToDevice, st));
    TRY(alloc(tmp, (void**)&near_list, sizeof(int2) * std::max<int64_t>(g->nnear, 1)));
    near_index_kernel<<<d->nblocks, 256, 0, st>>>(nt, block_off, g->cls, near_list);
    M25_CHECK_LAUNCH();
    TRY(alloc(g->allocs, (void**)&g->stat64, sizeof(double) * std::max<int64_t>(g->nnear, 1) * 672));
    TRY(alloc(g->allocs, (void**)&g->stat32, sizeof(float) * std::max<int64_t>(g->nnear, 1) * 672));
    TRY(alloc(g->allocs, (void**)&g->stat6, sizeof(float2) * std::max<int64_t>(g->nnear, 1) * 192));
    if (g->nnear) {
      int64_t n = g->nnear * 224;
      static_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(g->nnear, near_list, g->block_tris, g->tri_layer,
                                                                  g->level_z, g->cen, g->td64, g->stat64, g->stat32);
      stat_sums_kernel<<<(unsigned)((g->nnear * 32 + 255) / 256), 256, 0, st>>>(g->nnear, near_list, g->block_tris,
                                                                                g->td64, g->stat64, g->stat6);
      M25_CHECK_LAUNCH();
    }
    // pair statistics (test triangles x source triangles)
    std::vector<int32_t> hcls((size_t)d->nblocks * nt);
    M25_CUDA(cudaMemcpyAsync(hcls.data(), g->cls, sizeof(int32_t) * hcls.size(), cudaMemcpyDeviceToHost, st));
    M25_CUDA(cudaStreamSynchronize(st));
    for (int b = 0; b < d->nblocks; ++b) {
      int nslot = 0;
      for (int l = 0; l < 32; ++l) nslot += d->block_tris[b * 32 + l] >= 0;
      for (int s = 0; s < nt; ++s) {
        int c = hcls[(size_t)b * nt + s];
        g->npairs[c >= 0 ? 0 : (c == -1 ? 1 : 2)] += nslot;
      }
    }
  }
  // vias
  {
    std::vector<int32_t> pp(nt, -1);
    for (int i = 0; i < d->npad; ++i) pp[d->pad_tris[i]] = i;
    M25_CUDA(cudaMemcpyAsync(g->pad_pos, pp.data(), sizeof(int32_t) * nt, cudaMemcpyHostToDevice, st));
    if (d->nv) {
      int npe = d->seg_pad_off[d->nv];
      TRY(upload(g, &g->pad_tris, d->pad_tris, (size_t)d->npad));
      TRY(upload(g, &g->seg_pad_off, d->seg_pad_off, (size_t)d->nv + 1));
      TRY(upload(g, &g->seg_pad, d->seg_pad, (size_t)npe));
      TRY(upload(g, &g->seg_pad_w, d->seg_pad_w, (size_t)npe));
      TRY(upload(g, &g->seg_end_lev, d->seg_end_lev, (size_t)d->nv * 2));
      TRY(upload(g, &g->seg_span, d->seg_span, (size_t)d->nv * 2));
      TRY(upload(g, &g->seg_xy, d->seg_xy, (size_t)d->nv * 2));
      TRY(upload(g, &g->seg_drill, d->seg_drill, (size_t)d->nv));
    }
  }
  M25_CUDA(cudaStreamSynchronize(st));
  M25_CHECK_LAUNCH();
  free_all(tmp);
  *out = g;
  return M25_OK;
fail:
  cudaStreamSynchronize(st);
  free_all(tmp);
  free_all(g->allocs);
  delete g;
  return rc;
#undef TRY
}

extern "C" int m25_geometry_destroy(m25_geom* g) {
  if (!g) return M25_OK;
  cudaStreamSynchronize(g->ctx->stream);
  free_all(g->allocs);
  delete g;
  return M25_OK;
}

extern "C" int m25_geometry_stats(m25_geom* g, int64_t* out) {
  if (!g || !out) {
    set_error("m25_geometry_stats: null argument");
    return M25_ERR_VALUE;
  }
  out[0] = g->npairs[0];
  out[1] = g->npairs[1];
  out[2] = g->npairs[2];
  out[3] = g->nnear * 672 * (int64_t)sizeof(double);
  return M25_OK;
}
