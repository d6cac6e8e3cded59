// Internal state behind the C ABI (not installed; see include/m25.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "../../include/m25.h"
#include "m25_common.cuh"

namespace m25 {

constexpr int kMaxLev = 3;                 // metal levels per stack
constexpr int kMaxLevSq = kMaxLev * kMaxLev;

// Per-triangle data of the fill, all lengths relative to the triangle's own
// centroid (cx, cy) so that fp32 arithmetic keeps its precision.
// The triangle data the mixed fill's near pairs take in double-float (each
// value as an fp32 rounding h and its remainder l, h + l within 2^-48).
struct TriDF {
  float vh[3][2], vl[3][2];  // vertices about the centroid
  float cAh[3], cAl[3];      // RWG amplitudes
  float cVh[3], cVl[3];      // divergences
  float gzh[3][3], gzl[3][3];  // the self pair's conductor-loss factor Int_T (r - a_i).(r - a_j) dS cA_i cA_j
};

template <class T>
struct TriData {
  T v[3][2];   // vertices
  T q7[7][2];  // 7-point rule
  T w7[7];     // weights * area
  T q3[3][2];  // 3-point rule
  T w3[3];
  T cA[3];     // RWG amplitude sign * l / (2A)
  T cV[3];     // divergence sign * l / A
  T area;
  T size;      // longest edge
};

// A device buffer that grows on demand.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  int ensure(size_t n);
  void release();
  template <class T> T* as() const { return static_cast<T*>(p); }
};

}  // namespace m25

namespace m25 {
// Stages timed with CUDA events on the context's stream (m25_ctx_timing).
enum Stage { ST_GREENS, ST_FILL, ST_GATHER, ST_VIA, ST_PANEL, ST_PACK, ST_TRSM, ST_GEMM, ST_TRSV, ST_REFINE,
             ST_DEEMBED, ST_COUNT };
}

struct m25_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  bool timing = false;
  struct Mark { int stage; cudaEvent_t a, b; };
  std::vector<Mark> marks;
  std::vector<cudaEvent_t> event_pool;
  double stage_ms[m25::ST_COUNT] = {};
  long long stage_n[m25::ST_COUNT] = {};
  // workspace reused across calls
  m25::DevBuf H, Zw, Zlu, Zsplit, Bw, Xw, Rw, Dw, ipiv, scratch, deemb, Zsweep, Xsweep, flags;
  m25::DevBuf sched;  // work counters of the dynamically scheduled kernels
  bool flags_fresh = true;  // the ready flags of the triangular solves need zeroing
  int epoch = 0;            // value of a ready flag in the current sweep
  size_t yt_off = 0;        // offset of the tagged vector copy in the flag buffer (0: not placed yet)
  long long wave_spins = 0; // polls per ready-flag wait of the triangular solves (0: the default bound)
  // tuning knobs (m25_ctx_set_tuning; 0: the process default)
  int tune_cluster_min = 0; // smallest cluster of the LU panel (4, 8 or 16)
  int tune_wave_ctas = 0;   // CTA cap of the triangular solves
  int tune_tc_chunk = 0;    // steps of 32 tf32 per TMEM accumulation of the tensor-core update
  int tune_tc_bn = 0;       // tile N of the tensor-core update (128 or 192; 0: by the update's width)
  // caller-provided scratch instead of the workspace buffers (LU panel
  // candidates + barrier words; triangular-solve flags, already zeroed)
  char* ext_scratch = nullptr;
  int ext_gmax = 0;
  int* ext_flags = nullptr;
  std::vector<char> host_tmp;
};

struct m25_geom {
  m25_ctx* ctx = nullptr;
  int nt = 0, nb = 0, nlev = 0, nblocks = 0, nv = 0, npad = 0;
  double near_factor = 3.0, far_factor = 10.0;
  // device arrays
  double* cen = nullptr;                 // (nt,2) absolute centroids
  float4* cen_df = nullptr;              // (nt) the same in double-float (x h, x l, y h, y l), mixed fill
  m25::TriData<double>* td64 = nullptr;  // (nt)
  m25::TriData<float>* td32 = nullptr;   // (nt)
  m25::TriDF* tddf = nullptr;            // (nt) double-float copy for the mixed near pairs
  int32_t* tri_layer = nullptr;          // (nt)
  int32_t* tri_basis = nullptr;          // (nt,3)
  double* level_z = nullptr;             // (nlev)
  int32_t* block_tris = nullptr;         // (nblocks,32)
  int32_t* block_level = nullptr;        // (nblocks)
  int32_t* tpos = nullptr;               // (nt) block slot of each triangle (blk*32+lane)
  int32_t* edge_tri = nullptr;           // (nb,2)
  int32_t* edge_loc = nullptr;           // (nb,2)
  int32_t* cls = nullptr;                // (nblocks, nt) >= 0 near index, -1 mid, -2 far
  double* stat64 = nullptr;              // (nnear, 3, 7, 32) closed-form S0, S1x, S1y
  float* stat32 = nullptr;
  float2* stat6 = nullptr;               // (nnear, 6, 32) their test-point sums (mixed fill), double-float
  int64_t nnear = 0, npairs[3] = {0, 0, 0};
  // vias
  int32_t* pad_pos = nullptr;            // (nt) pad index or -1
  int32_t* pad_tris = nullptr;           // (npad)
  int32_t* seg_pad_off = nullptr;
  int32_t* seg_pad = nullptr;
  double* seg_pad_w = nullptr;
  int32_t* seg_end_lev = nullptr;        // (nv,2)
  double* seg_span = nullptr;            // (nv,2)
  double* seg_xy = nullptr;              // (nv,2)
  double* seg_drill = nullptr;           // (nv)
  std::vector<void*> allocs;
};

struct m25_greens {
  m25_ctx* ctx = nullptr;
  int nlev = 0, nrho = 0, single = 0;
  double freq = 0, omega = 0, stack_h = 0;
  double* rho = nullptr;       // (nrho)
  std::vector<double> rho_h;   // host copy
  double* S = nullptr;         // (3, nlev, nlev, nrho) complex: S_A, S_V, S_W
  double* coef = nullptr;      // (nlev*nlev, nrho-1, 4, 3) complex cubic coefficients
  float* coef32 = nullptr;     // fp32 copy
  float* rho32 = nullptr;
  double* lead = nullptr;      // (3, nlev, nlev) complex c_A, c_V, c_W (device)
  m25::zd* res = nullptr;      // (nrho, 3 nlev^2) Sommerfeld remainder (or the learned one)
  void* sur = nullptr;         // learned remainder: int accepted, then double relative error (device)
  double sur_info[3] = {0, 0, 0};  // host copy: accepted, judged error, radii integrated
  int sur_planned = 0;              // radii integrated when the learned remainder is accepted
  std::vector<m25::zd> lead_h; // host copy
  std::vector<double> dz_h;    // (nlev, nlev)
  std::vector<void*> allocs;
};

struct m25_interp {
  m25_ctx* ctx = nullptr;
  int n = 0, nb = 0, single = 0;
  double* pos = nullptr;          // (n, 3) basis centres
  std::vector<void*> slots;       // anchor matrices W, n x n complex128 or complex64
  std::vector<void*> allocs;
};

namespace m25 {
// Z (device, complex128, rows ldz apart) <- the interpolation of the anchors,
// on the stream of ctx (any context of the anchors' device)
int interp_eval_device(m25_ctx* ctx, m25_interp* ip, int nuse, const int32_t* slots, const double* L, double freq,
                       double ke, zd* Z, int64_t ldz);
// output of the mixed fill as double-float planes and the complex64 LU input
struct FillSplit {
  zf *Zh, *Zl, *LU;
  int64_t ldl;
};
// the compressed operator's near field and via rows (fill.cu)
int fill_listed(m25_ctx* ctx, m25_geom* geom, m25_greens* gr, zd zs, zd zsv, const int32_t* cidx, zd* Hc,
                const int32_t* perm, zd* ZxbT, zd* Zxx);
int alloc(std::vector<void*>& list, void** p, size_t bytes);
void free_all(std::vector<void*>& list);
// Stream-ordered variants for the per-frequency objects: unlike cudaFree,
// cudaFreeAsync does not wait for the work of every other stream.
int alloc_async(std::vector<void*>& list, void** p, size_t bytes, cudaStream_t st);
void free_all_async(std::vector<void*>& list, cudaStream_t st);

cudaEvent_t take_event(m25_ctx* c);

// Records CUDA events around the kernels of one stage when timing is on.
struct StageTimer {
  m25_ctx* c;
  int stage;
  cudaEvent_t a = nullptr;
  StageTimer(m25_ctx* ctx, int s) : c(ctx), stage(s) {
    if (c->timing) {
      a = take_event(c);
      cudaEventRecord(a, c->stream);
    }
  }
  ~StageTimer() {
    if (c->timing && a) {
      cudaEvent_t b = take_event(c);
      cudaEventRecord(b, c->stream);
      c->marks.push_back({stage, a, b});
    }
  }
};
}  // namespace m25
