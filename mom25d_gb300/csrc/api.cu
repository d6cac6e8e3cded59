// C ABI glue: contexts, error text, workspace, and the drivers of the fill
// (m25_assemble) and of the dense solve (m25_dense_solve).
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "m25_internal.h"

namespace m25 {

static thread_local std::string g_err;
void set_error(const std::string& msg) { g_err = msg; }
const char* last_error() { return g_err.c_str(); }

int DevBuf::ensure(size_t n) {
  if (n <= bytes) return M25_OK;
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
  cudaError_t e = cudaMalloc(&p, n);
  if (e != cudaSuccess) {
    p = nullptr;
    set_error(std::string("workspace cudaMalloc(") + std::to_string(n) + " B): " + cudaGetErrorString(e));
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? M25_ERR_MEMORY : M25_ERR_CUDA;
  }
  bytes = n;
  return M25_OK;
}

void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

// fill.cu
template <class T>
int fill_driver(m25_ctx* ctx, m25_geom* geom, m25_greens* gr, zd zs, zd zsv, void* Z, int64_t ldz, int where,
                bool far32, const FillSplit* split = nullptr);

// lu.cu
template <class T> int lu_factor(m25_ctx*, cx<T>*, int64_t, int, int32_t*, int, bool, int*);
int refine(m25_ctx*, int, int, const zf*, const zf*, int64_t, const zf*, int64_t, const int32_t*, const zd*, zd*,
           double, int, int*);
void split_to_z32(m25_ctx*, const zd*, int64_t, zf*, int64_t, zf*, zf*, int64_t, int, int, double*, zd*, int);
bool lu_tc_available();
template <class TF, class TV>
int lu_solve_wave(m25_ctx*, const cx<TF>*, int64_t, int, const int32_t*, const cx<TV>*, int, cx<TV>*,
                  const int32_t* perm = nullptr);
int lu_wave_error(m25_ctx*, int, int*);
int lu_wave_reset(m25_ctx*);

// panel width of the complex64 LU: 64 columns keep the panel of up to ~7000
// trailing rows in the shared memory of one 16-CTA cluster
constexpr int kPanelZ64 = 64;

}  // namespace m25

using namespace m25;

extern "C" const char* m25_last_error(void) { return last_error(); }
extern "C" int m25_version(void) { return 1; }

extern "C" int m25_ctx_create(int device, m25_ctx** out) {
  if (!out) {
    set_error("m25_ctx_create: null out");
    return M25_ERR_VALUE;
  }
  int ndev = 0;
  M25_CUDA(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) {
    set_error("m25_ctx_create: no such CUDA device");
    return M25_ERR_VALUE;
  }
  M25_CUDA(cudaSetDevice(device));
  m25_ctx* c = new m25_ctx();
  c->device = device;
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    set_error(std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    return M25_ERR_CUDA;
  }
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  {
    // keep the memory of freed per-frequency tables in the stream-ordered
    // pool instead of handing it back to the driver at each synchronisation
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
      uint64_t keep = 1ull << 30;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
  }
  *out = c;
  return M25_OK;
}

extern "C" int m25_ctx_destroy(m25_ctx* c) {
  if (!c) return M25_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (DevBuf* b : {&c->H, &c->Zw, &c->Zlu, &c->Zsplit, &c->Bw, &c->Xw, &c->Rw, &c->Dw, &c->ipiv, &c->scratch, &c->deemb,
                    &c->Zsweep, &c->Xsweep, &c->flags, &c->sched})
    b->release();
  cudaStreamDestroy(c->stream);
  delete c;
  return M25_OK;
}

extern "C" int m25_ctx_synchronize(m25_ctx* c) {
  if (!c) {
    set_error("m25_ctx_synchronize: null context");
    return M25_ERR_VALUE;
  }
  M25_CUDA(cudaStreamSynchronize(c->stream));
  return M25_OK;
}

extern "C" void* m25_ctx_stream(m25_ctx* c) { return c ? (void*)c->stream : nullptr; }

extern "C" int m25_ctx_mem_info(m25_ctx* c, uint64_t* free_bytes, uint64_t* total_bytes) {
  if (!c) {
    set_error("m25_ctx_mem_info: null context");
    return M25_ERR_VALUE;
  }
  M25_CUDA(cudaSetDevice(c->device));
  size_t f = 0, t = 0;
  M25_CUDA(cudaMemGetInfo(&f, &t));
  if (free_bytes) *free_bytes = f;
  if (total_bytes) *total_bytes = t;
  return M25_OK;
}

extern "C" int m25_ctx_set_tuning(m25_ctx* c, int32_t panel_cluster_min, int32_t wave_ctas, int32_t tc_chunk,
                                  int32_t tc_tile_n) {
  if (!c || panel_cluster_min < 0 || wave_ctas < 0 || tc_chunk < 0 || tc_chunk > 8 ||
      (tc_tile_n != 0 && tc_tile_n != 128 && tc_tile_n != 192)) {
    set_error("m25_ctx_set_tuning: null context or a knob out of range (>= 0; tc_chunk <= 8; tc_tile_n 0, 128 or 192)");
    return M25_ERR_VALUE;
  }
  c->tune_cluster_min = panel_cluster_min;
  c->tune_wave_ctas = wave_ctas;
  c->tune_tc_chunk = tc_chunk;
  c->tune_tc_bn = tc_tile_n;
  return M25_OK;
}

extern "C" int m25_ctx_set_wait_limit(m25_ctx* c, int64_t polls) {
  if (!c || polls < 0) {
    set_error("m25_ctx_set_wait_limit: null context or negative limit");
    return M25_ERR_VALUE;
  }
  c->wave_spins = polls;
  return M25_OK;
}

namespace m25 {
cudaEvent_t take_event(m25_ctx* c) {
  if (!c->event_pool.empty()) {
    cudaEvent_t e = c->event_pool.back();
    c->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}
}  // namespace m25

extern "C" int m25_ctx_timing(m25_ctx* c, int enable, double* ms_out, long long* count_out) {
  if (!c) {
    set_error("m25_ctx_timing: null context");
    return M25_ERR_VALUE;
  }
  M25_CUDA(cudaStreamSynchronize(c->stream));
  for (auto& m : c->marks) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, m.a, m.b) == cudaSuccess) {
      c->stage_ms[m.stage] += ms;
      c->stage_n[m.stage] += 1;
    }
    c->event_pool.push_back(m.a);
    c->event_pool.push_back(m.b);
  }
  c->marks.clear();
  for (int s = 0; s < ST_COUNT; ++s) {
    if (ms_out) ms_out[s] = c->stage_ms[s];
    if (count_out) count_out[s] = c->stage_n[s];
  }
  if (enable >= 0) {
    // any change of the switch starts a new accumulation
    for (int s = 0; s < ST_COUNT; ++s) {
      c->stage_ms[s] = 0;
      c->stage_n[s] = 0;
    }
    c->timing = enable != 0;
  }
  return M25_OK;
}

extern "C" int m25_assemble(m25_ctx* ctx, m25_geom* geom, m25_greens* gr, double zs_re, double zs_im, double zsv_re,
                            double zsv_im, int precision, void* Z, int64_t ldz, int where) {
  if (!ctx || !geom || !gr || !Z) {
    set_error("m25_assemble: null argument");
    return M25_ERR_VALUE;
  }
  if (gr->nlev != geom->nlev) {
    set_error("m25_assemble: Green's tables and mesh have different level counts");
    return M25_ERR_VALUE;
  }
  const int n = geom->nb + geom->nv;
  if (ldz < n) {
    set_error("m25_assemble: ldz < n");
    return M25_ERR_VALUE;
  }
  M25_CUDA(cudaSetDevice(ctx->device));
  // M25_MIXED: complex128 Z with the far pairs evaluated in fp32 (near / mid in fp64)
  if (precision == M25_FP64 || precision == M25_MIXED)
    return fill_driver<double>(ctx, geom, gr, zd(zs_re, zs_im), zd(zsv_re, zsv_im), Z, ldz, where,
                               precision == M25_MIXED);
  if (precision == M25_MIXED_FILL32)
    return fill_driver<float>(ctx, geom, gr, zd(zs_re, zs_im), zd(zsv_re, zsv_im), Z, ldz, where, false);
  set_error("m25_assemble: unknown precision");
  return M25_ERR_VALUE;
}

extern "C" int m25_lu_factor(m25_ctx* ctx, int32_t n, int precision, void* A, int64_t lda, int32_t* ipiv, int where,
                             int32_t flags, int32_t* info) {
  if (!ctx || !A || !ipiv || n <= 0 || lda < n || (precision != M25_FP64 && precision != M25_MIXED)) {
    set_error("m25_lu_factor: bad argument");
    return M25_ERR_VALUE;
  }
  M25_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  const size_t esz = precision == M25_FP64 ? sizeof(zd) : sizeof(zf);
  void* Ad = A;
  int32_t* pd = ipiv;
  int rc;
  if (where == M25_ON_HOST) {
    if ((rc = ctx->Zw.ensure(esz * (size_t)n * lda))) return rc;
    if ((rc = ctx->ipiv.ensure(sizeof(int32_t) * n))) return rc;
    Ad = ctx->Zw.p;
    pd = ctx->ipiv.as<int32_t>();
    M25_CUDA(cudaMemcpyAsync(Ad, A, esz * (size_t)n * lda, cudaMemcpyHostToDevice, st));
  }
  int zinfo = 0;
  if (precision == M25_FP64)
    rc = lu_factor<double>(ctx, static_cast<zd*>(Ad), lda, n, pd, 64, false, &zinfo);
  else
    rc = lu_factor<float>(ctx, static_cast<zf*>(Ad), lda, n, pd, kPanelZ64,
                          lu_tc_available() && !(flags & M25_LU_NO_TENSOR_CORES), &zinfo);
  if (rc) return rc;
  if (where == M25_ON_HOST) {
    M25_CUDA(cudaMemcpyAsync(A, Ad, esz * (size_t)n * lda, cudaMemcpyDeviceToHost, st));
    M25_CUDA(cudaMemcpyAsync(ipiv, pd, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
  }
  M25_CUDA(cudaStreamSynchronize(st));
  if (info) *info = zinfo;
  return M25_OK;
}

// presplit: Z is already the mixed path's double-float planes and LU input
static int dense_solve_impl(m25_ctx* ctx, int32_t n, int32_t nrhs, int precision, void* Z, const void* B, void* X,
                            int where, double tol, int32_t max_iter, int32_t* info, const FillSplit* presplit);

extern "C" int m25_dense_solve(m25_ctx* ctx, int32_t n, int32_t nrhs, int precision, void* Z, const void* B, void* X,
                               int where, double tol, int32_t max_iter, int32_t* info) {
  return dense_solve_impl(ctx, n, nrhs, precision, Z, B, X, where, tol, max_iter, info, nullptr);
}

namespace m25 {
// The mixed fill of a mesh without vias straight into the double-float
// planes of Z and the complex64 LU input (no complex128 Z, no split pass),
// then the mixed solve: the path of m25_sweep_point for M25_MIXED.
int fill_solve_mixed(m25_ctx* ctx, m25_geom* geom, m25_greens* gr, zd zs, zd zsv, int nrhs, const zd* B, zd* X,
                     double tol, int max_iter, int32_t* info) {
  const int n = geom->nb;
  const int64_t ldl = (n + 1) & ~1;
  const size_t nn = (size_t)n * n;
  int rc;
  if ((rc = ctx->Zsplit.ensure(sizeof(zf) * 2 * nn))) return rc;
  if ((rc = ctx->Zlu.ensure(sizeof(zf) * (size_t)n * ldl))) return rc;
  zf* h = ctx->Zsplit.as<zf>();
  const FillSplit sp{h, h + nn, ctx->Zlu.as<zf>(), ldl};
  if ((rc = fill_driver<double>(ctx, geom, gr, zs, zsv, nullptr, n, M25_ON_DEVICE, true, &sp))) return rc;
  return dense_solve_impl(ctx, n, nrhs, M25_MIXED, nullptr, B, X, M25_ON_DEVICE, tol, max_iter, info, &sp);
}
}  // namespace m25

static int dense_solve_impl(m25_ctx* ctx, int32_t n, int32_t nrhs, int precision, void* Z, const void* B, void* X,
                            int where, double tol, int32_t max_iter, int32_t* info, const FillSplit* presplit) {
  if (!ctx || !(Z || presplit) || !B || !X || n <= 0 || nrhs <= 0 || nrhs > 8) {
    set_error("m25_dense_solve: bad argument (1 <= nrhs <= 8)");
    return M25_ERR_VALUE;
  }
  M25_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->stream;
  const size_t nn = (size_t)n * n, nr = (size_t)n * nrhs;
  int rc;
  if ((rc = lu_wave_reset(ctx))) return rc;
  if ((rc = ctx->ipiv.ensure(sizeof(int32_t) * n))) return rc;
  if ((rc = ctx->Bw.ensure(sizeof(zd) * nr))) return rc;
  if ((rc = ctx->Xw.ensure(sizeof(zd) * nr))) return rc;
  zd* Bd = ctx->Bw.as<zd>();
  zd* Xd = ctx->Xw.as<zd>();
  M25_CUDA(cudaMemcpyAsync(Bd, B, sizeof(zd) * nr, where == M25_ON_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st));
  int zinfo = 0, steps = 0;
  if (precision == M25_FP64) {
    zd* Zd = static_cast<zd*>(Z);
    if (where == M25_ON_HOST) {
      if ((rc = ctx->Zw.ensure(sizeof(zd) * nn))) return rc;
      Zd = ctx->Zw.as<zd>();
      M25_CUDA(cudaMemcpyAsync(Zd, Z, sizeof(zd) * nn, cudaMemcpyHostToDevice, st));
    }
    if ((rc = lu_factor<double>(ctx, Zd, n, n, ctx->ipiv.as<int32_t>(), 64, false, &zinfo))) return rc;
    if (zinfo) {
      if (info) { info[0] = 0; info[1] = zinfo; }
      set_error("m25_dense_solve: exactly singular matrix (zero pivot)");
      return M25_ERR_NUMERIC;
    }
    if ((rc = lu_solve_wave<double, double>(ctx, Zd, n, n, ctx->ipiv.as<int32_t>(), Bd, nrhs, Xd))) return rc;
  } else if (precision == M25_MIXED || precision == M25_MIXED_FILL32) {
    // M25_MIXED: Z complex128 (cast for the LU); M25_MIXED_FILL32: Z is the complex64 fill
    // the LU's rows padded to an even length (16-byte rows for the tensor-core update's TMA)
    const int64_t ldl = presplit ? presplit->ldl : (n + 1) & ~1;
    if (!presplit && (rc = ctx->Zlu.ensure(sizeof(zf) * (size_t)n * ldl))) return rc;
    zf* LU = presplit ? presplit->LU : ctx->Zlu.as<zf>();
    const void* Zres = Z;
    if (where == M25_ON_HOST && !presplit) {
      size_t zb = (precision == M25_MIXED_FILL32 ? sizeof(zf) : sizeof(zd)) * nn;
      if ((rc = ctx->Zw.ensure(zb))) return rc;
      M25_CUDA(cudaMemcpyAsync(ctx->Zw.p, Z, zb, cudaMemcpyHostToDevice, st));
      Zres = ctx->Zw.p;
    }
    // Z for the residuals as complex64 planes Zh + Zl (fp64-level products on
    // the fp32 pipes); Zh is also the LU's input
    const zf* Zh = static_cast<const zf*>(Zres);
    const zf* Zl = nullptr;
    if (presplit) {
      Zh = presplit->Zh;
      Zl = presplit->Zl;
    } else if (precision == M25_MIXED_FILL32) {
      M25_CUDA(cudaMemcpy2DAsync(LU, sizeof(zf) * ldl, Zres, sizeof(zf) * n, sizeof(zf) * n, n,
                                 cudaMemcpyDeviceToDevice, st));
    } else {
      if ((rc = ctx->Zsplit.ensure(sizeof(zf) * 2 * nn))) return rc;
      zf* h = ctx->Zsplit.as<zf>();
      // rows equilibrated by powers of two (B with them; X unchanged)
      if ((rc = ctx->sched.ensure(256 + sizeof(double) * (size_t)n))) return rc;
      double* rs = reinterpret_cast<double*>(ctx->sched.as<char>() + 256);
      split_to_z32(ctx, static_cast<const zd*>(Zres), n, LU, ldl, h, h + nn, n, n, n, rs, Bd, nrhs);
      Zh = h;
      Zl = h + nn;
    }
    if ((rc = lu_factor<float>(ctx, LU, ldl, n, ctx->ipiv.as<int32_t>(), kPanelZ64, lu_tc_available(), &zinfo)))
      return rc;
    if (zinfo) {
      if (info) { info[0] = 0; info[1] = zinfo; }
      set_error("m25_dense_solve: zero pivot in the complex64 LU");
      return M25_ERR_NUMERIC;
    }
    rc = refine(ctx, n, nrhs, Zh, Zl, n, LU, ldl, ctx->ipiv.as<int32_t>(), Bd, Xd, tol, max_iter, &steps);
    if (rc) {
      // a triangular solve that gave up leaves garbage that the refinement
      // then reports as a numeric failure: name the wait instead
      int werr = 0;
      if (lu_wave_error(ctx, n, &werr) == M25_OK && werr) {
        set_error("dense solve: a wait of the triangular solve ran out");
        return M25_ERR_CUDA;
      }
      return rc;
    }
  } else {
    set_error("m25_dense_solve: unknown precision");
    return M25_ERR_VALUE;
  }
  M25_CUDA(cudaMemcpyAsync(X, Xd, sizeof(zd) * nr, where == M25_ON_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, st));
  int berr = 0;
  if ((rc = lu_wave_error(ctx, n, &berr))) return rc;
  if (berr) {
    set_error("dense solve: a wait of the triangular solve ran out");
    return M25_ERR_CUDA;
  }
  if (info) {
    info[0] = steps;
    info[1] = 0;
  }
  return M25_OK;
}
