// Frequency interpolation of the impedance matrix between anchor fills, the
// device form of mom25d's FreqInterp (Engine/mom25d/freqinterp.py:27-197).
//
// With the propagation phase between basis functions taken out and the
// 1/(j w) of the scalar potential undone, W = j w Z exp(+j k_e R_mn) is
// smooth in frequency; anchors are filled exactly, W is kept per anchor, and
// at another frequency the Lagrange combination of the order + 1 nearest
// anchors gives Z = W~ exp(-j k_e R) / (j w). Both kernels are elementwise
// over the n x n matrix (HBM-bound: the anchors are read once per point);
// R comes from the basis centres, 0 between two via unknowns (their block
// carries the Im gV(0) correction, the same for every pair:
// freqinterp.py:93-101). The anchor window and the weights are host logic
// (mom25d_gb300/freqinterp.py).
#include "m25_internal.h"

namespace m25 {

namespace {

constexpr int kMaxUse = 8;

struct EvalSrc {
  const void* W[kMaxUse];
  double L[kMaxUse];
};

__device__ __forceinline__ double basis_dist(const double* __restrict__ pos, int nb, int i, int j) {
  if (i >= nb && j >= nb) return 0.0;  // via-via: no phase extraction
  const double dx = pos[3 * i] - pos[3 * j], dy = pos[3 * i + 1] - pos[3 * j + 1], dz = pos[3 * i + 2] - pos[3 * j + 2];
  return sqrt(dx * dx + dy * dy + dz * dz);
}

// W = (j w) Z exp(+j ke R), in the order of the reference's product; one CTA
// per row (blockIdx.x), its threads along the row
template <class TW>
__global__ void interp_store_kernel(int n, int nb, const double* __restrict__ pos, const zd* __restrict__ Z,
                                    int64_t ldz, double w, double ke, cx<TW>* __restrict__ W) {
  const int i = blockIdx.x;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const zd z = Z[(int64_t)i * ldz + j];
    double s, c;
    sincos(ke * basis_dist(pos, nb, i, j), &s, &c);
    const zd jwz(-w * z.im, w * z.re);
    const zd v = jwz * zd(c, s);
    W[(int64_t)i * n + j] = cx<TW>((TW)v.re, (TW)v.im);
  }
}

// Z = (sum_a L_a W_a) exp(-j ke R) / (j w); one CTA per row
template <class TW>
__global__ void interp_eval_kernel(int n, int nb, const double* __restrict__ pos, int nuse, EvalSrc src, double w,
                                   double ke, zd* __restrict__ Z, int64_t ldz) {
  const int i = blockIdx.x;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const int64_t e = (int64_t)i * n + j;
    zd acc(0.0, 0.0);
    for (int a = 0; a < nuse; ++a) {
      const cx<TW> v = static_cast<const cx<TW>*>(src.W[a])[e];
      acc += zd(src.L[a] * (double)v.re, src.L[a] * (double)v.im);
    }
    double s, c;
    sincos(ke * basis_dist(pos, nb, i, j), &s, &c);
    const zd t = acc * zd(c, -s);
    Z[(int64_t)i * ldz + j] = zd(t.im / w, -t.re / w);  // t / (j w)
  }
}


}  // namespace

int interp_eval_device(m25_ctx* ctx, m25_interp* ip, int nuse, const int32_t* slots, const double* L, double freq,
                       double ke, zd* Z, int64_t ldz) {
  if (nuse < 1 || nuse > kMaxUse || !slots || !L) {
    set_error("m25_interp_eval: between 1 and 8 anchors");
    return M25_ERR_VALUE;
  }
  EvalSrc src{};
  for (int a = 0; a < nuse; ++a) {
    if (slots[a] < 0 || slots[a] >= (int)ip->slots.size()) {
      set_error("m25_interp_eval: slot out of range");
      return M25_ERR_VALUE;
    }
    src.W[a] = ip->slots[slots[a]];
    src.L[a] = L[a];
  }
  const double w = 2.0 * kPi * freq;
  if (ip->single)
    interp_eval_kernel<float><<<ip->n, 256, 0, ctx->stream>>>(ip->n, ip->nb, ip->pos, nuse, src, w, ke, Z, ldz);
  else
    interp_eval_kernel<double><<<ip->n, 256, 0, ctx->stream>>>(ip->n, ip->nb, ip->pos, nuse, src, w, ke, Z, ldz);
  M25_CHECK_LAUNCH();
  return M25_OK;
}

}  // namespace m25

using namespace m25;

extern "C" int m25_interp_create(m25_ctx* ctx, int32_t n, int32_t nb, const double* pos, int32_t nslots,
                                 int32_t single, m25_interp** out) {
  if (!ctx || !pos || !out || n <= 0 || nb < 0 || nb > n || nslots <= 0) {
    set_error("m25_interp_create: bad argument");
    return M25_ERR_VALUE;
  }
  M25_CUDA(cudaSetDevice(ctx->device));
  auto* ip = new m25_interp;
  ip->ctx = ctx;
  ip->n = n;
  ip->nb = nb;
  ip->single = single ? 1 : 0;
  const size_t wbytes = (single ? sizeof(zf) : sizeof(zd)) * (size_t)n * n;
  int rc = alloc(ip->allocs, (void**)&ip->pos, sizeof(double) * 3 * (size_t)n);
  for (int s = 0; rc == M25_OK && s < nslots; ++s) {
    void* p = nullptr;
    rc = alloc(ip->allocs, &p, wbytes);
    ip->slots.push_back(p);
  }
  if (rc == M25_OK && cudaMemcpyAsync(ip->pos, pos, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice,
                                      ctx->stream) != cudaSuccess) {
    set_error("m25_interp_create: copy of the basis centres failed");
    rc = M25_ERR_CUDA;
  }
  if (rc) {
    cudaStreamSynchronize(ctx->stream);
    free_all(ip->allocs);
    delete ip;
    return rc;
  }
  *out = ip;
  return M25_OK;
}

extern "C" int m25_interp_destroy(m25_interp* ip) {
  if (!ip) return M25_OK;
  cudaSetDevice(ip->ctx->device);
  cudaStreamSynchronize(ip->ctx->stream);
  free_all(ip->allocs);
  delete ip;
  return M25_OK;
}

extern "C" int m25_interp_store(m25_interp* ip, int32_t slot, const void* Z, int64_t ldz, int where, double freq,
                                double ke) {
  if (!ip || !Z || slot < 0 || slot >= (int)ip->slots.size() || ldz < ip->n || freq <= 0) {
    set_error("m25_interp_store: bad argument");
    return M25_ERR_VALUE;
  }
  m25_ctx* ctx = ip->ctx;
  M25_CUDA(cudaSetDevice(ctx->device));
  const zd* Zd = static_cast<const zd*>(Z);
  if (where == M25_ON_HOST) {
    int rc = ctx->Zw.ensure(sizeof(zd) * (size_t)ip->n * ip->n);
    if (rc) return rc;
    M25_CUDA(cudaMemcpy2DAsync(ctx->Zw.p, sizeof(zd) * ip->n, Z, sizeof(zd) * ldz, sizeof(zd) * ip->n, ip->n,
                               cudaMemcpyHostToDevice, ctx->stream));
    Zd = ctx->Zw.as<zd>();
    ldz = ip->n;
  }
  const double w = 2.0 * kPi * freq;
  if (ip->single)
    interp_store_kernel<float><<<ip->n, 256, 0, ctx->stream>>>(ip->n, ip->nb, ip->pos, Zd, ldz, w, ke,
                                                                 static_cast<zf*>(ip->slots[slot]));
  else
    interp_store_kernel<double><<<ip->n, 256, 0, ctx->stream>>>(ip->n, ip->nb, ip->pos, Zd, ldz, w, ke,
                                                                  static_cast<zd*>(ip->slots[slot]));
  M25_CHECK_LAUNCH();
  if (where == M25_ON_HOST) M25_CUDA(cudaStreamSynchronize(ctx->stream));
  return M25_OK;
}

extern "C" int m25_interp_eval(m25_interp* ip, int32_t nuse, const int32_t* slots, const double* L, double freq,
                               double ke, void* Z, int64_t ldz, int where) {
  if (!ip || !Z || ldz < ip->n || freq <= 0) {
    set_error("m25_interp_eval: bad argument");
    return M25_ERR_VALUE;
  }
  m25_ctx* ctx = ip->ctx;
  M25_CUDA(cudaSetDevice(ctx->device));
  zd* Zd = static_cast<zd*>(Z);
  int64_t ld = ldz;
  if (where == M25_ON_HOST) {
    int rc = ctx->Zw.ensure(sizeof(zd) * (size_t)ip->n * ip->n);
    if (rc) return rc;
    Zd = ctx->Zw.as<zd>();
    ld = ip->n;
  }
  int rc = interp_eval_device(ctx, ip, nuse, slots, L, freq, ke, Zd, ld);
  if (rc) return rc;
  if (where == M25_ON_HOST) {
    M25_CUDA(cudaMemcpy2DAsync(Z, sizeof(zd) * ldz, Zd, sizeof(zd) * ip->n, sizeof(zd) * ip->n, ip->n,
                               cudaMemcpyDeviceToHost, ctx->stream));
    M25_CUDA(cudaStreamSynchronize(ctx->stream));
  }
  return M25_OK;
}

extern "C" int m25_interp_anchor(m25_ctx* ctx, m25_geom* geom, m25_greens* gr, m25_interp* ip, int32_t slot,
                                 double zs_re, double zs_im, double zsv_re, double zsv_im, int precision, double ke) {
  if (!ctx || !geom || !gr || !ip || ip->ctx != ctx || ip->n != geom->nb + geom->nv) {
    set_error("m25_interp_anchor: bad argument (the anchors are filled on the context that made them)");
    return M25_ERR_VALUE;
  }
  if (precision != M25_FP64 && precision != M25_MIXED) {
    set_error("m25_interp_anchor: precision must be M25_FP64 or M25_MIXED");
    return M25_ERR_VALUE;
  }
  const int n = ip->n;
  int rc = ctx->Zsweep.ensure(sizeof(zd) * (size_t)n * n);
  if (rc) return rc;
  if ((rc = m25_assemble(ctx, geom, gr, zs_re, zs_im, zsv_re, zsv_im, precision, ctx->Zsweep.p, n, M25_ON_DEVICE)))
    return rc;
  return m25_interp_store(ip, slot, ctx->Zsweep.p, n, M25_ON_DEVICE, gr->freq, ke);
}
