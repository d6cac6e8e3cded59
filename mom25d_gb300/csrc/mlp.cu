// A small fp32 MLP with hand-written forward, backward and Adam kernels: the
// learned surrogate of the layered Green's remainder (m25_greens_desc
// .surrogate). tanh hidden layers of width kMlpH, a linear output layer.
//
// Parameters live in one float array, layer by layer: W_l (out x in,
// row-major) then b_l. Training minimises the mean over samples and outputs
// of (f(x) - y)^2. Every kernel is deterministic: one thread per sample for
// the training's forward and backward passes, one warp per sample for
// inference, and the weight gradients are reduced over the samples in a fixed
// order (no atomics).
#include <algorithm>
#include <cmath>
#include <vector>

#include "m25_internal.h"

namespace m25 {

constexpr int kMlpH = 64;
constexpr int kMlpMaxIn = 4;
constexpr int kMlpMaxOut = 64;
constexpr int kMlpMaxLayers = 4;  // hidden layers
constexpr int kMlpThreads = 128;

struct MlpDims {
  int n_in, n_layers, n_out;
  int64_t off[kMlpMaxLayers + 1];  // start of W_l; b_l follows it
};

__host__ __device__ inline int mlp_in(const MlpDims& d, int l) { return l == 0 ? d.n_in : kMlpH; }
__host__ __device__ inline int mlp_out(const MlpDims& d, int l) { return l == d.n_layers ? d.n_out : kMlpH; }

// Y = f(X); with STORE the hidden activations go to acts[(l * kMlpH + j) * n + s]
template <bool STORE>
__global__ void __launch_bounds__(kMlpThreads) mlp_fwd_kernel(MlpDims d, const float* __restrict__ P, int64_t np, int n,
                                                             const float* __restrict__ X, float* __restrict__ Y,
                                                             float* __restrict__ acts) {
  extern __shared__ float sp[];
  for (int64_t i = threadIdx.x; i < np; i += blockDim.x) sp[i] = P[i];
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float h[kMlpH];
  {
    const float* W = sp + d.off[0];
    const float* b = W + kMlpH * d.n_in;
    float x[kMlpMaxIn];
#pragma unroll
    for (int i = 0; i < kMlpMaxIn; ++i) x[i] = i < d.n_in ? X[(int64_t)s * d.n_in + i] : 0.f;
#pragma unroll
    for (int j = 0; j < kMlpH; ++j) {
      float a = b[j];
#pragma unroll
      for (int i = 0; i < kMlpMaxIn; ++i)
        if (i < d.n_in) a = fmaf(W[j * d.n_in + i], x[i], a);
      h[j] = tanhf(a);
      if (STORE) acts[(int64_t)j * n + s] = h[j];
    }
  }
  for (int l = 1; l < d.n_layers; ++l) {
    const float* W = sp + d.off[l];
    const float* b = W + kMlpH * kMlpH;
    float g[kMlpH];
#pragma unroll
    for (int j = 0; j < kMlpH; ++j) {
      float a = b[j];
#pragma unroll
      for (int i = 0; i < kMlpH; ++i) a = fmaf(W[j * kMlpH + i], h[i], a);
      g[j] = tanhf(a);
    }
#pragma unroll
    for (int j = 0; j < kMlpH; ++j) {
      h[j] = g[j];
      if (STORE) acts[((int64_t)l * kMlpH + j) * n + s] = h[j];
    }
  }
  if (Y == nullptr) return;  // training: the backward pass recomputes the outputs
  const float* W = sp + d.off[d.n_layers];
  const float* b = W + (int64_t)d.n_out * kMlpH;
  for (int j = 0; j < d.n_out; ++j) {
    float a = b[j];
#pragma unroll
    for (int i = 0; i < kMlpH; ++i) a = fmaf(W[j * kMlpH + i], h[i], a);
    Y[(int64_t)s * d.n_out + j] = a;
  }
}

// Y = f(X) for inference, one warp per sample: lane j forms hidden units j
// and j + 32 of every layer and outputs j, j + 32 (the same fused
// multiply-adds in the same order as mlp_fwd_kernel, so Y is bit for bit the
// same), the layer's activations passed through the warp's row of shared
// memory. The weights are stored transposed in shared memory so that the 32
// lanes read consecutive words. Shared memory: np + kInferWarps x kMlpH floats.
constexpr int kInferWarps = 8;
__global__ void __launch_bounds__(32 * kInferWarps) mlp_infer_kernel(MlpDims d, const float* __restrict__ P,
                                                                     int64_t np, int n, const float* __restrict__ X,
                                                                     float* __restrict__ Y) {
  extern __shared__ float sp[];
  for (int l = 0; l <= d.n_layers; ++l) {
    const int nin = mlp_in(d, l), nout = mlp_out(d, l);
    const float* W = P + d.off[l];
    float* Wt = sp + d.off[l];
    for (int e = threadIdx.x; e < nin * nout; e += blockDim.x) Wt[(e % nin) * nout + e / nin] = W[e];
    for (int e = threadIdx.x; e < nout; e += blockDim.x) Wt[nin * nout + e] = W[nin * nout + e];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* hs = sp + np + warp * kMlpH;
  for (int s = blockIdx.x * kInferWarps + warp; s < n; s += gridDim.x * kInferWarps) {
    {
      const float* Wt = sp + d.off[0];
      const float* b = Wt + kMlpH * d.n_in;
      float x[kMlpMaxIn];
#pragma unroll
      for (int i = 0; i < kMlpMaxIn; ++i) x[i] = i < d.n_in ? X[(int64_t)s * d.n_in + i] : 0.f;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int j = lane + 32 * h;
        float a = b[j];
#pragma unroll
        for (int i = 0; i < kMlpMaxIn; ++i)
          if (i < d.n_in) a = fmaf(Wt[i * kMlpH + j], x[i], a);
        hs[j] = tanhf(a);
      }
    }
    __syncwarp();
    for (int l = 1; l < d.n_layers; ++l) {
      const float* Wt = sp + d.off[l];
      const float* b = Wt + kMlpH * kMlpH;
      float a0 = b[lane], a1 = b[lane + 32];
#pragma unroll 16
      for (int i = 0; i < kMlpH; ++i) {
        const float hi = hs[i];
        a0 = fmaf(Wt[i * kMlpH + lane], hi, a0);
        a1 = fmaf(Wt[i * kMlpH + lane + 32], hi, a1);
      }
      __syncwarp();
      hs[lane] = tanhf(a0);
      hs[lane + 32] = tanhf(a1);
      __syncwarp();
    }
    const float* Wt = sp + d.off[d.n_layers];
    const float* b = Wt + (int64_t)d.n_out * kMlpH;
    for (int j = lane; j < d.n_out; j += 32) {
      float a = b[j];
#pragma unroll 16
      for (int i = 0; i < kMlpH; ++i) a = fmaf(Wt[i * d.n_out + j], hs[i], a);
      Y[(int64_t)s * d.n_out + j] = a;
    }
    __syncwarp();
  }
}

// Output error and the deltas of every layer (dL/d pre-activation) from the
// stored activations: deltas[(l * kMlpH + j) * n + s]. gscale = 2 / (samples
// x outputs) of the loss; sqerr[s] = sum_j (f_j - y_j)^2 when not null.
__global__ void __launch_bounds__(kMlpThreads) mlp_bwd_kernel(MlpDims d, const float* __restrict__ P, int64_t np, int n,
                                                             const float* __restrict__ T, const float* __restrict__ acts,
                                                             float* __restrict__ deltas, float* __restrict__ sqerr,
                                                             float gscale) {
  extern __shared__ float sp[];
  float* drow = sp + ((np + 31) & ~(int64_t)31);  // per thread: the delta of the layer above (stride 65)
  for (int64_t i = threadIdx.x; i < np; i += blockDim.x) sp[i] = P[i];
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float* dr = drow + threadIdx.x * (kMlpH + 1);
  const int L = d.n_layers;
  float a[kMlpH];
#pragma unroll
  for (int i = 0; i < kMlpH; ++i) a[i] = acts[((int64_t)(L - 1) * kMlpH + i) * n + s];
  float e2 = 0.f;
  {
    const float* W = sp + d.off[L];
    const float* b = W + (int64_t)d.n_out * kMlpH;
    for (int j = 0; j < d.n_out; ++j) {
      float y = b[j];
#pragma unroll
      for (int i = 0; i < kMlpH; ++i) y = fmaf(W[j * kMlpH + i], a[i], y);
      const float e = y - T[(int64_t)s * d.n_out + j];
      e2 = fmaf(e, e, e2);
      dr[j] = gscale * e;
      deltas[((int64_t)L * kMlpH + j) * n + s] = dr[j];
    }
  }
  if (sqerr) sqerr[s] = e2;
  for (int l = L - 1; l >= 0; --l) {
    // delta_l = (W_{l+1}^T delta_{l+1}) * (1 - a_l^2)
    const float* W = sp + d.off[l + 1];
    const int rows = mlp_out(d, l + 1);
    float dn[kMlpH];
#pragma unroll
    for (int i = 0; i < kMlpH; ++i) dn[i] = 0.f;
    for (int j = 0; j < rows; ++j) {
      const float dj = dr[j];
#pragma unroll
      for (int i = 0; i < kMlpH; ++i) dn[i] = fmaf(W[j * kMlpH + i], dj, dn[i]);
    }
#pragma unroll
    for (int i = 0; i < kMlpH; ++i) {
      dn[i] *= 1.f - a[i] * a[i];
      dr[i] = dn[i];
      deltas[((int64_t)l * kMlpH + i) * n + s] = dn[i];
    }
    if (l > 0) {
#pragma unroll
      for (int i = 0; i < kMlpH; ++i) a[i] = acts[((int64_t)(l - 1) * kMlpH + i) * n + s];
    }
  }
}

// dW_l[j][i] = sum_s delta_l[j][s] in_l[i][s], db_l[j] = sum_s delta_l[j][s]:
// one CTA per (layer, row j), a fixed split of the samples over the threads
// and a fixed reduction tree.
__global__ void __launch_bounds__(256) mlp_wgrad_kernel(MlpDims d, int n, const float* __restrict__ X,
                                                        const float* __restrict__ acts,
                                                        const float* __restrict__ deltas, float* __restrict__ G) {
  const int l = blockIdx.y, j = blockIdx.x;
  if (j >= mlp_out(d, l)) return;
  const int nin = mlp_in(d, l);
  float acc[kMlpH + 1];
#pragma unroll
  for (int i = 0; i <= kMlpH; ++i) acc[i] = 0.f;
  const float* dl = deltas + ((int64_t)l * kMlpH + j) * n;
  for (int s = threadIdx.x; s < n; s += blockDim.x) {
    const float dj = dl[s];
    if (l == 0) {
#pragma unroll
      for (int i = 0; i < kMlpMaxIn; ++i)
        if (i < nin) acc[i] = fmaf(dj, X[(int64_t)s * nin + i], acc[i]);
    } else {
      const float* in = acts + (int64_t)(l - 1) * kMlpH * n + s;
#pragma unroll
      for (int i = 0; i < kMlpH; ++i) acc[i] = fmaf(dj, in[(int64_t)i * n], acc[i]);
    }
    acc[kMlpH] += dj;
  }
  __shared__ float red[8][kMlpH + 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i <= kMlpH; ++i) {
    float v = acc[i];
    for (int o = 16; o; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][i] = v;
  }
  __syncthreads();
  for (int i = threadIdx.x; i <= nin; i += blockDim.x) {
    const int ii = i == nin ? kMlpH : i;
    float v = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w][ii];
    if (i < nin) G[d.off[l] + (int64_t)j * nin + i] = v;
    else G[d.off[l] + (int64_t)mlp_out(d, l) * nin + j] = v;
  }
}

__global__ void mlp_adam_kernel(int64_t np, float* __restrict__ P, const float* __restrict__ G, float* __restrict__ M1,
                                float* __restrict__ M2, float lr, float c1, float c2) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= np) return;
  const float g = G[i];
  const float m = 0.9f * M1[i] + 0.1f * g, v = 0.999f * M2[i] + 0.001f * g * g;
  M1[i] = m;
  M2[i] = v;
  P[i] -= lr * (m * c1) / (sqrtf(v * c2) + 1e-8f);
}

// minibatch rows drawn from a counter-based hash of (seed, step, row)
__device__ inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void mlp_gather_kernel(int n_all, int batch, int n_in, int n_out, uint64_t seed, int step,
                                  const float* __restrict__ X, const float* __restrict__ Y, float* __restrict__ Xb,
                                  float* __restrict__ Yb) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= batch) return;
  const int src = (int)(mix64(seed ^ mix64(((uint64_t)step << 32) | (uint32_t)r)) % (uint64_t)n_all);
  for (int i = 0; i < n_in; ++i) Xb[(int64_t)r * n_in + i] = X[(int64_t)src * n_in + i];
  for (int j = 0; j < n_out; ++j) Yb[(int64_t)r * n_out + j] = Y[(int64_t)src * n_out + j];
}

}  // namespace m25

using namespace m25;

struct m25_mlp {
  m25_ctx* ctx = nullptr;
  MlpDims d{};
  int64_t np = 0;
  int64_t adam_t = 0;
  std::vector<void*> allocs;
  float *P = nullptr, *M1 = nullptr, *M2 = nullptr, *G = nullptr;
  DevBuf data, work;
};

namespace m25 {

static size_t mlp_fwd_smem(const m25_mlp* m) { return sizeof(float) * (size_t)m->np; }
static size_t mlp_bwd_smem(const m25_mlp* m) {
  return sizeof(float) * ((((size_t)m->np + 31) & ~(size_t)31) + (size_t)kMlpThreads * (kMlpH + 1));
}

// forward pass of n samples already on the device (X (n, n_in), Y (n, n_out))
int mlp_forward_device(const m25_mlp* m, int n, const float* X, float* Y, cudaStream_t st) {
  if (n <= 0) return M25_OK;
  const int64_t blocks = std::min<int64_t>((n + kInferWarps - 1) / kInferWarps, 4096);
  mlp_infer_kernel<<<(unsigned)blocks, 32 * kInferWarps, sizeof(float) * ((size_t)m->np + kInferWarps * kMlpH), st>>>(
      m->d, m->P, m->np, n, X, Y);
  M25_CHECK_LAUNCH();
  return M25_OK;
}

int mlp_dims(const m25_mlp* m, int* n_in, int* n_out) {
  *n_in = m->d.n_in;
  *n_out = m->d.n_out;
  return M25_OK;
}

// loss gradient of n device samples into m->G; per-sample squared errors into sqerr (or null)
static int mlp_grad_device(m25_mlp* m, int n, const float* X, const float* Y, float* acts, float* deltas,
                           float* sqerr, cudaStream_t st) {
  const unsigned g = (unsigned)((n + kMlpThreads - 1) / kMlpThreads);
  mlp_fwd_kernel<true><<<g, kMlpThreads, mlp_fwd_smem(m), st>>>(m->d, m->P, m->np, n, X, nullptr, acts);
  mlp_bwd_kernel<<<g, kMlpThreads, mlp_bwd_smem(m), st>>>(m->d, m->P, m->np, n, Y, acts, deltas, sqerr,
                                                         2.0f / ((float)n * (float)m->d.n_out));
  mlp_wgrad_kernel<<<dim3(kMlpH, m->d.n_layers + 1), 256, 0, st>>>(m->d, n, X, acts, deltas, m->G);
  M25_CHECK_LAUNCH();
  return M25_OK;
}

}  // namespace m25

extern "C" int m25_mlp_create(m25_ctx* ctx, int32_t n_in, int32_t hidden, int32_t n_layers, int32_t n_out,
                              uint64_t seed, m25_mlp** out) {
  if (!ctx || !out || n_in < 1 || n_in > kMlpMaxIn || hidden != kMlpH || n_layers < 1 || n_layers > kMlpMaxLayers ||
      n_out < 1 || n_out > kMlpMaxOut) {
    set_error("m25_mlp_create: 1 <= n_in <= 4, hidden = 64, 1 <= n_layers <= 4, 1 <= n_out <= 64");
    return M25_ERR_VALUE;
  }
  M25_CUDA(cudaSetDevice(ctx->device));
  m25_mlp* m = new m25_mlp();
  m->ctx = ctx;
  m->d.n_in = n_in;
  m->d.n_layers = n_layers;
  m->d.n_out = n_out;
  int64_t off = 0;
  for (int l = 0; l <= n_layers; ++l) {
    m->d.off[l] = off;
    off += (int64_t)mlp_out(m->d, l) * mlp_in(m->d, l) + mlp_out(m->d, l);
  }
  m->np = off;
  // Glorot-uniform weights from a splitmix64 stream, zero biases
  std::vector<float> h(off, 0.f);
  uint64_t z = seed;
  auto next = [&z]() {
    z += 0x9E3779B97F4A7C15ull;
    uint64_t x = z;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    x ^= x >> 31;
    return (double)(x >> 11) * (1.0 / 9007199254740992.0);
  };
  for (int l = 0; l <= n_layers; ++l) {
    const int fi = mlp_in(m->d, l), fo = mlp_out(m->d, l);
    const double lim = std::sqrt(6.0 / (fi + fo));
    for (int64_t k = 0; k < (int64_t)fi * fo; ++k) h[m->d.off[l] + k] = (float)((2.0 * next() - 1.0) * lim);
  }
  int rc = M25_OK;
  for (float** p : {&m->P, &m->M1, &m->M2, &m->G})
    if ((rc = alloc(m->allocs, (void**)p, sizeof(float) * off))) {
      free_all(m->allocs);
      delete m;
      return rc;
    }
  cudaStream_t st = ctx->stream;
  M25_CUDA(cudaMemcpyAsync(m->P, h.data(), sizeof(float) * off, cudaMemcpyHostToDevice, st));
  M25_CUDA(cudaMemsetAsync(m->M1, 0, sizeof(float) * off, st));
  M25_CUDA(cudaMemsetAsync(m->M2, 0, sizeof(float) * off, st));
  M25_CUDA(cudaFuncSetAttribute(mlp_fwd_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024));
  M25_CUDA(cudaFuncSetAttribute(mlp_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024));
  M25_CUDA(cudaFuncSetAttribute(mlp_fwd_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024));
  M25_CUDA(cudaFuncSetAttribute(mlp_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024));
  if (mlp_bwd_smem(m) > 160 * 1024) {
    set_error("m25_mlp_create: network too large for shared memory");
    free_all(m->allocs);
    delete m;
    return M25_ERR_VALUE;
  }
  M25_CUDA(cudaStreamSynchronize(st));
  *out = m;
  return M25_OK;
}

extern "C" int m25_mlp_destroy(m25_mlp* m) {
  if (!m) return M25_OK;
  cudaStreamSynchronize(m->ctx->stream);
  m->data.release();
  m->work.release();
  free_all(m->allocs);
  delete m;
  return M25_OK;
}

extern "C" int m25_mlp_params(m25_mlp* m, int64_t* count, float* get, const float* set) {
  if (!m) {
    set_error("m25_mlp_params: null network");
    return M25_ERR_VALUE;
  }
  if (count) *count = m->np;
  cudaStream_t st = m->ctx->stream;
  if (set) {
    M25_CUDA(cudaMemcpyAsync(m->P, set, sizeof(float) * m->np, cudaMemcpyHostToDevice, st));
    M25_CUDA(cudaMemsetAsync(m->M1, 0, sizeof(float) * m->np, st));
    M25_CUDA(cudaMemsetAsync(m->M2, 0, sizeof(float) * m->np, st));
    m->adam_t = 0;
  }
  if (get) M25_CUDA(cudaMemcpyAsync(get, m->P, sizeof(float) * m->np, cudaMemcpyDeviceToHost, st));
  M25_CUDA(cudaStreamSynchronize(st));
  return M25_OK;
}

// device layout of a data set: X (n, n_in) | Y (n, n_out), then the work
// area for `rows` samples: acts (L, 64, rows) | deltas (L + 1, 64, rows) | sqerr (rows)
static int mlp_upload(m25_mlp* m, int n, const float* X, const float* Y, int rows, float** Xd, float** Yd,
                      float** acts, float** deltas, float** sqerr) {
  const size_t nx = (size_t)n * m->d.n_in, ny = (size_t)n * m->d.n_out;
  int rc;
  if ((rc = m->data.ensure(sizeof(float) * (nx + ny)))) return rc;
  const size_t L = m->d.n_layers;
  if ((rc = m->work.ensure(sizeof(float) * ((size_t)rows * (m->d.n_in + m->d.n_out) + L * kMlpH * rows +
                                             (L + 1) * kMlpH * rows + rows))))
    return rc;
  cudaStream_t st = m->ctx->stream;
  *Xd = m->data.as<float>();
  *Yd = *Xd + nx;
  M25_CUDA(cudaMemcpyAsync(*Xd, X, sizeof(float) * nx, cudaMemcpyHostToDevice, st));
  if (Y) M25_CUDA(cudaMemcpyAsync(*Yd, Y, sizeof(float) * ny, cudaMemcpyHostToDevice, st));
  float* w = m->work.as<float>() + (size_t)rows * (m->d.n_in + m->d.n_out);
  *acts = w;
  *deltas = w + L * kMlpH * rows;
  *sqerr = *deltas + (L + 1) * kMlpH * rows;
  return M25_OK;
}

extern "C" int m25_mlp_loss_grad(m25_mlp* m, int32_t n, const float* X, const float* Y, double* loss, float* grad) {
  if (!m || n < 1 || !X || !Y) {
    set_error("m25_mlp_loss_grad: bad argument");
    return M25_ERR_VALUE;
  }
  float *Xd, *Yd, *acts, *deltas, *sqerr;
  int rc = mlp_upload(m, n, X, Y, n, &Xd, &Yd, &acts, &deltas, &sqerr);
  if (rc) return rc;
  cudaStream_t st = m->ctx->stream;
  if ((rc = mlp_grad_device(m, n, Xd, Yd, acts, deltas, sqerr, st))) return rc;
  std::vector<float> e(n);
  M25_CUDA(cudaMemcpyAsync(e.data(), sqerr, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
  if (grad) M25_CUDA(cudaMemcpyAsync(grad, m->G, sizeof(float) * m->np, cudaMemcpyDeviceToHost, st));
  M25_CUDA(cudaStreamSynchronize(st));
  if (loss) {
    double s = 0;
    for (float v : e) s += v;
    *loss = s / ((double)n * m->d.n_out);
  }
  return M25_OK;
}

extern "C" int m25_mlp_train(m25_mlp* m, int32_t n, const float* X, const float* Y, int32_t steps, int32_t batch,
                             double lr, double lr_min, uint64_t seed, double* loss_out) {
  if (!m || n < 1 || !X || !Y || steps < 0 || batch < 1) {
    set_error("m25_mlp_train: bad argument");
    return M25_ERR_VALUE;
  }
  float *Xd, *Yd, *acts, *deltas, *sqerr;
  const int rows = std::max(batch, n);
  int rc = mlp_upload(m, n, X, Y, rows, &Xd, &Yd, &acts, &deltas, &sqerr);
  if (rc) return rc;
  cudaStream_t st = m->ctx->stream;
  float* Xb = m->work.as<float>();
  float* Yb = Xb + (size_t)batch * m->d.n_in;
  const unsigned ga = (unsigned)((m->np + 255) / 256);
  for (int it = 0; it < steps; ++it) {
    mlp_gather_kernel<<<(batch + 255) / 256, 256, 0, st>>>(n, batch, m->d.n_in, m->d.n_out, seed, it, Xd, Yd, Xb, Yb);
    if ((rc = mlp_grad_device(m, batch, Xb, Yb, acts, deltas, nullptr, st))) return rc;
    // cosine decay from lr to lr_min
    const double a = lr_min + 0.5 * (lr - lr_min) * (1.0 + std::cos(kPi * it / std::max(1, steps)));
    ++m->adam_t;
    const float c1 = (float)(1.0 / (1.0 - std::pow(0.9, (double)m->adam_t)));
    const float c2 = (float)(1.0 / (1.0 - std::pow(0.999, (double)m->adam_t)));
    mlp_adam_kernel<<<ga, 256, 0, st>>>(m->np, m->P, m->G, m->M1, m->M2, (float)a, c1, c2);
  }
  M25_CHECK_LAUNCH();
  if (loss_out) {
    // full-data loss after training, in fixed-size chunks
    double s = 0;
    std::vector<float> e;
    for (int c0 = 0; c0 < n; c0 += rows) {
      const int cn = std::min(rows, n - c0);
      if ((rc = mlp_grad_device(m, cn, Xd + (size_t)c0 * m->d.n_in, Yd + (size_t)c0 * m->d.n_out, acts, deltas, sqerr,
                                st)))
        return rc;
      e.resize(cn);
      M25_CUDA(cudaMemcpyAsync(e.data(), sqerr, sizeof(float) * cn, cudaMemcpyDeviceToHost, st));
      M25_CUDA(cudaStreamSynchronize(st));
      for (float v : e) s += v;
    }
    *loss_out = s / ((double)n * m->d.n_out);
  }
  M25_CUDA(cudaStreamSynchronize(st));
  return M25_OK;
}

extern "C" int m25_mlp_forward(m25_mlp* m, int32_t n, const float* X, float* Y) {
  if (!m || n < 1 || !X || !Y) {
    set_error("m25_mlp_forward: bad argument");
    return M25_ERR_VALUE;
  }
  float *Xd, *Yd, *acts, *deltas, *sqerr;
  int rc = mlp_upload(m, n, X, nullptr, 1, &Xd, &Yd, &acts, &deltas, &sqerr);
  if (rc) return rc;
  cudaStream_t st = m->ctx->stream;
  if ((rc = mlp_forward_device(m, n, Xd, Yd, st))) return rc;
  M25_CUDA(cudaMemcpyAsync(Y, Yd, sizeof(float) * (size_t)n * m->d.n_out, cudaMemcpyDeviceToHost, st));
  M25_CUDA(cudaStreamSynchronize(st));
  return M25_OK;
}
