// Tensor-core (tcgen05) trailing update of the complex64 LU:
//
//   A22 -= L21 U12          (complex, interleaved re/im, row-major, lda)
//
// of rank 128 per block of two panels, and of rank 64 on the second panel's
// columns (the factorisation's order is in lu.cu).
//
// written as one real GEMM on the interleaved storage: C (m x 2n') -=
// A (m x 2K) B (2K x 2n') with A the interleaved conj(L21) and B rows
// (U, -iU) alternating, which gives Re and Im of L U in the even and odd
// columns of C. Each fp32 operand is split into tf32 hi + lo parts, stored
// as two planes [hi | lo] of width P (P = 2K rounded up to 64) along K, and
// every k-block issues the three products hi.lo, lo.hi, hi.hi (3xTF32) from
// the same staged tiles: the operands are read once, not once per product.
//
// The tensor cores round their fp32 accumulation with a bias, so a long
// accumulation chain loses about four bits against fp32 fused multiply-adds.
// The K loop is therefore cut into chunks of a few k-blocks: each chunk is
// accumulated afresh in one of two TMEM buffers and the epilogue warps add the
// chunk results into fp32 registers with round-to-nearest (the accumulation
// outside the tensor cores of Ootomo & Yokota, 2022), which keeps the update
// at the accuracy of the SIMT one.
//
// Kernel (persistent, one CTA per SM, 320 threads): warp 0 issues TMA loads of
// 128B-swizzled K-major tiles (A hi, A lo 128 x 32, B hi, B lo 192 x 32 fp32)
// into a 2-stage mbarrier ring of 80 KB stages; warp 1 owns the TMEM (two
// 128 x 192 fp32 buffers) and one elected thread issues tcgen05.mma (M 128,
// N 192, K 8; 12 per k-block); warps 2-9 read the
// chunk results with tcgen05.ld and sum them, and at the end of a tile hand
// the negated sums to the TMA as 32 x 32 blocks (128B-swizzled staging, two
// buffers per warp) that are reduce-added into C in global memory
// (cp.reduce.async.bulk.tensor .add), so C is never read by the SMs and the
// update overlaps the next tile's MMAs. C's rows must be a multiple of 16
// bytes (an even leading dimension) and C 16-byte aligned. Every mbarrier
// wait is bounded in iterations and wall-clock time; on a timeout the CTA
// raises an error word, stops all roles, waits (bounded) for its TMA copies
// and MMAs, frees its TMEM and returns.
#include <cuda.h>

#include <algorithm>
#include <mutex>
#include <string>

#include "m25_internal.h"

namespace m25 {

namespace {

// k-blocks of 32 tf32 (128-byte rows, 128-byte swizzle) in a 2-stage ring (k-blocks
// of 16 in 4 stages of 40 KB, 64-byte swizzle, measured no faster: 47 % against 50 %
// tensor pipe on the largest n = 4096 launch)
constexpr int kBM = 128, kBK = 32, kStages = 2;
// N of a tile (real columns of C): 192 by default, 128 for narrow updates (and where
// the context's tuning asks for it); the kernel is instantiated for both
constexpr int kBNDefault = 192;
constexpr int kChunkK = 32;  // tf32 elements per TMEM accumulation per unit of the chunk setting
constexpr int kTmemCols = 512, kBufStride = 256;  // two accumulators, 256 columns apart
constexpr int kTileA = kBM * kBK * 4;
template <int BN>
constexpr int tile_b() { return BN * kBK * 4; }
// [A hi | A lo | B hi | B lo], each 1024-byte aligned
template <int BN>
constexpr int stage_bytes() { return 2 * (kTileA + tile_b<BN>()); }
constexpr int kEpiWarps = 8, kThreads = 64 + 32 * kEpiWarps;
constexpr int kOutBlock = 32 * 32 * 4;  // one 32 x 32 fp32 block of C, staged for the TMA reduce
template <int BN>
constexpr int smem_bytes() { return kStages * stage_bytes<BN>() + kEpiWarps * 2 * kOutBlock + 1024; }
constexpr long long kWaitLimit = 1LL << 24;
constexpr unsigned long long kWaitNs = 200ull * 1000 * 1000;  // 200 ms wall clock per wait

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}
// Bounded wait for the phase with the given parity: false on a timeout (an
// iteration limit and a wall-clock limit) or, when abort is given, as soon as
// another role of the CTA has raised it.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, const volatile int* abort = nullptr) {
  uint32_t addr = smem_u32(bar);
  unsigned long long t0;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t0));
  for (long long it = 0; it < kWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
    if (abort && *abort) return false;
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    if (t - t0 > kWaitNs) return false;
  }
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int c0, int c1, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];\n" ::
          "r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(smem_u32(bar))
      : "memory");
}

// C += tile (fp32 add) for the box at (c0, c1) of the tensor map, from shared memory
__device__ __forceinline__ void tma_reduce_add_2d(const CUtensorMap* map, const void* src, int c0, int c1) {
  asm volatile(
      "cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group [%0, {%1, %2}], [%3];\n" ::"l"(map),
      "r"(c0), "r"(c1), "r"(smem_u32(src))
      : "memory");
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;            // leading-dimension offset (unused with this swizzle)
  d |= (uint64_t)(1024 >> 4) << 32;  // stride between 8-row groups (8 rows of 128 bytes)
  d |= (uint64_t)1 << 46;            // descriptor version
  d |= (uint64_t)2 << 61;            // 128-byte swizzle
  return d;
}

// instruction descriptor: D f32, A and B tf32, both K-major, N = BN, M = 128
template <int BN>
constexpr uint32_t idesc() {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(kBM >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc_v,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc_v), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_u32(bar))
               : "memory");
}

struct TcArgs {
  int M, N, P;     // rows, real columns of C (its fp32 view), packed K extent per plane (multiple of 32)
  int pw;          // plane width: the lo plane starts pw floats after the hi plane (pw >= P)
  int tiles_m, ntiles;
  int chunk;       // k-blocks (of kBK) accumulated afresh in TMEM before the register sum
  int* err;
  int* counter;    // tiles handed out beyond the first gridDim.x (zero at launch)
};

constexpr int kTileRing = 4;  // tile indices in flight from the producer to the MMA and epilogue warps
constexpr int kTcHeader = 4096;

// one CTA per SM; 10 warps put three on one SM sub-partition, which caps a
// thread at 168 registers (BN / 2 <= 96 running sums per epilogue thread fit)
template <int BN>
__global__ void __launch_bounds__(kThreads, 1)
    tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   const __grid_constant__ CUtensorMap tmC, TcArgs a) {
  static_assert(BN == 128 || BN == 192, "tiles of 128 or 192 real columns");
  constexpr int kTileB = tile_b<BN>(), kStageBytes = stage_bytes<BN>();
  constexpr uint32_t kIdesc = idesc<BN>();
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte alignment of the swizzled tiles
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  float* stage_out = reinterpret_cast<float*>(base + kStages * kStageBytes);  // 2 blocks per epilogue warp
  __shared__ __align__(8) uint64_t full[kStages], empty[kStages], tfull[2], tempty[2], done;
  __shared__ __align__(8) uint64_t tile_full[kTileRing], tile_empty[kTileRing];
  __shared__ int tile_id[kTileRing];
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag, n_issued, n_consumed, skip;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = a.P / kBK;  // k-blocks of one plane
  const int nch = (nk + a.chunk - 1) / a.chunk;
  // an earlier CTA gave up: leave before taking TMEM
  if (threadIdx.x == 0) skip = *(volatile int*)a.err;
  __syncthreads();
  if (skip) return;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&tfull[b], 1);
      mbar_init(&tempty[b], kEpiWarps);
    }
    for (int r = 0; r < kTileRing; ++r) {
      mbar_init(&tile_full[r], 1);
      mbar_init(&tile_empty[r], 1 + kEpiWarps);
    }
    mbar_init(&done, 1);
    abort_flag = 0;
    n_issued = 0;
    n_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    asm volatile("prefetch.tensormap [%0];\n" ::"l"(&tmA) : "memory");
    asm volatile("prefetch.tensormap [%0];\n" ::"l"(&tmB) : "memory");
    asm volatile("prefetch.tensormap [%0];\n" ::"l"(&tmC) : "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_base;
  volatile int* abort_v = &abort_flag;

  if (warp == 0) {
    // TMA producer
    // tiles are handed out by a counter (CTAs that start late, behind the
    // kernels of concurrent sweeps, take fewer) and passed on through a ring
    // of tile indices; -1 ends the CTA's sequence
    if (lane == 0) {
      int it = 0;
      for (int lt = 0; !*abort_v; ++lt) {
        const int r = lt % kTileRing;
        int t = lt == 0 ? (int)blockIdx.x : (int)gridDim.x + atomicAdd(a.counter, 1);
        if (t >= a.ntiles) t = -1;
        if (lt >= kTileRing && !mbar_wait(&tile_empty[r], ((lt / kTileRing) - 1) & 1, abort_v)) {
          *abort_v = 1;
          break;
        }
        tile_id[r] = t;
        mbar_arrive(&tile_full[r]);
        if (t < 0) break;
        const int m0 = (t % a.tiles_m) * kBM, n0 = (t / a.tiles_m) * BN;
        for (int kb = 0; kb < nk; ++kb, ++it) {
          const int s = it % kStages;
          if (it >= kStages && !mbar_wait(&empty[s], ((it / kStages) - 1) & 1, abort_v)) {
            *abort_v = 1;
            break;
          }
          unsigned char* sa = base + s * kStageBytes;
          mbar_expect_tx(&full[s], kStageBytes);
          tma_load_2d(sa + kTileA, &tmA, a.pw + kb * kBK, m0, &full[s]);
          tma_load_2d(sa + 2 * kTileA + kTileB, &tmB, a.pw + kb * kBK, n0, &full[s]);
          tma_load_2d(sa, &tmA, kb * kBK, m0, &full[s]);
          tma_load_2d(sa + 2 * kTileA, &tmB, kb * kBK, n0, &full[s]);
          n_issued = it + 1;
        }
      }
    }
  } else if (warp == 1) {
    // MMA issuer
    if (lane == 0) {
      int it = 0, ch = 0;
      bool ok = true;
      for (int lt = 0; ok; ++lt) {
        const int r = lt % kTileRing;
        if (!mbar_wait(&tile_full[r], (lt / kTileRing) & 1, abort_v)) {
          ok = false;
          break;
        }
        const int t = *(volatile int*)&tile_id[r];
        mbar_arrive(&tile_empty[r]);
        if (t < 0) break;
        for (int c = 0; c < nch && ok; ++c, ++ch) {
          const int b = ch & 1;
          if (ch >= 2 && !mbar_wait(&tempty[b], ((ch >> 1) - 1) & 1, abort_v)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
          const uint32_t acc = tmem + (uint32_t)(b * kBufStride);
          const int kb1 = min(nk, (c + 1) * a.chunk);
          for (int kb = c * a.chunk; kb < kb1; ++kb, ++it) {
            const int s = it % kStages;
            if (!mbar_wait(&full[s], (it / kStages) & 1, abort_v)) {
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t sah = smem_u32(base + s * kStageBytes), sal = sah + kTileA;
            const uint32_t sbh = sah + 2 * kTileA, sbl = sbh + kTileB;
            // the two small products first, then hi.hi; 8 tf32 = 32 bytes per MMA
#pragma unroll
            for (int k = 0; k < kBK / 8; ++k)
              mma_tf32(acc, smem_desc(sah + 32 * k), smem_desc(sbl + 32 * k), kIdesc,
                       (kb > c * a.chunk || k) ? 1u : 0u);
#pragma unroll
            for (int k = 0; k < kBK / 8; ++k)
              mma_tf32(acc, smem_desc(sal + 32 * k), smem_desc(sbh + 32 * k), kIdesc, 1u);
#pragma unroll
            for (int k = 0; k < kBK / 8; ++k)
              mma_tf32(acc, smem_desc(sah + 32 * k), smem_desc(sbh + 32 * k), kIdesc, 1u);
            mma_commit(&empty[s]);  // frees the stage once these MMAs have read it
            n_consumed = it + 1;
          }
          if (ok) mma_commit(&tfull[b]);
        }
      }
      if (!ok) *abort_v = 1;
      mma_commit(&done);  // arrives once every MMA issued above has completed
    }
  } else {
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (rows of C), columns
    // h * 96 .. + 95, and reduce-adds minus their sum into C by TMA, one
    // 32 x 32 block at a time through two staging buffers
    const int q = warp & 3, h = (warp - 2) >> 2;
    float* stg = stage_out + (warp - 2) * 2 * (kOutBlock / 4);
    int ch = 0, nout = 0;
    bool ok = true;
    for (int lt = 0; ok; ++lt) {
      const int r = lt % kTileRing;
      ok = __all_sync(0xffffffffu, mbar_wait(&tile_full[r], (lt / kTileRing) & 1, abort_v));
      if (!ok) break;
      const int t = *(volatile int*)&tile_id[r];
      __syncwarp();
      if (lane == 0) mbar_arrive(&tile_empty[r]);
      if (t < 0) break;
      const int m0 = (t % a.tiles_m) * kBM, n0 = (t / a.tiles_m) * BN;
      float sum[BN / 2];
#pragma unroll
      for (int j = 0; j < BN / 2; ++j) sum[j] = 0.f;
      for (int c = 0; c < nch; ++c, ++ch) {
        const int b = ch & 1;
        ok = __all_sync(0xffffffffu, mbar_wait(&tfull[b], (ch >> 1) & 1, abort_v));
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        // batches of 16-column loads (three for BN = 192: two batches; two for
        // BN = 128: two batches), each batch waited for once (in the same asm
        // statement, so no use of r can move above the wait)
        constexpr int kPer = (BN / 2) % 48 == 0 ? 3 : 2;
#pragma unroll
        for (int gb = 0; gb < (BN / 2) / (16 * kPer); ++gb) {
          uint32_t r[16 * kPer];
          const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) +
                                 (uint32_t)(b * kBufStride + h * (BN / 2) + gb * 16 * kPer);
          if constexpr (kPer == 3) {
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%48];\n"
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%49];\n"
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47}, [%50];\n"
                "tcgen05.wait::ld.sync.aligned;\n"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47])
                : "r"(taddr), "r"(taddr + 16u), "r"(taddr + 32u)
                : "memory");
          } else {
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%32];\n"
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%33];\n"
                "tcgen05.wait::ld.sync.aligned;\n"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                : "r"(taddr), "r"(taddr + 16u)
                : "memory");
          }
#pragma unroll
          for (int j = 0; j < 16 * kPer; ++j) sum[gb * 16 * kPer + j] += __uint_as_float(r[j]);
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(&tempty[b]);
      }
      if (!ok) break;
#pragma unroll
      for (int g = 0; g < BN / 64; ++g, ++nout) {
        float* sb = stg + (nout & 1) * (kOutBlock / 4);
        // the reduce that last read this buffer (two blocks ago) has finished reading it
        if (nout >= 2 && lane == 0) asm volatile("cp.async.bulk.wait_group.read 1;\n" ::: "memory");
        __syncwarp();
        // row = lane: 8 chunks of 16 bytes at the 128B-swizzle positions c ^ (row % 8)
#pragma unroll
        for (int c4 = 0; c4 < 8; ++c4) {
          float4 v = make_float4(-sum[g * 32 + 4 * c4], -sum[g * 32 + 4 * c4 + 1], -sum[g * 32 + 4 * c4 + 2],
                                 -sum[g * 32 + 4 * c4 + 3]);
          *reinterpret_cast<float4*>(sb + lane * 32 + ((c4 ^ (lane & 7)) << 2)) = v;
        }
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // visible to the TMA
        __syncwarp();
        if (lane == 0) {
          tma_reduce_add_2d(&tmC, sb, n0 + h * (BN / 2) + g * 32, m0 + q * 32);
          asm volatile("cp.async.bulk.commit_group;\n" ::: "memory");
        }
      }
    }
    // the reduces are complete before the CTA leaves
    if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");
    __syncwarp();
    if (!ok) *abort_v = 1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (abort_flag) {
      atomicExch(a.err, 1);
      // copies still in flight land before the CTA leaves (bounded waits)
      for (int i = n_consumed; i < n_issued; ++i) mbar_wait(&full[i % kStages], (i / kStages) & 1);
    }
    mbar_wait(&done, 0);
  }
  // teardown: all MMAs and loads have completed; free the accumulators
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols));
  }
}

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// A3[r][s pw + koff + j] (j < P) for rows row0 + r of the columns k0 .. k0 +
// w - 1, planes s = [hi | lo] of the interleaved conj(L) (j = 2 t + f: f = 0
// real part, 1 minus imaginary part), zero for t >= w
__global__ void pack_a_kernel(const zf* __restrict__ LU, int64_t lda, int k0, int w, int row0, int m, int P, int pw,
                              int koff, float* __restrict__ A3) {
  const int K2p = 2 * P;
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (int64_t)m * K2p) return;
  int r = int(e / K2p), k2 = int(e % K2p);
  int s = k2 / P, j = k2 % P, t = j >> 1;
  float out = 0.f;
  if (t < w) {
    zf L = LU[(int64_t)(row0 + r) * lda + k0 + t];
    float v = (j & 1) ? -L.im : L.re;
    float hi = tf32_round(v);
    out = s == 1 ? tf32_round(v - hi) : hi;
  }
  A3[(int64_t)r * 2 * pw + s * pw + koff + j] = out;
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

int make_map(CUtensorMap* map, const float* ptr, int rows, int cols_k, int box_cols, int box_rows,
             CUtensorMapSwizzle swz, int64_t ld = 0) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) {
    set_error("tensor-core LU: cuTensorMapEncodeTiled is not available");
    return M25_ERR_CUDA;
  }
  cuuint64_t dims[2] = {(cuuint64_t)cols_k, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ld ? ld : cols_k) * sizeof(float)};
  cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(ptr), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("tensor-core LU: cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return M25_ERR_CUDA;
  }
  return M25_OK;
}

}  // namespace

bool lu_tc_available() {
  static const bool avail = [] {  // initialised once, also under concurrent first calls
    int dev = 0, major = 0, minor = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    const char* off = getenv("M25_NO_TENSOR_CORES");
    return major == 10 && minor == 3 && encode_fn() != nullptr && !(off && *off == '1');
  }();
  return avail;
}

// packed width of one plane for a panel block of w complex columns
inline int plane_width(int w) { return (2 * w + 63) / 64 * 64; }

inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// Operand buffer of the factorisation of an n x n matrix in super-blocks of
// 256 columns (two blocks of 128, each two panels of 64): a header of
// kTcHeader bytes (error word, then one tile counter per update launch from
// byte 16); A3 (n x 2 x 512) and B3 (2 n x 2 x 512): planes 512 floats wide,
// K of block a's columns in 0..255 and of block b's in 256..511 (A3 holds, in
// turn, block a's L for its rank-128 update of block b's columns, L_ba for
// the product on block b's rows of the trailing columns, and both blocks' L
// for the rank-256 update of the trailing matrix); then Ai and Bi of the
// rank-64 update of a block's second panel (plane width 128, m <= n - 64
// rows, 64 columns).
struct TcLayout {
  size_t a3, b3, ai, bi, total;
};
inline TcLayout tc_layout(int n) {
  TcLayout t;
  const size_t m = (size_t)std::max(n, 1);
  size_t off = kTcHeader;
  t.a3 = off;
  off += align256(sizeof(float) * m * 2 * 512);
  t.b3 = off;
  off += align256(sizeof(float) * 2 * m * 2 * 512);
  t.ai = off;
  off += align256(sizeof(float) * m * 2 * 128);
  t.bi = off;
  off += align256(sizeof(float) * 128 * 2 * 128);
  t.total = off;
  return t;
}

// update launches per super-block of 256 columns: two rank-64 updates, block
// a's rank-128 update of block b's columns, L_ba U_a, the rank-256 update
constexpr int kTcSlotsPerSuper = 5;

int lu_tc_prepare(m25_ctx* ctx, int n) {
  if (kTcSlotsPerSuper * ((n + 255) / 256) + 2 > (kTcHeader - 16) / 4) {
    set_error("tensor-core LU: too many panels");
    return M25_ERR_VALUE;
  }
  int rc = ctx->Dw.ensure(tc_layout(n).total);
  if (rc) return rc;
  M25_CUDA(cudaMemsetAsync(ctx->Dw.p, 0, kTcHeader, ctx->stream));
  return M25_OK;
}

int lu_tc_error(m25_ctx* ctx, int* flag) {
  *flag = 0;
  M25_CUDA(cudaMemcpyAsync(flag, ctx->Dw.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  M25_CUDA(cudaStreamSynchronize(ctx->stream));
  return M25_OK;
}

// the packed operand planes of a factorisation of order n (lu_tc_prepare first)
int lu_tc_buffers(m25_ctx* ctx, int n, float** A3, float** B3, float** Ai, float** Bi) {
  const TcLayout t = tc_layout(n);
  if (t.total > ctx->Dw.bytes) {
    set_error("tensor-core LU: operand buffer not prepared for this size");
    return M25_ERR_VALUE;
  }
  char* b = ctx->Dw.as<char>();
  *A3 = reinterpret_cast<float*>(b + t.a3);
  *B3 = reinterpret_cast<float*>(b + t.b3);
  *Ai = reinterpret_cast<float*>(b + t.ai);
  *Bi = reinterpret_cast<float*>(b + t.bi);
  return M25_OK;
}

// A3 rows 0 .. m - 1 (plane width pw, K offset koff, K extent P per plane)
// from the rows row0 .. row0 + m - 1 of the w columns k0 .. k0 + w - 1
int lu_tc_pack_a(m25_ctx* ctx, const zf* A, int64_t lda, int k0, int w, int row0, int m, int P, int pw, int koff,
                 float* A3) {
  if (m <= 0) return M25_OK;
  StageTimer tm(ctx, ST_PACK);
  const int64_t ta = (int64_t)m * 2 * P;
  pack_a_kernel<<<(unsigned)((ta + 255) / 256), 256, 0, ctx->stream>>>(A, lda, k0, w, row0, m, P, pw, koff, A3);
  M25_CHECK_LAUNCH();
  return M25_OK;
}

// C -= A3 B3 for C = A[r0 .. r0 + m - 1][c0 .. c0 + nc - 1] (complex64, in
// place): A3 (m rows) and B3 (2 nc rows) packed [hi | lo] planes of width pw
// floats, of which the first P (a multiple of 32) take part; slot: the
// header's tile counter of this launch (zeroed by lu_tc_prepare).
int lu_tc_update(m25_ctx* ctx, zf* A, int64_t lda, int r0, int c0, int m, int nc, int P, int pw, const float* A3,
                 const float* B3, int slot) {
  if (m <= 0 || nc <= 0) return M25_OK;
  cudaStream_t st = ctx->stream;
  const int n2 = 2 * nc;
  if (P % kBK || P > pw || pw % kBK || 16 + 4 * (size_t)(slot + 1) > (size_t)kTcHeader) {
    set_error("tensor-core LU: bad update shape");
    return M25_ERR_VALUE;
  }
  int* err = ctx->Dw.as<int>();
  CUtensorMap ma, mb;
  int rc;
  // tile N: the context's choice, else 128 for updates of at most 64 complex
  // columns (one tile without the third of a 192-column tile left empty),
  // 192 otherwise
  const int bn = ctx->tune_tc_bn == 128 || ctx->tune_tc_bn == 192 ? ctx->tune_tc_bn : (n2 <= 128 ? 128 : kBNDefault);
  if ((rc = make_map(&ma, A3, m, 2 * pw, kBK, kBM, CU_TENSOR_MAP_SWIZZLE_128B))) return rc;
  if ((rc = make_map(&mb, B3, n2, 2 * pw, kBK, bn, CU_TENSOR_MAP_SWIZZLE_128B))) return rc;
  // C: the fp32 view of the block, rows 2 lda floats apart, 32 x 32 boxes
  CUtensorMap mc;
  const float* C = reinterpret_cast<const float*>(A + (int64_t)r0 * lda + c0);
  if ((lda & 1) || (reinterpret_cast<uintptr_t>(C) & 15)) {
    set_error("tensor-core LU: C needs an even leading dimension and 16-byte alignment");
    return M25_ERR_VALUE;
  }
  if ((rc = make_map(&mc, C, m, n2, 32, 32, CU_TENSOR_MAP_SWIZZLE_128B, 2 * lda))) return rc;
  const int n_sm = ctx->num_sms;
  static const int chunk = [] {
    const char* e = getenv("M25_TC_CHUNK");
    return e ? std::max(1, atoi(e)) : 1;  // 32 tf32: 12 MMAs (3 products x K 32) per TMEM accumulation
  }();
  TcArgs ta;
  ta.M = m;
  ta.N = n2;
  ta.P = P;
  ta.pw = pw;
  ta.tiles_m = (m + kBM - 1) / kBM;
  ta.ntiles = ta.tiles_m * ((n2 + bn - 1) / bn);
  ta.chunk = (ctx->tune_tc_chunk > 0 ? ctx->tune_tc_chunk : chunk) * (kChunkK / kBK);  // in k-blocks
  ta.err = err;
  ta.counter = reinterpret_cast<int*>(ctx->Dw.as<char>() + 16) + slot;
  static const bool attr =
      cudaFuncSetAttribute(tc_gemm_kernel<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes<128>()) ==
          cudaSuccess &&
      cudaFuncSetAttribute(tc_gemm_kernel<192>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes<192>()) ==
          cudaSuccess;
  if (!attr) {
    set_error("tensor-core LU: the update's shared memory could not be reserved");
    return M25_ERR_CUDA;
  }
  StageTimer tm(ctx, ST_GEMM);
  if (bn == 128)
    tc_gemm_kernel<128><<<std::min(ta.ntiles, n_sm), kThreads, smem_bytes<128>(), st>>>(ma, mb, mc, ta);
  else
    tc_gemm_kernel<192><<<std::min(ta.ntiles, n_sm), kThreads, smem_bytes<192>(), st>>>(ma, mb, mc, ta);
  M25_CHECK_LAUNCH();
  return M25_OK;
}

}  // namespace m25
