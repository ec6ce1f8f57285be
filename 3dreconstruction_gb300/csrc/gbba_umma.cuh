// 5th-generation tensor-core (tcgen05) helpers for sm_103a: tensor-memory
// allocation, shared-memory matrix descriptors, kind::tf32 MMA with FP32
// accumulation in tensor memory, completion through an mbarrier, and the
// tensor-memory loads of the epilogue.  Written as inline PTX.
//
// Operand layout (both operands K-major, no swizzle): a 128 x KC tile is a
// grid of "core matrices" of 8 rows x 16 bytes (4 FP32 values per row, rows
// 16 bytes apart, 128 bytes per core matrix).  Core matrix (r8, k4) sits at
// byte ((r8 * KC / 4) + k4) * 128 from the tile base, so core matrices that
// are neighbours along K are 128 bytes apart (the descriptor's leading
// dimension byte offset) and neighbours along M/N are KC * 32 bytes apart
// (its stride dimension byte offset).
//
// FP32 accuracy from TF32 inputs (3xTF32): every operand value x is split as
// x = hi + lo with hi = x rounded to TF32 and lo = x - hi (exact in FP32),
// and A B^T is accumulated as lo_A hi_B + hi_A lo_B + hi_A hi_B, which leaves
// an error of about 2^-22 relative per product.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gbba {
namespace umma {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Tensor memory: allocated and freed by one whole warp.
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy shared-memory stores become visible to the tensor core's
// (async-proxy) operand reads.
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// Bounded wait for the phase with the given parity; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit = 1u << 24) {
  for (uint32_t it = 0; it < limit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (M/N) byte offsets between core matrices, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::tf32: FP32 accumulator (bits 4-5 = 1),
// A and B TF32 (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0),
// N / 8 at bits 17-22, M / 16 at bits 24-28.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D (+)= A B^T on the tensor core, issued by a single thread.
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.u32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// The mbarrier receives one arrival once every MMA this thread issued before
// has completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

// 32 consecutive accumulator columns of this thread's tensor-memory lane
// (warp w of the CTA reaches lanes 32 (w % 4) .. 32 (w % 4) + 31).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float v[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// ------------------------------------------------------------------ 128 x 128 tile GEMM, K in chunks of 32
constexpr int kTile = 128;
constexpr int kChunk = 32;
constexpr int kOperandFloats = kTile * kChunk;  // one 128 x 32 operand tile (16 KB)

// Shared memory of one tile GEMM: hi and lo parts of the A and B chunks, the
// completion barrier and the tensor-memory base address.
struct GemmSmem {
  float a_hi[kOperandFloats], a_lo[kOperandFloats], b_hi[kOperandFloats], b_lo[kOperandFloats];
  uint64_t bar;
  uint32_t tmem_base;
  uint32_t phase;
};

// Core-layout offset (in floats) of row r, columns 4q..4q+3 of a 128 x 32 chunk.
__device__ __forceinline__ int core_offset(int r, int q) { return ((r >> 3) * (kChunk / 4) + q) * 32 + (r & 7) * 4; }

// One thread's share of a 128 x 32 chunk of a row-major FP32 block: with T
// threads, thread t loads float4 number t, t + T, ... (row idx / 8, columns
// 4 (idx % 8)..), kPer of them.  The loads are issued together (prefetch) and
// stored as hi / lo parts in core layout later (commit), so that a chunk's
// global-memory latency overlaps the previous chunk's MMAs.
template <int kThreads>
struct ChunkRegs {
  static constexpr int kPer = kTile * kChunk / 4 / kThreads;
  float4 v[kPer];
  __device__ __forceinline__ void prefetch(const float* __restrict__ src, int64_t ld, int k0, int valid_rows, int tid) {
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int idx = tid + u * kThreads, r = idx >> 3, q = idx & 7;
      v[u] = r < valid_rows ? __ldcg(reinterpret_cast<const float4*>(src + (int64_t)r * ld + k0 + 4 * q))
                            : make_float4(0.f, 0.f, 0.f, 0.f);
    }
  }
  __device__ __forceinline__ void commit(float* hi, float* lo, int tid) const {
#pragma unroll
    for (int u = 0; u < kPer; ++u) {
      const int idx = tid + u * kThreads, r = idx >> 3, q = idx & 7;
      float4 h, l;
      h.x = tf32_round(v[u].x); l.x = v[u].x - h.x;
      h.y = tf32_round(v[u].y); l.y = v[u].y - h.y;
      h.z = tf32_round(v[u].z); l.z = v[u].z - h.z;
      h.w = tf32_round(v[u].w); l.w = v[u].w - h.w;
      const int o = core_offset(r, q);
      *reinterpret_cast<float4*>(hi + o) = h;
      *reinterpret_cast<float4*>(lo + o) = l;
    }
  }
};

// Set-up by the whole CTA (warp 0 allocates `ncols` tensor-memory columns).
__device__ __forceinline__ void gemm_setup(GemmSmem& g, uint32_t ncols) {
  if (threadIdx.x == 0) {
    mbar_init(&g.bar, 1);
    g.phase = 0;
  }
  if (threadIdx.x < 32) {
    tmem_alloc(&g.tmem_base, ncols);
    tmem_relinquish();
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
}
__device__ __forceinline__ void gemm_teardown(GemmSmem& g, uint32_t ncols) {
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (threadIdx.x < 32) tmem_dealloc(g.tmem_base, ncols);
}

// acc (tensor memory, columns col0..col0+127) = A B^T over K = 32 * nchunks,
// A and B 128-row row-major FP32 blocks (row strides lda, ldb), 3xTF32; rows
// at or beyond a_rows / b_rows are taken as zero (and not read).  All
// kThreads threads of the CTA call it.  The next chunk's loads are in flight
// while the tensor core works on the current one.  Returns false when a
// bounded wait for the tensor core ran out (the caller records the error).
template <int kThreads>
__device__ __forceinline__ bool gemm_tile(GemmSmem& g, uint32_t col0, const float* __restrict__ A, int64_t lda,
                                          const float* __restrict__ B, int64_t ldb, int nchunks, int a_rows = kTile,
                                          int b_rows = kTile) {
  const int tid = threadIdx.x;
  constexpr uint32_t idesc = idesc_tf32(kTile, kTile);
  constexpr uint32_t LBO = 128, SBO = kChunk * 32;
  ChunkRegs<kThreads> ra, rb;
  ra.prefetch(A, lda, 0, a_rows, tid);
  rb.prefetch(B, ldb, 0, b_rows, tid);
  bool ok = true;
  for (int c = 0; c < nchunks; ++c) {
    if (c > 0) {
      // the MMAs of chunk c-1 read the staging buffers asynchronously: wait
      // for them before the buffers are overwritten
      ok = __syncthreads_and(mbar_wait(&g.bar, g.phase) && ok) != 0;
      if (tid == 0) g.phase ^= 1u;
      fence_after_sync();
      if (!ok) break;
    }
    ra.commit(g.a_hi, g.a_lo, tid);
    rb.commit(g.b_hi, g.b_lo, tid);
    if (c + 1 < nchunks) {
      ra.prefetch(A, lda, (c + 1) * kChunk, a_rows, tid);
      rb.prefetch(B, ldb, (c + 1) * kChunk, b_rows, tid);
    }
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      fence_after_sync();
      const uint32_t ah = smem_addr(g.a_hi), al = smem_addr(g.a_lo), bh = smem_addr(g.b_hi), bl = smem_addr(g.b_lo);
#pragma unroll
      for (int kk = 0; kk < kChunk / 8; ++kk) {
        const uint32_t o = kk * 2 * 128;  // two core matrices (8 TF32 values) along K per MMA
        mma_tf32(g.tmem_base + col0, smem_desc(al + o, LBO, SBO), smem_desc(bh + o, LBO, SBO), idesc,
                 (c | kk) != 0);
        mma_tf32(g.tmem_base + col0, smem_desc(ah + o, LBO, SBO), smem_desc(bl + o, LBO, SBO), idesc, 1);
        mma_tf32(g.tmem_base + col0, smem_desc(ah + o, LBO, SBO), smem_desc(bh + o, LBO, SBO), idesc, 1);
      }
      mma_commit(&g.bar);
    }
  }
  if (ok) {
    ok = __syncthreads_and(mbar_wait(&g.bar, g.phase)) != 0;
    if (tid == 0) g.phase ^= 1u;
    fence_after_sync();
    __syncthreads();
  }
  return ok;
}

}  // namespace umma
}  // namespace gbba
