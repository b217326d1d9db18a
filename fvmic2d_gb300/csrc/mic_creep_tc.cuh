// mic_creep_tc.cuh -- tensor-core (tcgen05) inference of the creep surrogate for one tile of
// 128 markers per 128-thread block.
//
// Layer 1 (4 -> 64) and the SiLUs run on the CUDA cores in FP32.  The hidden layer
// z2 = h1 W2^T (M = 128 markers, N = 64, K = 64) runs as tcgen05.mma kind::f16 with BF16
// operands and an FP32 accumulator in tensor memory.  W2 is BF16 by construction (bf16_round);
// the FP32 activations enter as two BF16 pieces, h1_hi W2 + h1_lo W2 with h1_hi = bf16(h1) and
// h1_lo = bf16(h1 - h1_hi), so the layer is FP32-accurate in h1.  Thread t of the block owns
// marker row t: it writes that row of the A operand, and reads row t of the accumulator back
// (TMEM lane t) with tcgen05.ld.  Shared memory per block (42 KB) and at most 102 registers a
// thread let kBlocksPerSM = 5 blocks share an SM; their TMEM (5 x 64 of 512 columns) never
// makes an allocation wait.
//
// Shared-memory operand layout (no swizzle, K-major core matrices of 8 rows x 16 bytes):
// element (row, k) of a 64-wide operand sits at (row/8)*1024 + (k/8)*128 + (row%8)*16 + (k%8)*2,
// so the stride between core matrices along K (leading byte offset) is 128 bytes and along the
// rows (stride byte offset) 1024 bytes.  The MMA over k in [16j, 16j+16) starts at +256 j.
//
// Every wait on the MMA's completion barrier is bounded (the limit is a context setting,
// mic_creep_set_tc_wait_limit); a block whose wait runs out stops using the tensor cores,
// reports it, and its markers take the exact solve.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include "mic_creep.cuh"

namespace mic {
namespace tc {

constexpr int kTile = 128;              // markers per block tile = MMA M = TMEM lanes
constexpr int kTmemCols = 64;           // FP32 accumulator columns (N)
constexpr int kBlocksPerSM = 5;         // blocks that fit an SM (launch bounds: at most 102 registers)
// blocks per SM of the persistent grids (all that fit: leaving one SM slot to the first
// projection's partial sums on the second stream measured slower)
constexpr int kGridBlocksPerSM = 5;
constexpr uint32_t kOpA = 128 * 64 * 2;  // bytes of one A operand (hi or lo)
constexpr uint32_t kOpB = 64 * 64 * 2;   // bytes of one B operand
// small parameters in shared memory, neuron-major so that each neuron's are two 16-byte loads:
// float4 {W1[k][0..3]}, float4 {b1[k], b2[k], w3[k], 0} for k < 64, then b3
constexpr int kNSmall = 8 * kH + 4;

struct Smem {  // offsets from a 128-byte aligned base (the no-swizzle operands need 16 bytes)
  static constexpr uint32_t a_hi = 0, a_lo = kOpA, b = 2 * kOpA;
  static constexpr uint32_t small = 2 * kOpA + kOpB;                 // kNSmall floats
  static constexpr uint32_t bar = small + ((kNSmall * 4 + 15) / 16) * 16;  // mbarrier (8 B)
  static constexpr uint32_t taddr = bar + 8;                          // TMEM address (4 B)
  static constexpr uint32_t bytes = taddr + 8;
};
constexpr uint32_t kAlign = 128;
constexpr size_t kDynSmem = Smem::bytes + kAlign;  // + alignment slack
// kBlocksPerSM blocks' dynamic and static shared memory (the job record, 1.4 KB) and the 1 KB the
// hardware reserves per block, within the SM's 228 KB
static_assert(kBlocksPerSM * (kDynSmem + 1536 + 1024) <= 228 * 1024, "tensor-core blocks do not fit an SM");

// instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12 = 1),
// both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(64 >> 3) << 17) |
                            ((uint32_t)(128 >> 4) << 24);

__device__ __forceinline__ uint32_t core_offset(int row, int k) {
  return (uint32_t)((row >> 3) * 1024 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor: start >> 4 (bits 0-13), leading byte offset >> 4 (16-29),
// stride byte offset >> 4 (32-45), descriptor version 1 (bits 46-47), no swizzle (61-63 = 0)
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) |
         (1ull << 46);
}

__device__ __forceinline__ uint32_t bf16_pair(float lo_elem, float hi_elem) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo_elem, hi_elem);  // .x = first (lower address)
  return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ void mbar_init(uint32_t bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// bounded wait on phase `parity` of the barrier; false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int limit) {
  for (int i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// one warp: allocate kTmemCols columns, address written to shared memory at dst
__device__ __forceinline__ void tmem_alloc(uint32_t dst) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst), "r"(kTmemCols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(kTmemCols) : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
               : "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  // the registers are written asynchronously: tie every use to the completion wait
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                 "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]),
                 "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]),
                 "+r"(r[29]), "+r"(r[30]), "+r"(r[31])
               :
               : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

constexpr int kWaitLimit = 1 << 20;  // default try_wait rounds before a block gives up on the MMA
constexpr int kDrainLimit = 1 << 22;  // try_wait rounds of the final drain before TMEM is freed

// Per-block state of the tensor-core surrogate.
struct Block {
  unsigned char *base;  // 1024-aligned dynamic shared memory
  uint32_t sbase;       // its shared-window address
  uint32_t tmem;        // TMEM accumulator address (lane 0, first column)
  uint32_t phase;       // parity of the next barrier completion
  int ok;               // block-uniform: tensor path usable
  int pending;          // a committed MMA whose completion was not observed
};

// All kTile threads: write W2 (hi/lo BF16, the B operand) and the small parameters of network p
// into the block's shared memory (no fence, no barrier).
__device__ __forceinline__ void stage_params(Block &B, const float *__restrict__ p) {
  const int t = threadIdx.x;
  // W2 rows n (outputs) x k (inputs) as BF16, K-major core matrices; 64 x 8 groups of 8 elements
  for (int g = t; g < kH * 8; g += kTile) {
    const int n = g >> 3, kg = g & 7;
    uint32_t w[4];
#pragma unroll
    for (int e = 0; e < 4; ++e)
      w[e] = bf16_pair(p[kOffW2 + n * kH + kg * 8 + 2 * e], p[kOffW2 + n * kH + kg * 8 + 2 * e + 1]);
    *reinterpret_cast<uint4 *>(B.base + Smem::b + core_offset(n, kg * 8)) = make_uint4(w[0], w[1], w[2], w[3]);
  }
  float4 *sp4 = reinterpret_cast<float4 *>(B.base + Smem::small);
  for (int k = t; k < kH; k += kTile) {
    sp4[2 * k] = make_float4(p[kOffW1 + 4 * k], p[kOffW1 + 4 * k + 1], p[kOffW1 + 4 * k + 2], p[kOffW1 + 4 * k + 3]);
    sp4[2 * k + 1] = make_float4(p[kOffB1 + k], p[kOffB2 + k], p[kOffW3 + k], 0.0f);
  }
  if (t == 0) sp4[2 * kH] = make_float4(p[kOffB3], 0.0f, 0.0f, 0.0f);
}

// All kTile threads: carve shared memory, stage W2 (BF16) and the small parameters, allocate
// TMEM (warp 0) and initialise the barrier (thread 0).
__device__ __forceinline__ void setup(Block &B, unsigned char *dyn, const float *__restrict__ p) {
  const uint32_t s0 = (uint32_t)__cvta_generic_to_shared(dyn);
  const uint32_t pad = (kAlign - (s0 & (kAlign - 1))) & (kAlign - 1);
  B.base = dyn + pad;
  B.sbase = s0 + pad;
  B.phase = 0;
  B.ok = 1;
  B.pending = 0;
  const int t = threadIdx.x;
  stage_params(B, p);
  if (t < 32) tmem_alloc(B.sbase + Smem::taddr);
  if (t == 0) mbar_init(B.sbase + Smem::bar);
  fence_proxy_async();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  B.tmem = *reinterpret_cast<volatile uint32_t *>(B.base + Smem::taddr);
}

// All kTile threads, block-uniform, between two guesses: replace the staged network by p (a batch
// of ensemble members whose networks live in different buffers).  Every MMA of the block has
// completed by then (guess returns after its completion wait), so the operands are free; a
// block that gave up on the tensor path keeps what it has (an abandoned MMA may still read it,
// and its markers take the exact solve anyway).
__device__ __forceinline__ void restage(Block &B, const float *__restrict__ p) {
  __syncthreads();  // every thread has finished the last epilogue's reads of the small parameters
  if (B.ok) stage_params(B, p);
  fence_proxy_async();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
}

// All kTile threads, block-uniform: network output y for this thread's features (NaN when the
// block has stopped using the tensor path).  `active` threads carry real features; the others
// feed zeros and ignore the result.  wait_limit: try_wait rounds on the MMA's completion before
// the block gives up (the context's setting, default kWaitLimit).
// The loops over the 64 neurons are not unrolled whole (`unroll 1` on the outer loops): the
// yield kernel that inlines this is large, and with its MLP unrolled its warps stalled on
// instruction fetch about as often as on memory; rolled, the kernel runs 10% faster for a few
// loop instructions more.
__device__ __forceinline__ float guess(Block &B, const float f[4], int wait_limit, unsigned long long *timeouts) {
  const int t = threadIdx.x;
  const float4 *sp4 = reinterpret_cast<const float4 *>(B.base + Smem::small);
  if (B.ok) {
    // layer 1 on the CUDA cores, row t of A as hi and lo BF16 pieces
#pragma unroll 1
    for (int kg = 0; kg < 8; ++kg) {
      uint32_t hi[4], lo[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        float h[2];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
          const int k = kg * 8 + 2 * e + u;
          const float4 w = sp4[2 * k];
          const float z = fmaf(w.w, f[3], fmaf(w.z, f[2], fmaf(w.y, f[1], fmaf(w.x, f[0], sp4[2 * k + 1].x))));
          h[u] = silu(z);
        }
        const float h0 = __bfloat162float(__float2bfloat16_rn(h[0])), h1 = __bfloat162float(__float2bfloat16_rn(h[1]));
        hi[e] = bf16_pair(h0, h1);
        lo[e] = bf16_pair(h[0] - h0, h[1] - h1);
      }
      const uint32_t off = core_offset(t, kg * 8);
      *reinterpret_cast<uint4 *>(B.base + Smem::a_hi + off) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
      *reinterpret_cast<uint4 *>(B.base + Smem::a_lo + off) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
    }
  }
  fence_proxy_async();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (!B.ok) return __int_as_float(0x7fc00000);
  if (t == 0) {
    const uint32_t ahi = B.sbase + Smem::a_hi, alo = B.sbase + Smem::a_lo, bw = B.sbase + Smem::b;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t o = 256u * j;
      mma_bf16(B.tmem, smem_desc(ahi + o), smem_desc(bw + o), j > 0 ? 1u : 0u);
      mma_bf16(B.tmem, smem_desc(alo + o), smem_desc(bw + o), 1u);
    }
    mma_commit(B.sbase + Smem::bar);
  }
  const bool done = mbar_wait(B.sbase + Smem::bar, B.phase, wait_limit);
  if (!__syncthreads_and(done)) {  // block-uniform give-up: never touch the accumulator again
    B.ok = 0;
    B.pending = 1;
    if (t == 0) atomicAdd(timeouts, 1ULL);
    return __int_as_float(0x7fc00000);
  }
  B.phase ^= 1u;
  fence_after_sync();
  // epilogue: row t of the accumulator (TMEM lanes 32w.. for warp w), bias, SiLU, output layer
  const uint32_t row = B.tmem + ((uint32_t)(t & ~31) << 16);
  float y = sp4[2 * kH].x;
#pragma unroll 1
  for (int half = 0; half < 2; ++half) {
    float z[32];
    tmem_ld32(row + 32u * half, z);
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      const float4 q = sp4[2 * (32 * half + i) + 1];  // b1, b2, w3 of neuron n
      y = fmaf(q.z, silu(z[i] + q.y), y);
    }
  }
  // the next tile's MMA may overwrite the accumulator only after every lane has read it
  fence_before_sync();
  return y;
}

// All kTile threads at the end: drain (bounded) a committed MMA whose completion was not
// observed, then free TMEM (warp 0).  The drain waits on the same barrier phase the give-up
// abandoned: the MMA chain writes only this block's TMEM columns and arrives on the barrier when
// it is done, so once the phase completes nothing is in flight and the columns can be freed.
// A drain that runs out as well (the tensor pipe never signalled) is counted in
// *drain_timeouts and the columns are freed regardless, since a CTA must release its TMEM
// before it exits; a nonzero count means the accumulator may have been overwritten after the
// free and the pass's tensor-core results are void (its markers took the exact solve).
__device__ __forceinline__ void teardown(Block &B, unsigned long long *drain_timeouts) {
  if (B.pending) {
    const bool drained = mbar_wait(B.sbase + Smem::bar, B.phase, kDrainLimit);
    if (!__syncthreads_and(drained) && threadIdx.x == 0) atomicAdd(drain_timeouts, 1ULL);
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (threadIdx.x < 32) tmem_dealloc(B.tmem);
}

}  // namespace tc
}  // namespace mic
