// Split-precision GEMM on the 5th-generation tensor cores (tcgen05) for the
// DFT stages of the precision form.
//
//   D[m][n] = sum_k A[m][k] * B[n][k]        (FP32 accumulation in TMEM)
//
// A and B are given as 16-bit (BF16 or FP16) "hi" and "lo" parts of FP32
// values (x = hi + lo, lo = round16(x - hi)); the product is accumulated from
// the three terms  A_hi B_hi + A_lo B_hi + A_hi B_lo  (the lo*lo term is below
// FP32 rounding), which restores ~16 (BF16) or ~22 (FP16) significant bits.
//
// Operand layout in global memory ("blocked core-matrix" layout, produced
// directly by the kernels that write the operands): rows are cut into tiles
// of TR rows (A: 128, B: BN), K into chunks of 64; a (tile, chunk) block is
// TR*64 contiguous elements made of 8x8 core matrices (8 rows x 16 bytes,
// rows 16 bytes apart) ordered [row group][k group]:
//
//   off(r, k) = ((tile * KC + chunk) * (TR/8) + rg) * 512 + kg * 64 + (r%8)*8 + k%8
//   tile = r / TR, rg = (r % TR) / 8, chunk = k / 64, kg = (k % 64) / 8
//
// which is the tcgen05 K-major no-swizzle canonical layout with leading
// (K-direction) byte offset 128 and stride (row-group) byte offset 1024, so a
// block moves to shared memory with one bulk copy (cp.async.bulk) and is read
// by the MMA in place.
//
// One CTA of 128 threads computes a 128 x BN tile: thread 0 issues the bulk
// copies (double-buffered K chunks, mbarrier transaction counts) and the
// MMAs (M=128, N=BN, K=16 each, 12 per chunk); the accumulator lives in BN
// TMEM columns; all four warps then read their 32 TMEM lanes (rows) back
// with tcgen05.ld and hand them to the epilogue.  Every wait is bounded: on
// timeout the CTA records LGB_ERR_DEVICE_TIMEOUT in *err, waits (bounded) for
// its in-flight bulk copies and MMAs, frees its TMEM and returns.  If one of
// those last waits also runs out, asynchronous work of the CTA may still be
// pending when it exits: after LGB_ERR_DEVICE_TIMEOUT the caller treats the
// CUDA context as unusable (no further launches on it).
#pragma once

#include <stdint.h>

#include "common.cuh"

namespace lgb {

constexpr int kTcM = 128;     // MMA rows per CTA (TMEM lanes)
constexpr int kTcKC = 64;     // K elements per pipeline chunk
constexpr int kTcThreads = 128;
constexpr unsigned kTcSpinLimit = 1u << 22;  // mbarrier polls before giving up (~seconds at most)

__host__ __device__ constexpr size_t tc_block_elems(int rows) { return (size_t)rows * kTcKC; }

// element offset of (r, k) in the blocked layout with TR-row tiles and KC chunks
__host__ __device__ inline size_t tc_offset(int r, int k, int TR, int KC) {
  const int tile = r / TR, rr = r - tile * TR;
  const int chunk = k / kTcKC, kk = k - chunk * kTcKC;
  return (((size_t)tile * KC + chunk) * (TR / 8) + rr / 8) * 512 + (size_t)(kk / 8) * 64 + (rr % 8) * 8 + kk % 8;
}

// ----------------------------------------------------------------------------
// PTX wrappers
// ----------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// true once the phase with the given parity has completed
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait; false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned limit = kTcSpinLimit) {
  for (unsigned i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// 1-D bulk copy global -> shared, completing `bytes` transactions on bar
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// warp-collective TMEM allocation; the base address is written to *slot
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// K-major, no-swizzle shared-memory matrix descriptor
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
  return d;                // base offset 0, layout type 0 (no swizzle)
}

// instruction descriptor, kind::f16: FP32 accumulator, A/B BF16 (or FP16), both K-major
__host__ __device__ constexpr uint32_t mma_idesc(int M, int N, bool f16) {
  return (1u << 4)                      // D format: F32
         | ((f16 ? 0u : 1u) << 7)       // A format: F16 = 0, BF16 = 1
         | ((f16 ? 0u : 1u) << 10)      // B format
         | ((uint32_t)(N >> 3) << 17)   // N / 8
         | ((uint32_t)(M >> 4) << 24);  // M / 16
}

__device__ __forceinline__ void mma_f16(uint32_t taddr, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// ----------------------------------------------------------------------------
// 16-bit split of FP32 values
// ----------------------------------------------------------------------------
template <bool F16>
struct Split16;
template <>
struct Split16<false> {  // BF16
  static __device__ __forceinline__ void run(float x, uint16_t* hi, uint16_t* lo) {
    const __nv_bfloat16 h = __float2bfloat16_rn(x);
    const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
    *hi = __bfloat16_as_ushort(h);
    *lo = __bfloat16_as_ushort(l);
  }
};
template <>
struct Split16<true> {  // FP16
  static __device__ __forceinline__ void run(float x, uint16_t* hi, uint16_t* lo) {
    const __half h = __float2half_rn(x);
    const __half l = __float2half_rn(x - __half2float(h));
    *hi = __half_as_ushort(h);
    *lo = __half_as_ushort(l);
  }
};

// ----------------------------------------------------------------------------
// The GEMM kernel.  Epi::apply(row, col0, v[32], params) consumes 32 columns
// of one output row (row = global m, col0 = global n of v[0]).
// ----------------------------------------------------------------------------
struct TcGemmArgs {
  const uint16_t* a_hi;
  const uint16_t* a_lo;
  const uint16_t* b_hi;
  const uint16_t* b_lo;
  int k_chunks;  // K / 64
  int terms;     // 1: hi*hi only; 3: hi*hi + lo*hi + hi*lo
  int* err;      // LGB_ERR_DEVICE_TIMEOUT on a bounded-wait timeout
  int kc_split;  // > 0: CTA z accumulates chunks [z*kc_split, (z+1)*kc_split) only (split K; the
                 // epilogue then adds its partial sums atomically); 0: all chunks
};

// Shared memory of one CTA: two pipeline stages of [A hi | A lo | B hi | B lo]
// K chunks, or [A hi | B hi] when the kernel is built without lo terms (LO =
// false: half the footprint, so more CTAs fit an SM for single-term GEMMs).
template <int BN, bool LO = true>
struct TcSmem {
  static constexpr int A_BYTES = kTcM * kTcKC * 2;  // 16 KB
  static constexpr int B_BYTES = BN * kTcKC * 2;
  static constexpr int B_OFF = (LO ? 2 : 1) * A_BYTES;  // B hi within a stage
  static constexpr int STAGE = (LO ? 2 : 1) * (A_BYTES + B_BYTES);
  static constexpr int STAGES = 2;
  static constexpr int BYTES = STAGES * STAGE + 1024 /* alignment */ + 128 /* barriers */;
};

template <class Epi, int BN, bool F16, bool LO = true>
__global__ void __launch_bounds__(kTcThreads, 1)
    tc_gemm_kernel(TcGemmArgs g, typename Epi::Params ep) {
  static_assert(BN % 32 == 0 && BN >= 32 && BN <= 256, "N tile");
  using S = TcSmem<BN, LO>;
  extern __shared__ uint8_t tc_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tc_raw) + 1023) & ~(uintptr_t)1023);
  uint64_t* full = reinterpret_cast<uint64_t*>(base + S::STAGES * S::STAGE);
  uint64_t* empty = full + 2;
  uint64_t* done = full + 4;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(full + 6);
  __shared__ int s_fail;

  const int warp = threadIdx.x >> 5;
  const int m_tile = blockIdx.y, n_tile = blockIdx.x;
  const int KC = g.k_chunks;
  const int kc0 = g.kc_split > 0 ? (int)blockIdx.z * g.kc_split : 0;  // first chunk of this CTA
  const int NK = g.kc_split > 0 ? min(KC - kc0, g.kc_split) : KC;     // chunks of this CTA (>= 1)
  const bool lo_terms = LO && g.terms == 3;  // built without lo buffers: hi*hi only

  if (threadIdx.x == 0) {
    for (int i = 0; i < 2; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    mbar_init(done, 1);
    s_fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(tslot, BN < 32 ? 32 : BN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  if (threadIdx.x == 0) {
    const size_t a_blk = tc_block_elems(kTcM), b_blk = tc_block_elems(BN);
    const uint32_t stage_bytes = lo_terms ? (uint32_t)S::STAGE : (uint32_t)(S::A_BYTES + S::B_BYTES);
    auto load = [&](int kc) {
      uint8_t* st = base + (kc & 1) * S::STAGE;
      const size_t ao = ((size_t)m_tile * KC + kc0 + kc) * a_blk, bo = ((size_t)n_tile * KC + kc0 + kc) * b_blk;
      mbar_expect_tx(&full[kc & 1], stage_bytes);
      bulk_g2s(st, g.a_hi + ao, S::A_BYTES, &full[kc & 1]);
      bulk_g2s(st + S::B_OFF, g.b_hi + bo, S::B_BYTES, &full[kc & 1]);
      if (lo_terms) {
        bulk_g2s(st + S::A_BYTES, g.a_lo + ao, S::A_BYTES, &full[kc & 1]);
        bulk_g2s(st + S::B_OFF + S::B_BYTES, g.b_lo + bo, S::B_BYTES, &full[kc & 1]);
      }
    };
    const uint32_t idesc = mma_idesc(kTcM, BN, F16);
    bool ok = true;
    int issued = 0, landed = 0;  // chunks whose copies were issued / have been waited for
    load(0);
    ++issued;
    if (NK > 1) {
      load(1);
      ++issued;
    }
    for (int kc = 0; kc < NK && ok; ++kc) {
      const int s = kc & 1;
      if (!mbar_wait(&full[s], (kc >> 1) & 1)) {
        ok = false;
        break;
      }
      ++landed;
      tc_fence_after();
      const uint32_t sa = smem_u32(base + s * S::STAGE);
      const uint32_t sb = sa + S::B_OFF;
      // term order: hi*hi, lo(A)*hi(B), hi(A)*lo(B)
      for (int t = 0; t < (lo_terms ? 3 : 1); ++t) {
        const uint32_t a0 = sa + (t == 1 ? S::A_BYTES : 0);
        const uint32_t b0 = sb + (t == 2 ? S::B_BYTES : 0);
#pragma unroll
        for (int j = 0; j < kTcKC / 16; ++j) {
          const uint64_t ad = smem_desc(a0 + j * 256, 128, 1024);
          const uint64_t bd = smem_desc(b0 + j * 256, 128, 1024);
          mma_f16(tmem, ad, bd, idesc, (kc | t | j) != 0);
        }
      }
      mma_commit(&empty[s]);
      // chunk kc+1 goes into the stage of chunk kc-1 once that chunk's MMAs have
      // read it; chunk kc's MMAs keep the tensor pipe busy meanwhile
      if (kc >= 1 && kc + 1 < NK) {
        if (!mbar_wait(&empty[(kc - 1) & 1], ((kc - 1) >> 1) & 1)) {
          ok = false;
          break;
        }
        load(kc + 1);
        ++issued;
      }
    }
    if (!ok) {
      s_fail = 1;
      atomicExch(g.err, LGB_ERR_DEVICE_TIMEOUT);
      // copies still in flight target this CTA's shared memory: wait (bounded)
      // for each before the CTA may exit
      for (int j = landed; j < issued; ++j) mbar_wait(&full[j & 1], (j >> 1) & 1);
    }
    mma_commit(done);  // tracks every MMA this thread issued
  }
  __syncthreads();
  // wait for the accumulator (bounded, every thread)
  const bool have = mbar_wait(done, 0);
  tc_fence_after();
  if (!have && threadIdx.x == 0) atomicExch(g.err, LGB_ERR_DEVICE_TIMEOUT);
  const bool good = have && !s_fail;
  // epilogue: warp w owns TMEM lanes [32w, 32w + 32)
  if (__all_sync(0xffffffffu, good)) {
    const int row = m_tile * kTcM + warp * 32 + (threadIdx.x & 31);
    const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 32) {
      float v[32];
      tmem_ld32(lane_addr + (uint32_t)c0, v);
      Epi::apply(row, n_tile * BN + c0, v, ep);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, BN < 32 ? 32 : BN);
}

}  // namespace lgb
