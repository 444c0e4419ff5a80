// Fifth-generation tensor cores (sm_100a family): TMEM accumulators,
// single-thread MMA issue with operands described in shared memory, mbarrier
// completion, and the split-TF32 128 x 128 tile product built on them.
// kind::f16 MMAs on BF16 operands use the same layout with 64 entries per
// 128-byte row (K = 16 per MMA, the same 32-byte step).
//
// Operand layout: K-major, 128-byte swizzle.  A 128 x 32 FP32 tile is 128 rows
// of 128 bytes; 16-byte chunk c of row r is stored at chunk position
// c ^ (r % 8), rows of 8 form 1024-byte atoms (the tile starts on a 1024-byte
// boundary).  Descriptor: start address >> 4, stride between 8-row groups
// 1024 bytes, 128-byte swizzle; one MMA consumes K = 8 (32 bytes), the next
// K step advances the start address by 32 bytes inside the swizzled rows.
//
// Every wait on an mbarrier is bounded; a timeout sets ST_TIMEOUT in the
// caller's status word and the tile is abandoned after the MMAs already
// issued have been waited for (again bounded) and the TMEM released.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace nqg {

namespace t5 {

constexpr long long WAIT_LIMIT = 1ll << 24;  // mbarrier polls before a wait gives up

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// K-major, 128-byte swizzle shared-memory matrix descriptor.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address, 16-byte units
  d |= (uint64_t)1 << 16;                    // leading byte offset (unused by swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset: next 8-row group
  d |= (uint64_t)1 << 46;                    // descriptor version
  d |= (uint64_t)2 << 61;                    // 128-byte swizzle
  return d;
}

// Instruction descriptor: kind::tf32, FP32 accumulator, both operands K-major.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
  return (1u << 4)                        // D format F32
         | (2u << 7)                      // A format TF32
         | (2u << 10)                     // B format TF32
         | ((uint32_t)(N >> 3) << 17)     // N / 8
         | ((uint32_t)(M >> 4) << 24);    // M / 16
}

// Instruction descriptor: kind::f16 with BF16 A and B, FP32 accumulator, both
// operands K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4)                        // D format F32
         | (1u << 7)                      // A format BF16
         | (1u << 10)                     // B format BF16
         | ((uint32_t)(N >> 3) << 17)     // N / 8
         | ((uint32_t)(M >> 4) << 24);    // M / 16
}

__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
// One K = 16 step of BF16 operands (32 bytes of each swizzled row, as one
// K = 8 step of TF32).
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait for phase `parity` of an mbarrier; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
  for (long long it = 0; it < WAIT_LIMIT; ++it)
    if (mbar_test(mbar, parity)) return true;
  return false;
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}
// Bulk copy global -> shared (no tensor map): both addresses 16-byte aligned,
// size a multiple of 16; completion counted in bytes on the mbarrier.
__device__ __forceinline__ void bulk_g2s(uint32_t dst_smem, const void *src, uint32_t bytes, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst_smem),
      "l"(src), "r"(bytes), "r"(mbar)
      : "memory");
}

// 32 lanes x 32 consecutive 32-bit columns: thread i of the warp receives
// lane (taddr.lane + i), columns [taddr.col, taddr.col + 32).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
        "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
        "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ uint32_t tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// Split-BF16 pair: x = hi + lo with hi = bf16(x), lo = bf16(x - hi) (round to
// nearest even; |x - hi - lo| <= 2^-16 |x| for normal values), two
// consecutive K entries per 32-bit word, x0 in the low half (lower address).
__device__ __forceinline__ void bf16_split2(float x0, float x1, uint32_t &hi, uint32_t &lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);
  const __nv_bfloat162 l = __floats2bfloat162_rn(x0 - __low2float(h), x1 - __high2float(h));
  hi = *reinterpret_cast<const uint32_t *>(&h);
  lo = *reinterpret_cast<const uint32_t *>(&l);
}

// Tile geometry of the split-TF32 product.
constexpr int TM = 128, TN = 128, TK = 32;        // rows, columns, K per stage
constexpr int OPND_BYTES = TM * TK * 4;           // one 128 x 32 FP32 operand tile (16 KB)
constexpr int STAGE_BYTES = 4 * OPND_BYTES;       // A hi, A lo, B hi, B lo
constexpr int THREADS = 128;                      // four warps: TMEM lanes 0-127
// dynamic shared memory of a tile product with NST operand stages
__host__ __device__ constexpr int smem_bytes(int nst) { return nst * STAGE_BYTES + 1024 + 64; }

// Thread r writes row r (32 FP32 values of K) of an operand tile, split into
// hi / lo TF32 parts, in the swizzled layout.
__device__ __forceinline__ void store_row_split(unsigned char *hi_tile, unsigned char *lo_tile, int r,
                                                const float (&x)[TK]) {
#pragma unroll
  for (int c = 0; c < TK / 4; ++c) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      h[q] = tf32_rna(x[4 * c + q]);
      l[q] = tf32_rna(x[4 * c + q] - __uint_as_float(h[q]));
    }
    const int off = r * 128 + ((c ^ (r & 7)) << 4);
    *reinterpret_cast<uint4 *>(hi_tile + off) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4 *>(lo_tile + off) = make_uint4(l[0], l[1], l[2], l[3]);
  }
}

// acc(128 x 128) = A(128 x kdim) * B(128 x kdim)^T with split-TF32 products,
// by a CTA of THREADS threads.  Row loaders fa(r, k0, x) / fb(n, k0, x) fill
// x[0..TK) with entries k0 .. k0+TK-1 of operand row r / n (0 outside the
// operands), called with r, n = threadIdx.x.  The
// epilogue ep(r, c0, v) receives, for row r = threadIdx.x, the 32 product
// values of columns [c0, c0 + 32).  smem_raw: smem_bytes(NSTAGE) of dynamic
// shared memory (NSTAGE operand stages of 64 KB: with one stage three CTAs fit
// on an SM; the next K chunk is loaded into registers while the MMAs run).
// Called at most once per CTA (the TMEM allocation permit is relinquished).  Returns false on a timeout (ST_TIMEOUT set in *status).
template <int NSTAGE, class FA, class FB, class EP>
__device__ bool tile_tf32x3(int kdim, FA fa, FB fb, EP ep, unsigned char *smem_raw, int *status) {
  const int tid = threadIdx.x, warp = tid >> 5;
  unsigned char *base =
      reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  uint64_t *mbar = reinterpret_cast<uint64_t *>(base + NSTAGE * STAGE_BYTES);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(base + NSTAGE * STAGE_BYTES + 32);
  __shared__ int s_fail;
  if (warp == 0) tmem_alloc(smem_u32(tslot), TN);
  if (tid == 0) {
    s_fail = 0;
    for (int s = 0; s < NSTAGE; ++s) mbar_init(smem_u32(&mbar[s]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tslot;
  constexpr uint32_t IDESC = idesc_tf32(TM, TN);
  uint32_t uses[NSTAGE] = {};
  const int nchunk = (kdim + TK - 1) / TK;
  int last_stage = -1;
  bool ok = true;
  // operand rows of the next chunk are loaded into registers while the
  // tensor cores work on the current one
  float xa[TK], xb[TK];
  if (nchunk > 0) {
    fa(tid, 0, xa);
    fb(tid, 0, xb);
  }
  for (int ch = 0; ch < nchunk && ok; ++ch) {
    const int s = ch % NSTAGE;
    unsigned char *stg = base + s * STAGE_BYTES;
    // the MMAs that last read this stage must have completed
    if (uses[s] > 0) {
      if (tid == 0 && !mbar_wait(smem_u32(&mbar[s]), (uses[s] - 1) & 1)) s_fail = 1;
      __syncthreads();
      if (s_fail) {
        ok = false;
        break;
      }
    }
    store_row_split(stg, stg + OPND_BYTES, tid, xa);
    store_row_split(stg + 2 * OPND_BYTES, stg + 3 * OPND_BYTES, tid, xb);
    fence_proxy_async();
    __syncthreads();
    if (tid == 0) {
      fence_after();
      const uint32_t a_hi = smem_u32(stg), a_lo = a_hi + OPND_BYTES;
      const uint32_t b_hi = a_hi + 2 * OPND_BYTES, b_lo = a_hi + 3 * OPND_BYTES;
#pragma unroll
      for (int ks = 0; ks < TK / 8; ++ks) {
        const uint32_t off = ks * 32;
        const uint32_t acc0 = (ch > 0 || ks > 0) ? 1u : 0u;
        mma_tf32(tmem, desc_sw128(a_lo + off), desc_sw128(b_hi + off), IDESC, acc0);
        mma_tf32(tmem, desc_sw128(a_hi + off), desc_sw128(b_lo + off), IDESC, 1u);
        mma_tf32(tmem, desc_sw128(a_hi + off), desc_sw128(b_hi + off), IDESC, 1u);
      }
      mma_commit(smem_u32(&mbar[s]));
    }
    ++uses[s];
    last_stage = s;
    if (ch + 1 < nchunk) {
      fa(tid, (ch + 1) * TK, xa);
      fb(tid, (ch + 1) * TK, xb);
    }
  }
  // wait for every issued MMA (bounded), then read the accumulator
  if (tid == 0) {
    for (int s = 0; s < NSTAGE; ++s)
      if (uses[s] > 0 && !mbar_wait(smem_u32(&mbar[s]), (uses[s] - 1) & 1)) s_fail = 1;
  }
  __syncthreads();
  fence_after();
  ok = ok && !s_fail && last_stage >= 0;
  if (tid == 0)
    for (int s = 0; s < NSTAGE; ++s) asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&mbar[s])) : "memory");
  if (ok) {
#pragma unroll 1
    for (int c0 = 0; c0 < TN; c0 += 32) {
      uint32_t v[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      ep(tid, c0, v);
    }
  } else if (tid == 0) {
    atomicOr(status, 4 /* ST_TIMEOUT */);
  }
  fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, TN);
  return ok;
}

}  // namespace t5

}  // namespace nqg
