// Blackwell (sm_103a) building blocks shared by the tensor-core scan kernels: tile
// geometry, mbarriers with bounded waits, TMA tile loads, tcgen05 MMA / commit / TMEM
// loads, and the tensor-map encoder.  Everything here is inline PTX written for this
// project; no library kernels are involved.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "common.cuh"

namespace lshg {
namespace tc {

constexpr int BM = 128;                     // queries per tile = UMMA M = TMEM lanes
constexpr int BN = 128;                     // base points per tile = UMMA N
constexpr int KD = 128;                     // padded dimension (bf16 rows of 256 B)
constexpr int KHALF = 64;                   // bf16 elements per 128-byte swizzle row
constexpr int HALF_BYTES = BN * KHALF * 2;  // 16 KB: one 64-column half of a tile
constexpr int TILE_BYTES = 2 * HALF_BYTES;  // 32 KB: one 128 x 128 bf16 tile
constexpr uint64_t kWaitNs = 2000000000ull; // every pipeline wait gives up after ~2 s

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// try_wait that may suspend the thread until the phase completes or `hint_ns` passes, so
// waiting warps do not take issue slots from the working ones.
__device__ __forceinline__ bool mbar_try_sleep(uint32_t bar, uint32_t parity, uint32_t hint_ns) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity), "r"(hint_ns)
      : "memory");
  return ok != 0;
}
// Bounded wait: gives up when another role aborted (unless `ignore_abort`) or after
// kWaitNs, raising the CTA's abort flag.
static __device__ __noinline__ bool mbar_wait_slow(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                            bool ignore_abort) {
  const uint64_t t0 = global_ns();
  while (true) {
    if (mbar_try_sleep(bar, parity, 20000u)) return true;
    if (!ignore_abort && *abort_flag) return false;
    if (global_ns() - t0 > kWaitNs) {
      *abort_flag = 1;
      return false;
    }
  }
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag,
                                          bool ignore_abort = false) {
  if (mbar_try(bar, parity)) return true;
  return mbar_wait_slow(bar, parity, abort_flag, ignore_abort);
}

// 1-D bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned) from global
// into this CTA's shared memory, completion counted in bytes on `bar`.
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// 2-D TMA tile load into shared memory, completion counted in bytes on `bar`.
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Instruction descriptor: kind::f16, A = B = BF16, D = F32, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(
          tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
// One 128 x N x (16 * ksteps) product; A is a 128-row tile and B an N-row tile, both
// stored as two 64-column swizzled halves (A half = 16 KB, B half = N * 128 B).  Rows are
// zero beyond the data dimension d, so ksteps = ceil(d / 16) gives the same FP32 sums as
// all eight steps (the skipped steps would add exact zeros).
template <int N>
__device__ __forceinline__ void umma_tile(uint32_t d_tmem, uint32_t a_base, uint32_t b_base, int ksteps) {
  constexpr uint32_t idesc = idesc_bf16(BM, N);
#pragma unroll
  for (int kk = 0; kk < KD / 16; ++kk) {
    if (kk < ksteps) {
      const uint32_t koff = (kk & 3) * 32;
      umma_bf16(d_tmem, smem_desc(a_base + (kk >> 2) * HALF_BYTES + koff),
                smem_desc(b_base + (kk >> 2) * (N * 128) + koff), idesc, kk > 0 ? 1u : 0u);
    }
  }
}
// K steps [k0, k1) of umma_tile: a tile's MMAs issued in pieces, each after its own part
// of the operands has landed.  Step 0 clears the accumulator.
template <int N>
__device__ __forceinline__ void umma_steps(uint32_t d_tmem, uint32_t a_base, uint32_t b_base, int k0, int k1) {
  constexpr uint32_t idesc = idesc_bf16(BM, N);
#pragma unroll
  for (int kk = 0; kk < KD / 16; ++kk) {
    if (kk >= k0 && kk < k1) {
      const uint32_t koff = (kk & 3) * 32;
      umma_bf16(d_tmem, smem_desc(a_base + (kk >> 2) * HALF_BYTES + koff),
                smem_desc(b_base + (kk >> 2) * (N * 128) + koff), idesc, kk > 0 ? 1u : 0u);
    }
  }
}
__host__ __device__ inline int tc_ksteps(int d) { return d <= 0 ? 1 : (d > KD ? KD / 16 : (d + 15) / 16); }

// FP8 operands: rows of KD E4M3 bytes (one 128-byte swizzle row holds the whole K).
// Instruction descriptor: kind::f8f6f4, A = B = E4M3 (format 0), D = F32, K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_e4m3(int M, int N) {
  return (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__device__ __forceinline__ void umma_e4m3(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}" ::"r"(
          tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
// One 128 x N x (32 * ksteps) E4M3 product: each step advances 32 bytes (K = 32) along the
// single 128-byte row of A (128-row tile) and B (N-row tile); as with BF16, rows are zero
// past d, so ksteps = ceil(d / 32) gives the same sums as all four steps.
template <int N>
__device__ __forceinline__ void umma_tile_e4m3(uint32_t d_tmem, uint32_t a_base, uint32_t b_base, int ksteps) {
  constexpr uint32_t idesc = idesc_e4m3(BM, N);
#pragma unroll
  for (int kk = 0; kk < KD / 32; ++kk) {
    if (kk < ksteps) {
      const uint32_t koff = kk * 32;
      umma_e4m3(d_tmem, smem_desc(a_base + koff), smem_desc(b_base + koff), idesc, kk > 0 ? 1u : 0u);
    }
  }
}
__host__ __device__ inline int tc_ksteps_e4m3(int d) { return d <= 0 ? 1 : (d > KD ? KD / 32 : (d + 31) / 32); }
// E4M3 codes hold unit vectors times this factor: every component (|v| <= 1) stays within
// the format's range (448) and components down to 2^-14 stay in its normal range.
constexpr float kE4M3Scale = 256.0f;
__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t slot_smem, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot_smem), "r"(cols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t tmem, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(cols) : "memory");
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 64 consecutive TMEM columns of this thread's lane (issue only; complete with tmem_wait_ld).
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, uint32_t (&r)[64]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,"
      "%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]),
        "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]),
        "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]),
        "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]),
        "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
      : "r"(taddr));
}

// Three-input maximum (sm_100+ max.f32 with three sources).
__device__ __forceinline__ float max3f(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// Maximum of the 8 consecutive scores v[8g .. 8g+7].
__device__ __forceinline__ float max8(const uint32_t (&v)[64], int g) {
  return max3f(max3f(__uint_as_float(v[8 * g]), __uint_as_float(v[8 * g + 1]), __uint_as_float(v[8 * g + 2])),
               max3f(__uint_as_float(v[8 * g + 3]), __uint_as_float(v[8 * g + 4]), __uint_as_float(v[8 * g + 5])),
               fmaxf(__uint_as_float(v[8 * g + 6]), __uint_as_float(v[8 * g + 7])));
}

// Tensor map over `rows` bf16 rows of KD elements; boxes of 64 columns x box_rows rows
// with 128-byte swizzle (the layout smem_desc describes).
CUtensorMap make_map(const void* base, int64_t rows, int box_rows = BM, int box_cols = KHALF);
// Rows of KD E4M3 bytes; boxes of box_rows rows x 128 bytes with 128-byte swizzle.
CUtensorMap make_map_e4m3(const void* base, int64_t rows, int box_rows);

}  // namespace tc
}  // namespace lshg
