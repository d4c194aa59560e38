// gemm_tc.cu -- batched sensitivity products on the 5th-generation tensor
// cores (tcgen05 + TMA + TMEM) with FP64-class accuracy from 16-bit inputs.
//
//   P[split][n][m] = sum_{k in split} (Ahi Bhi + Ahi Blo + Alo Bhi)[m][k][n]
//
// A [M][K] and B [N][K] are K-major fp16 (or bf16) hi / lo pairs, rows padded
// to a multiple of 64 elements.  Forward: A = J (rows x cells), B = models;
// adjoint: A = J^T (cells x rows), B = scaled residuals.
//
// Accuracy.  The tensor core's FP32 accumulation loses about 2e-8 relative
// per MMA step, growing linearly with the number of steps that feed one
// accumulator.  So every kStepsPerDrain 16-wide steps (32 cells) go to a
// fresh TMEM accumulator -- first the cross terms hi*lo + lo*hi (about 2^-11
// of the total), then the hi*hi products, so the large terms meet an
// accumulator of their own size -- and the drain warps add it, with
// round-to-nearest FP32 adds, into sums held in registers while the next
// steps are multiplied into the other accumulators (four in rotation).
// Splits of at most 128 k-blocks keep the register sums short; the caller
// adds the splits as FP32 two-sum pairs.
//
// One CTA computes a 128 x BN tile of one K split with 10 warps:
//   warp 0      TMA producer (Ahi, Alo, Bhi, Blo per stage, 128-byte swizzle)
//   warp 1      TMEM allocation; lane 0 issues the MMAs
//   warps 2-9   drain: warp w reads TMEM lanes 32*(w%4).. and columns
//               (w-2)/4 * BN/2 .. + BN/2, sums them per k-block, writes the tile
// Every mbarrier wait is bounded by a %globaltimer deadline; on expiry the
// CTA records an error code, stops issuing, drains what it issued (again
// bounded), frees its TMEM and returns.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <set>
#include <utility>

#include "stored.h"

namespace j3g {
namespace {

constexpr int BM = 128;
constexpr int BK = 64;  // 16-bit elements per 128-byte swizzled row
constexpr int kGemmThreads = 320;
constexpr int kDrainWarps = 8;
// hi*hi MMA steps (16 products each) per TMEM accumulator before it is
// drained into the register sums; 2 halves the tensor-core rounding of 4
constexpr int kStepsPerDrain = 2;
constexpr int kDrainsPerBlock = (BK / 16) / kStepsPerDrain;
constexpr int kAccBufs = 4;  // TMEM accumulators in rotation (4 x BN columns)
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s per wait
// With the test fault (GemmOperands::fault) the drain warps withhold their
// accumulator releases and the MMA issuer gives up on a release after this
// long; every other wait keeps kWaitNs, so that no copy or MMA is still in
// flight when the CTA tears down.  The failure path of the bounded waits is
// tested this way, with no GPU fault.
constexpr unsigned long long kTestWaitNs = 20000000ull;  // 20 ms

template <int BN, bool F16> struct Cfg {
  static constexpr int STAGES = BN == 128 ? 3 : 4;
  static constexpr int A_BYTES = BM * BK * 2;
  static constexpr int B_BYTES = BN * BK * 2;
  static constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
  static constexpr int NBAR = 2 * STAGES + 2 * kAccBufs;  // stage full / empty, buffer full / empty
  static constexpr int SMEM = STAGES * STAGE_BYTES + NBAR * 8 + 16 + 1024;
  static constexpr uint32_t TMEM_COLS = kAccBufs * BN;  // accumulator buffers, power of two
  // kind::f16 instruction descriptor: D F32 (bit 4), A and B format at bits
  // 7 and 10 (0 = F16, 1 = BF16), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
  static constexpr uint32_t FMT = F16 ? 0u : 1u;
  static constexpr uint32_t IDESC = (1u << 4) | (FMT << 7) | (FMT << 10) |
                                    ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
  static constexpr int COLS_PER_WARP = BN / 2;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: true when the phase completed, false after `limit_ns`.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity,
                                          unsigned long long limit_ns = kWaitNs) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = now_ns();
  while (true) {
    if (mbar_try(bar, parity)) return true;
    if (now_ns() - t0 > limit_ns) return false;
  }
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// One 128 x 64 tile of a matrix in the tiled layout (see tiled_index): a 3-D
// map {64 columns, 128 rows, tile}, box {64, 128, 1}.
__device__ __forceinline__ void tma_load_tile(uint32_t dst, const CUtensorMap *map, int tile,
                                              uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(0), "r"(tile), "r"(bar)
      : "memory");
}

// UMMA shared-memory descriptor of a K-major tile stored with the 128-byte
// swizzle (rows of 128 B, 8-row atoms 1024 B apart): start address >> 4 in
// bits 0-13, leading offset 16 B (unused for this layout) in bits 16-29,
// stride offset 1024 B in bits 32-45, the fixed 0b001 in bits 46-48, base
// offset 0 (atoms 1024-byte aligned), swizzle mode 2 (128 B) in bits 61-63.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                     uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 16 consecutive FP32 columns of this warp's 32 TMEM lanes (one per thread),
// without the wait: several loads are issued back to back and completed by
// one tmem_wait_ld over all their registers.
__device__ __forceinline__ void tmem_ld16_async(uint32_t taddr, uint32_t *v) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15])
      : "r"(taddr));
}

// s0 += a0 and s1 += a1 as one paired FP32 instruction (add.rn.f32x2,
// sm_100 and later): two round-to-nearest IEEE adds in half the issue slots.
__device__ __forceinline__ void fadd2_rn(float &s0, float &s1, uint32_t a0, uint32_t a1) {
  asm("{\n .reg .b64 x, y;\n mov.b64 x, {%0, %1};\n mov.b64 y, {%2, %3};\n"
      " add.rn.f32x2 x, x, y;\n mov.b64 {%0, %1}, x;\n}"
      : "+f"(s0), "+f"(s1)
      : "r"(a0), "r"(a1));
}

// Register dependence on 16 loaded values: uses of v stay after this point.
__device__ __forceinline__ void reg_fence16(uint32_t *v) {
  asm volatile(""
               : "+r"(v[0]), "+r"(v[1]), "+r"(v[2]), "+r"(v[3]), "+r"(v[4]), "+r"(v[5]),
                 "+r"(v[6]), "+r"(v[7]), "+r"(v[8]), "+r"(v[9]), "+r"(v[10]), "+r"(v[11]),
                 "+r"(v[12]), "+r"(v[13]), "+r"(v[14]), "+r"(v[15])
               :
               : "memory");
}

// Completes every tcgen05.ld this thread issued; the register fences after it
// keep the uses of the NV x 16 loaded values behind the wait.
template <int NV>
__device__ __forceinline__ void tmem_wait_ld(uint32_t (&v)[NV][16]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < NV; ++i) reg_fence16(v[i]);
}


template <int BN, bool F16>
__global__ void __launch_bounds__(kGemmThreads, 1)
    k_gemm_x3(const __grid_constant__ CUtensorMap tmAhi, const __grid_constant__ CUtensorMap tmAlo,
              const __grid_constant__ CUtensorMap tmBhi, const __grid_constant__ CUtensorMap tmBlo,
              int kb_per_split, int kb_total, int M, int N, int ntn, float *__restrict__ P,
              long long ldp, long long slice, int *__restrict__ err, int fault) {
  using C = Cfg<BN, F16>;
  constexpr int S = C::STAGES;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                              ~static_cast<uintptr_t>(1023));
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + S * C::STAGE_BYTES);
  uint64_t *full = bars, *empty = bars + S;
  uint64_t *a_full = bars + 2 * S, *a_empty = bars + 2 * S + kAccBufs;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + C::NBAR);
  volatile int *fail = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // x runs over (M tile, N tile) with the ntn N tiles fastest (see launch_bn)
  const int n0 = (int)(blockIdx.x % ntn) * BN, m0 = (int)(blockIdx.x / ntn) * BM;
  const int kb0 = blockIdx.z * kb_per_split;
  const int nkb = min(kb_total, kb0 + kb_per_split) - kb0;
  const int ndrain = nkb * kDrainsPerBlock;

  if (threadIdx.x == 0) {
    for (int s = 0; s < 2 * S; ++s) mbar_init(smem_u32(bars + s), 1);
    for (int b = 0; b < kAccBufs; ++b) {
      mbar_init(smem_u32(a_full + b), 1);
      mbar_init(smem_u32(a_empty + b), kDrainWarps);
    }
    *fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmAhi)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmAlo)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmBhi)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmBlo)) : "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(C::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int issued = 0;
      for (int i = 0; i < nkb; ++i) {
        const int s = i % S;
        const uint32_t ph = (uint32_t)(i / S) & 1u;
        if (i >= S && !mbar_wait(smem_u32(empty + s), ph ^ 1u)) {
          atomicExch(err, 1);
          *fail = 1;
          break;
        }
        if (*fail) break;
        uint8_t *st = smem + s * C::STAGE_BYTES;
        const uint32_t fb = smem_u32(full + s);
        mbar_expect_tx(fb, (uint32_t)C::STAGE_BYTES);
        const int kx = (kb0 + i) * BK;
        const int at = (m0 / BM) * kb_total + kb0 + i;  // A tile (tiled layout)
        tma_load_tile(smem_u32(st), &tmAhi, at, fb);
        tma_load_tile(smem_u32(st + C::A_BYTES), &tmAlo, at, fb);
        tma_load_2d(smem_u32(st + 2 * C::A_BYTES), &tmBhi, kx, n0, fb);
        tma_load_2d(smem_u32(st + 2 * C::A_BYTES + C::B_BYTES), &tmBlo, kx, n0, fb);
        issued = i + 1;
      }
      // the last stages may still be landing; let them complete (bounded)
      for (int i = (issued > S ? issued - S : 0); i < issued; ++i)
        mbar_wait(smem_u32(full + (i % S)), (uint32_t)(i / S) & 1u);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    // Drain d covers kStepsPerDrain 16-wide steps of one k-block and goes to
    // accumulator buffer d % kAccBufs: first the small cross terms (the
    // buffer starts from zero), then the hi*hi products, so that the large
    // terms are added last to an accumulator of their own size.
    if (lane == 0) {
      bool ok = true;
      for (int i = 0; i < nkb && ok; ++i) {
        const int s = i % S;
        if (!mbar_wait(smem_u32(full + s), (uint32_t)(i / S) & 1u)) {
          atomicExch(err, 2);
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t base = smem_u32(smem + s * C::STAGE_BYTES);
        const uint32_t ahi = base, alo = base + C::A_BYTES;
        const uint32_t bhi = base + 2 * C::A_BYTES, blo = bhi + C::B_BYTES;
#pragma unroll
        for (int j = 0; j < kDrainsPerBlock; ++j) {
          const int d = i * kDrainsPerBlock + j;
          const int b = d % kAccBufs;
          if (d >= kAccBufs &&
              !mbar_wait(smem_u32(a_empty + b), ((uint32_t)(d / kAccBufs) & 1u) ^ 1u,
                         fault ? kTestWaitNs : kWaitNs)) {
            // the buffer of drain d - kAccBufs was never emptied
            atomicExch(err, 3);
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t acc = tmem + (uint32_t)(b * BN);
#pragma unroll
          for (int t = 0; t < kStepsPerDrain; ++t) {
            const uint32_t off = (j * kStepsPerDrain + t) * 32;  // 16 elements = 32 bytes
            umma(acc, sw128_desc(ahi + off), sw128_desc(blo + off), C::IDESC, t > 0 ? 1u : 0u);
            umma(acc, sw128_desc(alo + off), sw128_desc(bhi + off), C::IDESC, 1u);
          }
#pragma unroll
          for (int t = 0; t < kStepsPerDrain; ++t) {
            const uint32_t off = (j * kStepsPerDrain + t) * 32;
            umma(acc, sw128_desc(ahi + off), sw128_desc(bhi + off), C::IDESC, 1u);
          }
          umma_commit(smem_u32(a_full + b));  // this drain's products are ready
        }
        if (!ok) break;
        umma_commit(smem_u32(empty + s));  // smem stage free once these MMAs finish
      }
      if (!ok) *fail = 1;
    }
  } else {
    // ---------------- drain warps ----------------
    const int q = warp & 3;                                   // TMEM lane quarter
    const int ch = (warp - 2) >> 2;                           // column half
    const uint32_t lane_off = (uint32_t)(q * 32) << 16;
    const uint32_t col0 = (uint32_t)(ch * C::COLS_PER_WARP);
    float s[C::COLS_PER_WARP];  // round-to-nearest FP32 sums of the drained accumulators
#pragma unroll
    for (int j = 0; j < C::COLS_PER_WARP; ++j) s[j] = 0.0f;
    for (int d = 0; d < ndrain; ++d) {
      const int b = d % kAccBufs;
      bool got = mbar_wait(smem_u32(a_full + b), (uint32_t)(d / kAccBufs) & 1u);
      got = __all_sync(0xffffffffu, got ? 1 : 0) != 0;
      if (!got) {
        if (lane == 0) atomicExch(err, 4);
        break;
      }
      tc_fence_after();
      const uint32_t acc = tmem + (uint32_t)(b * BN) + lane_off + col0;
      // all loads of the drain in flight together, one wait
      constexpr int NV = C::COLS_PER_WARP / 16;
      uint32_t v[NV][16];
#pragma unroll
      for (int h = 0; h < NV; ++h) tmem_ld16_async(acc + 16u * h, v[h]);
      tmem_wait_ld(v);
#pragma unroll
      for (int h = 0; h < NV; ++h) {
#pragma unroll
        for (int j = 0; j < 16; j += 2)
          fadd2_rn(s[16 * h + j], s[16 * h + j + 1], v[h][j], v[h][j + 1]);
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0 && !fault) mbar_arrive(smem_u32(a_empty + b));
    }
    const int row = m0 + q * 32 + lane;
    float *out = P + (long long)blockIdx.z * slice;
    if (row < M) {
#pragma unroll
      for (int j = 0; j < C::COLS_PER_WARP; ++j) {
        const int n = n0 + (int)col0 + j;
        if (n < N) out[(long long)n * ldp + row] = s[j];
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(C::TMEM_COLS)
                 : "memory");
  }
}

// ---------------------------------------------------------------------------
// CTA-pair kernel for N tiles of 256 (cta_group::2).  A cluster of two CTAs on
// two SMs computes a 256 x 256 tile: each CTA stages its own 128 rows of A and
// its own 128 rows (models) of B; the even CTA issues 256 x 256 x 16 MMAs that
// read both CTAs' shared memory and write each CTA's 128 x 256 accumulator
// into that CTA's TMEM.  Per instruction this is four times the work of the
// 128 x 128 form, whose issue cost otherwise caps the tensor pipe near half
// rate, and each SM loads half of B.
//
// Barriers (same offsets in both CTAs):
//   full[s]    even CTA only: both CTAs' TMA bytes of stage s (the odd CTA's
//              copies signal it through the pair form of the TMA load)
//   empty[s]   both CTAs: stage s free (MMA commit, multicast to the pair)
//   a_full[b]  both CTAs: accumulator b ready (MMA commit, multicast)
//   a_empty[b] even CTA only: accumulator b drained in both CTAs (one relaxed
//              arrival per drain warp of either CTA)
//   done       even CTA only: every issued MMA finished
// Waits are bounded as in k_gemm_x3; on expiry a CTA records an error code,
// stops issuing and runs on to the closing cluster barrier, which both CTAs
// always reach before the TMEM is freed.
constexpr int kPairN = 256;   // N of the tile (and of each MMA)
// Drain warps: four per TMEM lane quarter, each summing 64 of the 256
// accumulator columns (64 FP32 sums and one 16-column load in flight fit the
// 112 registers a thread gets at 576 threads).
constexpr int kPairDrainWarps = 16;
constexpr int kPairThreads = 64 + 32 * kPairDrainWarps;  // TMA warp, MMA warp, drain warps
constexpr int kPairAcc = 2;   // accumulators of 256 columns: all 512 TMEM columns
constexpr int kPairLoads = 1; // TMEM loads (16 columns each) in flight per wait

template <bool F16> struct PairCfg {
  static constexpr int STAGES = 3;
  static constexpr int A_BYTES = BM * BK * 2;          // this CTA's 128 rows of A
  static constexpr int B_BYTES = (kPairN / 2) * BK * 2;  // this CTA's 128 rows of B
  static constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;
  static constexpr int NBAR = 2 * STAGES + 2 * kPairAcc + 1;
  static constexpr int SMEM = STAGES * STAGE_BYTES + NBAR * 8 + 16 + 1024;
  static constexpr uint32_t TMEM_COLS = kPairAcc * kPairN;
  static constexpr uint32_t FMT = F16 ? 0u : 1u;
  // M = 256 across the pair, N = 256
  static constexpr uint32_t IDESC = (1u << 4) | (FMT << 7) | (FMT << 10) |
                                    ((uint32_t)(kPairN >> 3) << 17) | ((uint32_t)(256 >> 4) << 24);
  static constexpr int COLS_PER_WARP = kPairN / (kPairDrainWarps / 4);
};

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// Address of the same shared-memory object in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t peer_addr(uint32_t local, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
  return r;
}

__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::
                   : "memory");
}

// Arrive on a barrier of another CTA of the cluster.  Relaxed: a release at
// cluster scope would wait for this SM's outstanding memory traffic (the TMA
// stream) on every drain; the TMEM reads it signals are already complete
// (tcgen05.wait::ld) when it issues.
__device__ __forceinline__ void mbar_arrive_remote(uint32_t cluster_bar) {
  asm volatile("mbarrier.arrive.relaxed.cluster.shared::cluster.b64 _, [%0];" ::"r"(cluster_bar)
               : "memory");
}


// TMA load into this CTA's shared memory that signals an mbarrier of either
// CTA of the pair (cluster address).
__device__ __forceinline__ void tma_load_2d_pair(uint32_t dst, const CUtensorMap *map, int x,
                                                 int y, uint32_t cluster_bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(cluster_bar)
      : "memory");
}

__device__ __forceinline__ void tma_load_tile_pair(uint32_t dst, const CUtensorMap *map, int tile,
                                                   uint32_t cluster_bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(0), "r"(tile), "r"(cluster_bar)
      : "memory");
}

__device__ __forceinline__ void umma_pair(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive on the barrier at this offset in both CTAs once the issued MMAs finish.
__device__ __forceinline__ void umma_commit_pair(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64"
      " [%0], %1;" ::"r"(bar),
      "h"((uint16_t)3)
      : "memory");
}

// The same on this CTA's barrier only.
__device__ __forceinline__ void umma_commit_pair_local(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   bar)
               : "memory");
}

template <bool F16>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kPairThreads, 1)
    k_gemm_pair(const __grid_constant__ CUtensorMap tmAhi,
                const __grid_constant__ CUtensorMap tmAlo,
                const __grid_constant__ CUtensorMap tmBhi,
                const __grid_constant__ CUtensorMap tmBlo, int kb_per_split, int kb_total, int M,
                int N, float *__restrict__ P, long long ldp, long long slice,
                int *__restrict__ err, int fault) {
  using C = PairCfg<F16>;
  constexpr int S = C::STAGES;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                              ~static_cast<uintptr_t>(1023));
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem + S * C::STAGE_BYTES);
  uint64_t *full = bars, *empty = bars + S;
  uint64_t *a_full = bars + 2 * S, *a_empty = bars + 2 * S + kPairAcc;
  uint64_t *done = bars + 2 * S + 2 * kPairAcc;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + C::NBAR);
  volatile int *fail = reinterpret_cast<volatile int *>(tmem_slot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = cluster_rank();            // 0: issues the MMAs
  const int m0 = (blockIdx.x >> 1) * 256 + (int)rank * BM;  // this CTA's rows of A and P
  const int n0 = blockIdx.y * kPairN;                       // the pair's models
  const int nb0 = n0 + (int)rank * (kPairN / 2);            // this CTA's rows of B
  const int kb0 = blockIdx.z * kb_per_split;
  const int nkb = min(kb_total, kb0 + kb_per_split) - kb0;
  const int ndrain = nkb * kDrainsPerBlock;

  if (threadIdx.x == 0) {
    for (int s = 0; s < 2 * S; ++s) mbar_init(smem_u32(bars + s), 1);
    for (int b = 0; b < kPairAcc; ++b) {
      mbar_init(smem_u32(a_full + b), 1);
      mbar_init(smem_u32(a_empty + b), 2 * kPairDrainWarps);  // one per drain warp of the pair
    }
    mbar_init(smem_u32(done), 1);
    *fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmAhi)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmAlo)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmBhi)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmBlo)) : "memory");
  }
  if (warp == 1) {  // one warp of each CTA allocates the pair's TMEM together
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(C::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  cluster_sync_all();  // both CTAs' barriers initialised before any cross-CTA signal
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---------------- TMA producer (both CTAs) ----------------
    if (lane == 0) {
      int issued = 0;
      for (int i = 0; i < nkb; ++i) {
        const int s = i % S;
        const uint32_t ph = (uint32_t)(i / S) & 1u;
        // no early exit on this CTA's fail flag: both producers stop at the
        // same k-block (the empty commits reach both CTAs), so the even CTA's
        // wait below covers every copy the odd CTA issued
        if (i >= S && !mbar_wait(smem_u32(empty + s), ph ^ 1u)) {
          atomicExch(err, 1);
          *fail = 1;
          break;
        }
        uint8_t *st = smem + s * C::STAGE_BYTES;
        const uint32_t fb_local = smem_u32(full + s);
        if (rank == 0) mbar_expect_tx(fb_local, 2u * (uint32_t)C::STAGE_BYTES);
        const uint32_t fb = peer_addr(fb_local, 0);
        const int kx = (kb0 + i) * BK;
        const int at = (m0 / BM) * kb_total + kb0 + i;  // A tile (tiled layout)
        tma_load_tile_pair(smem_u32(st), &tmAhi, at, fb);
        tma_load_tile_pair(smem_u32(st + C::A_BYTES), &tmAlo, at, fb);
        tma_load_2d_pair(smem_u32(st + 2 * C::A_BYTES), &tmBhi, kx, nb0, fb);
        tma_load_2d_pair(smem_u32(st + 2 * C::A_BYTES + C::B_BYTES), &tmBlo, kx, nb0, fb);
        issued = i + 1;
      }
      // the even CTA's full barriers count both CTAs' copies: let the last
      // stages land (bounded) before the closing cluster barrier
      if (rank == 0)
        for (int i = (issued > S ? issued - S : 0); i < issued; ++i)
          mbar_wait(smem_u32(full + (i % S)), (uint32_t)(i / S) & 1u);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer (even CTA) ----------------
    if (lane == 0 && rank == 0) {
      bool ok = true;
      int issued = 0;
      for (int i = 0; i < nkb && ok; ++i) {
        const int s = i % S;
        if (!mbar_wait(smem_u32(full + s), (uint32_t)(i / S) & 1u)) {
          atomicExch(err, 2);
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t base = smem_u32(smem + s * C::STAGE_BYTES);
        const uint32_t ahi = base, alo = base + C::A_BYTES;
        const uint32_t bhi = base + 2 * C::A_BYTES, blo = bhi + C::B_BYTES;
#pragma unroll
        for (int j = 0; j < kDrainsPerBlock; ++j) {
          const int d = i * kDrainsPerBlock + j;
          const int b = d % kPairAcc;
          if (d >= kPairAcc &&
              !mbar_wait(smem_u32(a_empty + b), ((uint32_t)(d / kPairAcc) & 1u) ^ 1u,
                         fault ? kTestWaitNs : kWaitNs)) {
            atomicExch(err, 3);
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t acc = tmem + (uint32_t)(b * kPairN);
#pragma unroll
          for (int t = 0; t < kStepsPerDrain; ++t) {
            const uint32_t off = (j * kStepsPerDrain + t) * 32;
            umma_pair(acc, sw128_desc(ahi + off), sw128_desc(blo + off), C::IDESC,
                      t > 0 ? 1u : 0u);
            umma_pair(acc, sw128_desc(alo + off), sw128_desc(bhi + off), C::IDESC, 1u);
          }
#pragma unroll
          for (int t = 0; t < kStepsPerDrain; ++t) {
            const uint32_t off = (j * kStepsPerDrain + t) * 32;
            umma_pair(acc, sw128_desc(ahi + off), sw128_desc(bhi + off), C::IDESC, 1u);
          }
          umma_commit_pair(smem_u32(a_full + b));
        }
        if (!ok) break;
        issued = i + 1;
        // stage s is reloaded only for k-block i + S
        if (i + S < nkb) umma_commit_pair(smem_u32(empty + s));
      }
      if (!ok) *fail = 1;
      (void)issued;
      // every MMA issued so far has finished before the pair tears down
      umma_commit_pair_local(smem_u32(done));
      if (!mbar_wait(smem_u32(done), 0u)) atomicExch(err, 5);
    }
  } else {
    // ---------------- drain warps (both CTAs) ----------------
    const int q = warp & 3;          // TMEM lane quarter
    const int ch = (warp - 2) >> 2;  // column group of COLS_PER_WARP
    const uint32_t lane_off = (uint32_t)(q * 32) << 16;
    const uint32_t col0 = (uint32_t)(ch * C::COLS_PER_WARP);
    float s[C::COLS_PER_WARP];
#pragma unroll
    for (int j = 0; j < C::COLS_PER_WARP; ++j) s[j] = 0.0f;
    for (int d = 0; d < ndrain; ++d) {
      const int b = d % kPairAcc;
      // the lanes decide together: tcgen05.ld below is warp-collective
      const bool got =
          __all_sync(0xffffffffu, mbar_wait(smem_u32(a_full + b), (uint32_t)(d / kPairAcc) & 1u));
      if (!got) {
        if (lane == 0) atomicExch(err, 4);
        break;
      }
      tc_fence_after();
      const uint32_t acc = tmem + (uint32_t)(b * kPairN) + lane_off + col0;
#pragma unroll
      for (int h0 = 0; h0 < C::COLS_PER_WARP / 16; h0 += kPairLoads) {
        uint32_t v[kPairLoads][16];
#pragma unroll
        for (int h = 0; h < kPairLoads; ++h) tmem_ld16_async(acc + 16u * (h0 + h), v[h]);
        tmem_wait_ld(v);
#pragma unroll
        for (int h = 0; h < kPairLoads; ++h) {
#pragma unroll
          for (int j = 0; j < 16; j += 2)
            fadd2_rn(s[16 * (h0 + h) + j], s[16 * (h0 + h) + j + 1], v[h][j], v[h][j + 1]);
        }
      }
      tc_fence_before();
      __syncwarp();
      // accumulator b is reused by drain d + kPairAcc: one relaxed arrival per
      // drain warp once its loads are complete (no named barrier per drain)
      if (lane == 0 && d + kPairAcc < ndrain && !fault) {
        if (rank == 0)
          mbar_arrive(smem_u32(a_empty + b));
        else
          mbar_arrive_remote(peer_addr(smem_u32(a_empty + b), 0));
      }
    }
    const int row = m0 + q * 32 + lane;
    float *out = P + (long long)blockIdx.z * slice;
    if (row < M) {
#pragma unroll
      for (int j = 0; j < C::COLS_PER_WARP; ++j) {
        const int n = n0 + (int)col0 + j;
        if (n < N) out[(long long)n * ldp + row] = s[j];
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  cluster_sync_all();  // neither CTA frees TMEM or exits while the pair still works
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(C::TMEM_COLS)
                 : "memory");
  }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

// 2-D K-major 16-bit map: rows x ld elements (ld multiple of 64), box BK x box_rows.
bool make_map(CUtensorMap *map, const void *base, long long rows, long long ld, int box_rows,
              bool f16) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)ld, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  return fn(map, f16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
            const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// 3-D map of an operand in the tiled layout: rows (padded to 128) x ld.
bool make_tiled_map(CUtensorMap *map, const void *base, long long rows, long long ld, bool f16) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  const long long tiles = tiled_rows(rows) / BM * (ld / BK);
  cuuint64_t dims[3] = {(cuuint64_t)BK, (cuuint64_t)BM, (cuuint64_t)tiles};
  cuuint64_t strides[2] = {(cuuint64_t)BK * 2, (cuuint64_t)BK * BM * 2};
  cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)BM, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  return fn(map, f16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3,
            const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Dynamic shared-memory opt-in of a kernel, once per kernel and device: the
// launchers stay free of non-stream CUDA calls after the first launch, so a
// caller can capture later launches in a CUDA graph.
cudaError_t allow_smem_once(const void *kernel, int bytes) {
  static std::mutex mu;
  static std::set<std::pair<const void *, int>> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  if (done.count({kernel, dev})) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) done.insert({kernel, dev});
  return e;
}

template <int BN, bool F16>
cudaError_t launch_bn(const GemmOperands &g, int nsplit, float *P, long long ldp, long long slice,
                      int *err, cudaStream_t st) {
  CUtensorMap ah, al, bh, bl;
  if (!make_tiled_map(&ah, g.a_hi, g.m, g.ld, F16) || !make_tiled_map(&al, g.a_lo, g.m, g.ld, F16) ||
      !make_map(&bh, g.b_hi, g.n_pad, g.ld, BN, F16) ||
      !make_map(&bl, g.b_lo, g.n_pad, g.ld, BN, F16))
    return cudaErrorInvalidValue;
  const int kb_total = (int)(g.ld / BK);
  const int kb_per = (kb_total + nsplit - 1) / nsplit;
  const int nsp = (kb_total + kb_per - 1) / kb_per;
  cudaError_t e = allow_smem_once(reinterpret_cast<const void *>(k_gemm_x3<BN, F16>),
                                  Cfg<BN, F16>::SMEM);
  if (e != cudaSuccess) return e;
  // N tiles vary fastest so the CTAs sharing an A tile run side by side (L2
  // reuse); M and N tiles share grid x, whose limit (2^31 - 1) no mesh reaches
  const int ntn = (int)(g.n_pad / BN);
  const long long nmt = (g.m + BM - 1) / BM;
  dim3 grid((unsigned)(nmt * ntn), 1u, (unsigned)nsp);
  k_gemm_x3<BN, F16><<<grid, kGemmThreads, Cfg<BN, F16>::SMEM, st>>>(
      ah, al, bh, bl, kb_per, kb_total, (int)g.m, (int)g.n, ntn, P, ldp, slice, err, g.fault);
  return cudaGetLastError();
}

template <bool F16>
cudaError_t launch_pair(const GemmOperands &g, int nsplit, float *P, long long ldp,
                        long long slice, int *err, cudaStream_t st) {
  CUtensorMap ah, al, bh, bl;
  if (!make_tiled_map(&ah, g.a_hi, g.m, g.ld, F16) || !make_tiled_map(&al, g.a_lo, g.m, g.ld, F16) ||
      !make_map(&bh, g.b_hi, g.n_pad, g.ld, kPairN / 2, F16) ||
      !make_map(&bl, g.b_lo, g.n_pad, g.ld, kPairN / 2, F16))
    return cudaErrorInvalidValue;
  const int kb_total = (int)(g.ld / BK);
  const int kb_per = (kb_total + nsplit - 1) / nsplit;
  const int nsp = (kb_total + kb_per - 1) / kb_per;
  cudaError_t e = allow_smem_once(reinterpret_cast<const void *>(k_gemm_pair<F16>),
                                  PairCfg<F16>::SMEM);
  if (e != cudaSuccess) return e;
  // x: CTA pairs over M (two CTAs of 128 rows each), y: N tiles of 256, z: K splits
  dim3 grid((unsigned)(2 * ((g.m + 255) / 256)), (unsigned)(g.n_pad / kPairN), (unsigned)nsp);
  k_gemm_pair<F16><<<grid, kPairThreads, PairCfg<F16>::SMEM, st>>>(
      ah, al, bh, bl, kb_per, kb_total, (int)g.m, (int)g.n, P, ldp, slice, err, g.fault);
  return cudaGetLastError();
}

}  // namespace

// N tile of the batched products: 64 or 128 on one SM, 256 on a CTA pair.
int gemm_n_tile(int n) { return n <= 64 ? 64 : (n <= 128 ? 128 : kPairN); }

int gemm_kb_per_split(long long ld, int nsplit) {
  const int kb_total = (int)(ld / BK);
  return (kb_total + nsplit - 1) / nsplit;
}

int gemm_splits_used(long long ld, int nsplit) {
  const int kb_total = (int)(ld / BK);
  const int kb_per = (kb_total + nsplit - 1) / nsplit;
  return (kb_total + kb_per - 1) / kb_per;
}

cudaError_t launch_gemm_x3(const GemmOperands &g, int nsplit, float *P, long long ldp,
                           long long slice, int *err, cudaStream_t st, int tile) {
  const int nt = tile ? tile : gemm_n_tile((int)g.n);
  if (nt != 64 && nt != 128 && nt != kPairN) return cudaErrorInvalidValue;
  if (g.ld % BK != 0 || g.n_pad % nt != 0 || nsplit < 1) return cudaErrorInvalidValue;
  if ((reinterpret_cast<uintptr_t>(g.a_hi) | reinterpret_cast<uintptr_t>(g.a_lo) |
       reinterpret_cast<uintptr_t>(g.b_hi) | reinterpret_cast<uintptr_t>(g.b_lo)) & 15)
    return cudaErrorMisalignedAddress;
  if (g.f16) {
    if (nt == kPairN) return launch_pair<true>(g, nsplit, P, ldp, slice, err, st);
    if (nt == 64) return launch_bn<64, true>(g, nsplit, P, ldp, slice, err, st);
    return launch_bn<128, true>(g, nsplit, P, ldp, slice, err, st);
  }
  if (nt == kPairN) return launch_pair<false>(g, nsplit, P, ldp, slice, err, st);
  if (nt == 64) return launch_bn<64, false>(g, nsplit, P, ldp, slice, err, st);
  return launch_bn<128, false>(g, nsplit, P, ldp, slice, err, st);
}

}  // namespace j3g
