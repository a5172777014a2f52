// The 3x3x3, 32 -> 32 channel convolutions of the learned preconditioner on
// the 5th-generation tensor cores: TMA tensor loads, tcgen05.mma (kind::f16,
// BF16 operands, FP32 accumulators in tensor memory), warp-specialised.
// Forward and backward-data use it (backward-data on the flipped,
// transposed weights).
//
// Implicit GEMM per tile of 128 consecutive positions p (channels-last
// activations act[p][c], p = x + N (y + N z), N a power of two >= 8):
//   out[p][co] = sum_t sum_ci A_t[p][ci] W[t][co][ci],  A_t[p] = in[p shifted by tap t]
// M = 128 positions, N = 32 output channels, K = 32 channels per tap, 27 taps.
//  - A_t is one TMA load of a 4-D box {32 channels, BX, BY, BZ} of the
//    activation tensor [z][y][x][c] at the tile's corner shifted by the tap:
//    the 128 rows of the box are the tile's positions in order, and the
//    zero fill of the tensor map outside the grid is the convolution's
//    zero padding.  The box lands in the 64-byte-swizzled K-major layout
//    (rows of 64 bytes).  A pipeline stage holds the nine (x, y) shifts of
//    one z shift (nine boxes, 72 KB): one barrier round trip and one commit
//    per nine taps, two stages.
//  - The weights (B, 32 x 27*32) are written once per CTA into shared memory
//    in the 128-byte-swizzled K-major layout (56 KB).
//  - Warp 4 (one lane) issues the TMA loads, warp 5 (one lane) the MMAs
//    (two K = 16 instructions per tap, six per stage) and their commits,
//    warps 0-3 read the
//    accumulator back (warp w owns TMEM lanes 32w..32w+31 = its rows),
//    rectify (forward), round to BF16 and store 64 contiguous bytes per
//    position.  Full / empty mbarriers between loads and MMAs, two
//    accumulators in TMEM between MMAs and the epilogue, so loads, MMAs and
//    stores of consecutive tiles overlap.  Persistent CTAs, one per SM.
// Every mbarrier wait is bounded; on a timeout the kernel records it in the
// status word, waits (bounded) for its copies and MMAs in flight, frees its
// tensor memory and returns.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace gbfem {
namespace cnn {

constexpr int kCtThreads = 192;
constexpr int kCtM = 128, kCtN = 32, kCtTaps = 27;
constexpr int kCtTapBytes = kCtM * 64;           // 8 KB: 128 rows of 32 BF16
// A stage holds the nine (x, y) shifts of one z shift.  Measured at 64^3 Q3
// (forward pass): one tap per stage (16 stages) 0.568 ms, three (6 stages)
// 0.463 ms, nine (2 stages) 0.438 ms: the cost is the barrier round trip
// and commit per stage, not the loads.
constexpr int kCtTapsPerStage = 9;
constexpr int kCtStepsPerTile = kCtTaps / kCtTapsPerStage;
constexpr int kCtStages = 2;
constexpr uint32_t kCtBBytes = 14 * kCtN * 128;  // 56 KB: 14 atoms of 64 BF16 (taps 2a, 2a+1)
constexpr uint32_t kCtStageBytes = kCtTapsPerStage * kCtTapBytes;  // 24 KB
constexpr size_t kCtSmem = size_t(kCtBBytes) + kCtStages * size_t(kCtStageBytes) + 1024;
constexpr uint32_t kCtWaitLimit = 1u << 24;
constexpr uint32_t kCtCols = 64;  // two 32-column FP32 accumulators
// kind::f16, FP32 accumulator, A and B BF16, both K-major, N = 32, M = 128
constexpr uint32_t kCtIdesc = (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(kCtN >> 3) << 17) |
                              (uint32_t(kCtM >> 4) << 24);

__device__ __forceinline__ uint32_t ct_smem(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// byte offset of BF16 element (row, k) of the B operand (32 rows, K-major,
// 128-byte swizzle: atoms of 64 elements, 8-row groups of 1 KB)
__device__ __forceinline__ uint32_t ct_swz128(int row, int k) {
  const uint32_t off = uint32_t(k >> 6) * uint32_t(kCtN) * 128u + uint32_t(row >> 3) * 1024u +
                       uint32_t(row & 7) * 128u + uint32_t(k & 63) * 2u;
  return off ^ (((off >> 7) & 7u) << 4);
}

// shared-memory matrix descriptor, K-major: swizzle 2 = 128 B (8-row groups
// of 1024 bytes), 4 = 64 B (8-row groups of 512 bytes)
__device__ __forceinline__ uint64_t ct_desc(uint32_t saddr, uint32_t swizzle, uint32_t group_bytes) {
  uint64_t d = uint64_t((saddr & 0x3FFFFu) >> 4);
  d |= uint64_t(1) << 16;
  d |= uint64_t(group_bytes >> 4) << 32;
  d |= uint64_t(1) << 46;
  d |= uint64_t(swizzle) << 61;
  return d;
}

__device__ __forceinline__ bool ct_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t it = 0; it < kCtWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(ct_smem(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

template <bool RELU>
__global__ void __launch_bounds__(kCtThreads, 1)
    conv_tma_kernel(const __grid_constant__ CUtensorMap map, const __nv_bfloat16* __restrict__ wt,
                    __nv_bfloat16* __restrict__ out, int N, int* __restrict__ status) {
  extern __shared__ unsigned char ct_raw[];
  __shared__ __align__(8) uint64_t full[kCtStages], empty[kCtStages], acc_full[2], acc_empty[2];
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  const long long P = (long long)N * N * N;
  const long long ntiles = P / kCtM;
  if ((long long)blockIdx.x >= ntiles) return;  // uniform over the CTA
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  unsigned char* base = ct_raw + ((1024u - (ct_smem(ct_raw) & 1023u)) & 1023u);
  unsigned char* sB = base;
  unsigned char* sA = base + kCtBBytes;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(ct_smem(&tmem_base)),
                 "r"(kCtCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int s = 0; s < kCtStages; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(ct_smem(&full[s])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(ct_smem(&empty[s])) : "memory");
    }
    for (int b = 0; b < 2; ++b) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(ct_smem(&acc_full[b])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;" ::"r"(ct_smem(&acc_empty[b])) : "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
  }
  // weights: B[co][32 t + ci] = wt[t][co][ci] (tap 27 of the last atom is zero)
  for (int idx = tid; idx < 28 * kCtN * 4; idx += kCtThreads) {
    const int t = idx >> 7, co = (idx >> 2) & 31, c8 = idx & 3;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (t < kCtTaps) v = __ldg(reinterpret_cast<const uint4*>(wt + (t * kCtN + co) * 32 + c8 * 8));
    *reinterpret_cast<uint4*>(sB + ct_swz128(co, t * 32 + c8 * 8)) = v;
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (warp == 4) {
    // ---- TMA producer --------------------------------------------------------
    if (lane == 0) {
      asm volatile("prefetch.tensormap [%0];" ::"l"(&map) : "memory");
      uint32_t g = 0;
      bool ok = true;
      for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
        const long long p0 = tile * kCtM;
        const int x0 = int(p0 % N), y0 = int((p0 / N) % N), z0 = int(p0 / ((long long)N * N));
        for (int j = 0; j < kCtStepsPerTile; ++j, ++g) {
          const uint32_t s = g % kCtStages;
          if (g >= kCtStages && !ct_wait(&empty[s], ((g / kCtStages) - 1) & 1u)) {
            ok = false;
            break;
          }
          if (abort_flag) {
            ok = false;
            break;
          }
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(ct_smem(&full[s])),
                       "r"(kCtStageBytes)
                       : "memory");
          // tap t = kCtTapsPerStage j + k: shifts t % 3 - 1, (t / 3) % 3 - 1, t / 9 - 1
#pragma unroll
          for (int k = 0; k < kCtTapsPerStage; ++k) {
            const int t = kCtTapsPerStage * j + k;
            asm volatile(
                "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
                "%5}], [%6];" ::"r"(ct_smem(sA + s * kCtStageBytes + k * kCtTapBytes)),
                "l"(&map), "r"(0), "r"(x0 + t % 3 - 1), "r"(y0 + (t / 3) % 3 - 1), "r"(z0 + t / 9 - 1),
                "r"(ct_smem(&full[s]))
                : "memory");
          }
        }
      }
      if (!ok) abort_flag = 1;
      // the loads issued last have landed (all of them on the normal path)
      const uint32_t last = g < kCtStages ? g : kCtStages;
      for (uint32_t k = 1; k <= last; ++k) ct_wait(&full[(g - k) % kCtStages], ((g - k) / kCtStages) & 1u);
    }
  } else if (warp == 5) {
    // ---- MMA issuer ----------------------------------------------------------
    if (lane == 0) {
      const uint64_t adesc0 = ct_desc(ct_smem(sA), 4u, 512u);
      const uint64_t bdesc0 = ct_desc(ct_smem(sB), 2u, 1024u);
      uint32_t g = 0, it = 0;
      bool ok = true, issued = false;
      for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++it) {
        const uint32_t b = it & 1u;
        if (it >= 2 && !ct_wait(&acc_empty[b], ((it >> 1) - 1) & 1u)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        for (int j = 0; j < kCtStepsPerTile; ++j, ++g) {
          const uint32_t s = g % kCtStages;
          if (!ct_wait(&full[s], (g / kCtStages) & 1u) || abort_flag) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
          for (int k = 0; k < kCtTapsPerStage; ++k) {
            const int t = kCtTapsPerStage * j + k;
            const uint64_t ad = adesc0 + (uint64_t(s * kCtStageBytes + k * kCtTapBytes) >> 4);
            const uint64_t bd = bdesc0 + (uint64_t((t >> 1) * (kCtN * 128) + (t & 1) * 64) >> 4);
#pragma unroll
            for (int kk = 0; kk < 2; ++kk) {
              const uint32_t acc = (t > 0 || kk > 0) ? 1u : 0u;
              asm volatile(
                  "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                  "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem + b * kCtN),
                  "l"(ad + uint64_t(2 * kk)), "l"(bd + uint64_t(2 * kk)), "r"(kCtIdesc), "r"(acc)
                  : "memory");
            }
          }
          asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                           ct_smem(&empty[s]))
                       : "memory");
          issued = true;
        }
        if (!ok) break;
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         ct_smem(&acc_full[b]))
                     : "memory");
      }
      if (!ok) {
        abort_flag = 1;
        // the MMAs issued last have completed before tensor memory is freed
        if (issued) ct_wait(&empty[(g - 1) % kCtStages], ((g - 1) / kCtStages) & 1u);
      }
    }
  } else {
    // ---- epilogue: warps 0-3 ---------------------------------------------------
    uint32_t it = 0;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
      const uint32_t b = it & 1u;
      const bool ok = ct_wait(&acc_full[b], (it >> 1) & 1u) && !abort_flag;
      if (!__all_sync(0xffffffffu, ok ? 1 : 0)) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      uint32_t r[32];
#pragma unroll
      for (int c = 0; c < 32; c += 8)
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                     : "=r"(r[c]), "=r"(r[c + 1]), "=r"(r[c + 2]), "=r"(r[c + 3]), "=r"(r[c + 4]), "=r"(r[c + 5]),
                       "=r"(r[c + 6]), "=r"(r[c + 7])
                     : "r"(tmem + (uint32_t(32 * warp) << 16) + b * kCtN + uint32_t(c))
                     : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(ct_smem(&acc_empty[b])) : "memory");
      const long long p = tile * kCtM + 32 * warp + lane;
      uint32_t packed[16];
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        float lo = __uint_as_float(r[2 * c]), hi = __uint_as_float(r[2 * c + 1]);
        if (RELU) {
          lo = lo > 0.f ? lo : 0.f;
          hi = hi > 0.f ? hi : 0.f;
        }
        const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
        packed[c] = *reinterpret_cast<const uint32_t*>(&v);
      }
      uint4* dst = reinterpret_cast<uint4*>(out + p * 32);
#pragma unroll
      for (int q = 0; q < 4; ++q)
        dst[q] = make_uint4(packed[4 * q], packed[4 * q + 1], packed[4 * q + 2], packed[4 * q + 3]);
    }
  }
  __syncthreads();
  if (abort_flag && tid == 0) atomicExch(status, 1);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCtCols) : "memory");
}

}  // namespace cnn
}  // namespace gbfem
