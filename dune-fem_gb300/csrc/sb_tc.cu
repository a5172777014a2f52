// Scaled shared-block Jacobi on the 5th-generation tensor cores (tcgen05).
//
// The preconditioner z_c = H_t(c)^-1 r_c / kappa_c of a cellwise-kappa DG
// operator (solver.cu) applied to tiles of up to 32 cells of one boundary
// type t is a dense product Z = H_t^-1 R of a (n^3 x n^3) inverse and an
// (n^3 x 32) tile of residuals, n^3 <= 125.  Here each tile is one sequence
// of tcgen05.mma instructions (kind::tf32, M = 128 rows of H^-1, N = 32
// cells, K = 8 per instruction) accumulating in tensor memory:
//  - FP32 accuracy by the 3xTF32 split (Ootomo & Yokota, IJHPCA 2022): with
//    A = A_hi + A_lo and B = B_hi + B_lo rounded to TF32,
//    A B ~ A_hi B_hi + A_hi B_lo + A_lo B_hi, three MMAs per K step;
//  - the operands sit in shared memory in the K-major layout with the
//    128-byte swizzle (8 rows of 128 bytes per swizzle atom, 16-byte chunks
//    XOR-ed with the row); A_hi | A_lo of every type are precomputed in that
//    layout once (k_sb_tc_image) and staged into shared memory with one bulk
//    TMA copy (cp.async.bulk) whenever the type changes;
//  - one persistent CTA (512 threads) per SM over a contiguous range of
//    tiles, sorted by type.  While the MMAs of tile i run, all threads issue
//    the loads of tile i+2's residuals (coalesced along each cell's dofs, into
//    registers), split tile i+1's (loaded one iteration earlier) into B_hi,
//    B_lo and write them in the swizzled layout (a warp writes one 128-byte
//    row: no bank conflicts); then the 16 warps read tile i's 128 x 32
//    accumulator with tcgen05.ld (warp w reads TMEM lanes 32 (w mod 4) ..
//    + 31, 8 of the 32 columns), divide by kappa_c and store z (each
//    cell's rows are contiguous).
//    Cell indices are read four tiles ahead and kappa two tiles ahead, so
//    no iteration waits on a chain of dependent loads.  B and the
//    accumulators are double-buffered (two 32-column FP32 accumulators in
//    TMEM).
// Every wait on an mbarrier is bounded: on a timeout the kernel records it in
// a status word (gbfem_preconditioner_status), stops issuing work, frees its
// tensor memory and returns.
#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>
#include <vector>

#include "gbfem_internal.cuh"
#include "solver_impl.hpp"

namespace gbfem {

constexpr int kTcThreads = 512;
constexpr int kTcWarps = kTcThreads / 32;
constexpr int kTcM = 128;
// (the tile list of the CTA, kTcMaxTilesPerCta x 3 ints, is static shared memory)
constexpr uint32_t kTcWaitLimit = 1u << 24;      // try_wait polls before a wait is declared failed
constexpr int kTcMaxTilesPerCta = 1024;          // tile list staged in shared memory (12 KB)
constexpr int kIssuer = (kTcWarps - 1) * 32;     // the thread that issues the MMAs and the TMA copies

// Tile shape: TN cells per tile (the MMA's N), TK the padded block size (K).
// Blocks of up to 128 dofs (Q4) take 32-cell tiles with K = 128; blocks of up
// to 64 dofs (Q3 and below) 64-cell tiles with K = 64, which halves the
// number of tiles and with it the per-tile cost (barriers, MMA completion,
// epilogue) that dominates the apply.
template <int TN, int TK>
struct TcShape {
  static constexpr int CellsPerWarp = TN / kTcWarps;     // gather: cells per warp and tile
  static constexpr int ColsPerWarp = TN * 4 / kTcWarps;  // epilogue: accumulator columns per warp
  static constexpr int Slots = TN / 32;                  // cell indices a lane holds per tile
  static constexpr int KAtoms = TK / 32;                 // 128-byte K atoms (32 TF32 values)
  static constexpr uint32_t ABytes = kTcM * TK * 4;      // one of A_hi / A_lo
  static constexpr uint32_t BBytes = TN * TK * 4;        // one of B_hi / B_lo
  static constexpr size_t Smem = 2 * size_t(ABytes) + 4 * size_t(BBytes) + 1024;  // + alignment slack
  static constexpr uint32_t Cols = 2 * TN;               // two TN-column FP32 accumulators
  // kind::tf32, FP32 accumulator, A and B TF32, both K-major, N = TN, M = 128
  static constexpr uint32_t Idesc = (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(TN >> 3) << 17) |
                                    (uint32_t(kTcM >> 4) << 24);
  static_assert(CellsPerWarp * kTcWarps == TN && ColsPerWarp % 8 == 0 && Slots >= 1 && Slots <= 2, "tile shape");
};
using TcQ4 = TcShape<32, 128>;
using TcQ3 = TcShape<64, 64>;

// Byte offset of element (row m, k) of a K-major operand with `rows` rows
// and K = 128 in the 128-byte-swizzled layout: four K atoms of 32 elements,
// each [rows / 8 groups][8 rows][128 bytes], chunk (16 bytes) index XOR row.
__host__ __device__ __forceinline__ uint32_t tc_swz_offset(int m, int k, int rows) {
  const uint32_t off = uint32_t(k >> 5) * uint32_t(rows) * 128u + uint32_t(m >> 3) * 1024u + uint32_t(m & 7) * 128u +
                       uint32_t(k & 31) * 4u;
  return off ^ (((off >> 7) & 7u) << 4);
}

__device__ __forceinline__ uint32_t tc_smem(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ float tc_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
  uint64_t d = uint64_t((saddr & 0x3FFFFu) >> 4);  // start address
  d |= uint64_t(1) << 16;                           // leading byte offset (unused with this swizzle)
  d |= uint64_t(1024u >> 4) << 32;                  // stride byte offset
  d |= uint64_t(1) << 46;                           // descriptor version
  d |= uint64_t(2) << 61;                           // 128-byte swizzle
  return d;
}

__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(tc_smem(bar))
               : "memory");
}

__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t it = 0; it < kTcWaitLimit; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(tc_smem(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 8 consecutive accumulator columns of this warp's 32 TMEM lanes.
__device__ __forceinline__ void tc_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr)
               : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// A_hi | A_lo of every type: element (i, j) = H_t^-1[i][j] = hinvT[t][j nb + i]
// (rows padded to 128 and K to TK with zeros), TF32-rounded, swizzled.
template <int TK>
__global__ void k_sb_tc_image(const float* __restrict__ hinvT, int ntypes, int nb, float* __restrict__ img) {
  const long long total = (long long)ntypes * kTcM * TK;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int t = int(e / (kTcM * TK));
    const int rem = int(e - (long long)t * kTcM * TK);
    const int m = rem / TK, k = rem - m * TK;
    const float v = (m < nb && k < nb) ? hinvT[(long long)t * nb * nb + (long long)k * nb + m] : 0.0f;
    const float hi = tc_tf32(v), lo = tc_tf32(v - hi);
    const uint32_t off = tc_swz_offset(m, k, kTcM) >> 2;
    img[(long long)(2 * t) * (kTcM * TK) + off] = hi;
    img[(long long)(2 * t + 1) * (kTcM * TK) + off] = lo;
  }
}

// element q (0 or 1) of a lane's per-tile slot array, without indexing
// registers by a runtime value
template <int SL, typename V>
__device__ __forceinline__ V tc_pick(const V (&a)[SL], int q) {
  if (SL == 1) return a[0];
  return q ? a[SL - 1] : a[0];
}

// tiles: (type, start, count) with 1 <= count <= TN, sorted by type.
template <int TN, int TK>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_sb_tc_apply(const float* __restrict__ img, const float* __restrict__ kcell, const int* __restrict__ cells,
                  const int* __restrict__ tiles, int ntiles, const float* __restrict__ r, float* __restrict__ z, int nb,
                  int* __restrict__ status) {
  using S = TcShape<TN, TK>;
  constexpr int SL = S::Slots, CPW = S::CellsPerWarp, KA = S::KAtoms, CW = S::ColsPerWarp;
  extern __shared__ unsigned char tc_raw[];
  __shared__ __align__(8) uint64_t bar_mma, bar_a;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  __shared__ int smeta[3 * kTcMaxTilesPerCta];  // (type, start, count) of the CTA's tiles
  const int i0 = int((long long)blockIdx.x * ntiles / gridDim.x);
  const int i1 = int((long long)(blockIdx.x + 1) * ntiles / gridDim.x);
  if (i0 >= i1) return;  // the same for the whole CTA, before any set-up
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // 1024-byte aligned operand area (the swizzle pattern follows address bits 4-9)
  unsigned char* base =
      tc_raw + ((1024u - (tc_smem(tc_raw) & 1023u)) & 1023u);
  unsigned char* sA = base;                    // A_hi | A_lo
  unsigned char* sB = base + 2 * S::ABytes;    // [buffer][hi | lo]
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem(&tmem_base)),
                 "r"(S::Cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  for (int e = tid; e < 3 * (i1 - i0); e += kTcThreads) smeta[e] = tiles[3 * i0 + e];
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&bar_mma)) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&bar_a)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    abort_flag = 0;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;

  // Software pipeline (per lane): the tile list and cell indices are read
  // four tiles ahead, kappa two tiles ahead, and the residuals of tile i+2
  // are loaded into registers while tile i+1's (loaded one iteration
  // earlier) are written to shared memory, so no iteration waits on a chain
  // of dependent global loads.
  const int* meta = smeta - 3 * i0;  // meta[3 i + 0..2]: type, start, count of tile i
  // Loads are issued under a predicate into a zeroed register and nothing
  // uses their value before it is needed (no select or reciprocal right
  // after the load): the warp does not wait for them here.
  // a lane holds the indices (and kappas) of cells lane and 32 + lane of a tile
  auto cell_of = [&](int i, int (&v)[SL]) {
#pragma unroll
    for (int q = 0; q < SL; ++q) {
      v[q] = 0;
      if (i < i1 && 32 * q + lane < meta[3 * i + 2]) v[q] = __ldg(cells + meta[3 * i + 1] + 32 * q + lane);
    }
  };
  auto kappa_of = [&](int i, const int (&mycell)[SL], float (&v)[SL]) {
#pragma unroll
    for (int q = 0; q < SL; ++q) {
      v[q] = 1.0f;
      if (i < i1 && 32 * q + lane < meta[3 * i + 2]) v[q] = __ldg(kcell + mycell[q]);
    }
  };
  // warp w takes cells w, w+16, .., lanes the dofs k = 32 a + lane of each
  // (one coalesced 128-byte row each); cell w + 16 m sits in slot m / 2,
  // lane 16 (m mod 2) + w
  auto load_vals = [&](int i, const int (&mycell)[SL], float (&v)[CPW][KA]) {
    const int count = meta[3 * i + 2];
#pragma unroll
    for (int m = 0; m < CPW; ++m) {
      const int c = warp + kTcWarps * m;
      const int cell = __shfl_sync(0xffffffffu, mycell[m >> 1 < SL ? m >> 1 : SL - 1], c & 31);
#pragma unroll
      for (int a = 0; a < KA; ++a) {
        const int k = 32 * a + lane;
        v[m][a] = 0.0f;
        if (c < count && k < nb) v[m][a] = __ldg(r + (long long)cell * nb + k);
      }
    }
  };
  // B_hi, B_lo of buffer b; a warp writes one 128-byte row per store
  auto store_vals = [&](const float (&v)[CPW][KA], int b) {
    unsigned char* bh = sB + (2 * b) * S::BBytes;
    unsigned char* bl = bh + S::BBytes;
#pragma unroll
    for (int m = 0; m < CPW; ++m)
#pragma unroll
      for (int a = 0; a < KA; ++a) {
        const uint32_t off = tc_swz_offset(warp + kTcWarps * m, 32 * a + lane, TN);
        const float hi = tc_tf32(v[m][a]);
        *reinterpret_cast<float*>(bh + off) = hi;
        *reinterpret_cast<float*>(bl + off) = tc_tf32(v[m][a] - hi);
      }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // visible to the tensor cores
  };

  const int ksteps = (nb + 7) / 8;  // K steps that touch nonzero data
  int cur_type = -1;
  uint32_t a_phase = 0;
  // the issuing thread (lane 0 of warp 7, which has no epilogue work):
  // stage the tile's inverse if its type changed, then the tile's MMAs
  auto issue = [&](int i, int b) -> bool {
    const int type = meta[3 * i];
    if (type != cur_type) {
      const uint32_t bytes = 2 * S::ABytes;
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc_smem(&bar_a)), "r"(bytes)
                   : "memory");
      const unsigned char* src = reinterpret_cast<const unsigned char*>(img) + (size_t)type * bytes;
      for (uint32_t o = 0; o < bytes; o += 32768u)
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                tc_smem(sA + o)),
            "l"(src + o), "r"(32768u), "r"(tc_smem(&bar_a))
            : "memory");
      if (!tc_wait(&bar_a, a_phase & 1u)) return false;
      ++a_phase;
      cur_type = type;
    }
    tc_fence_after();
    // descriptors advance by the K offset in their start-address field
    // (16-byte units): 32 bytes per K step inside a 128-byte atom, the
    // atom's size from one atom to the next
    const uint64_t dah = tc_desc(tc_smem(sA)), dal = tc_desc(tc_smem(sA) + S::ABytes);
    const uint64_t dbh = tc_desc(tc_smem(sB + (2 * b) * S::BBytes)), dbl = tc_desc(tc_smem(sB + (2 * b + 1) * S::BBytes));
    const uint32_t d = tmem + uint32_t(b) * TN;
    for (int kb = 0; kb < ksteps; ++kb) {
      const uint64_t ao = (uint64_t(kb >> 2) * (kTcM * 128u) + uint64_t(kb & 3) * 32u) >> 4;
      const uint64_t bo = (uint64_t(kb >> 2) * (TN * 128u) + uint64_t(kb & 3) * 32u) >> 4;
      tc_mma(d, dah + ao, dbh + bo, S::Idesc, kb > 0 ? 1u : 0u);
      tc_mma(d, dah + ao, dbl + bo, S::Idesc, 1u);
      tc_mma(d, dal + ao, dbh + bo, S::Idesc, 1u);
    }
    tc_commit(&bar_mma);
    return true;
  };

  // Rings indexed by the tile's position in the range: cell indices and
  // kappa in four slots (tile t in slot (t - i0) & 3), residuals in two
  // (parity).  The loop below is unrolled by four so that every slot is a
  // fixed register set: no copy at the end of an iteration waits for the
  // loads just issued.
  int cr[4][SL];
  float ir[4][SL];
  float va[CPW][KA], vb[CPW][KA];
  cell_of(i0, cr[0]);
  cell_of(i0 + 1, cr[1]);
  cell_of(i0 + 2, cr[2]);
  cell_of(i0 + 3, cr[3]);
  kappa_of(i0, cr[0], ir[0]);
  kappa_of(i0 + 1, cr[1], ir[1]);
#pragma unroll
  for (int q = 0; q < SL; ++q) ir[2][q] = ir[3][q] = 1.0f;
  load_vals(i0, cr[0], va);
  if (i0 + 1 < i1) load_vals(i0 + 1, cr[1], vb);
  store_vals(va, 0);
  __syncthreads();
  if (tid == kIssuer && !issue(i0, 0)) abort_flag = 1;
  __syncthreads();
  // tile i, position j = (i - i0) & 3 (compile-time)
  auto body = [&](auto J, int i) -> bool {
    constexpr int j = decltype(J)::value;
    const int b = j & 1;
    float(&vnext)[CPW][KA] = (j & 1) ? vb : va;  // tile i+2 (tile i's slot, stored last iteration)
    float(&vcur)[CPW][KA] = (j & 1) ? va : vb;   // tile i+1 (loaded last iteration)
    if (i + 2 < i1) load_vals(i + 2, cr[(j + 2) & 3], vnext);
    if (i + 1 < i1) store_vals(vcur, b ^ 1);
    {
      // tile i's accumulator: warp w reads TMEM lanes 32 (w mod 4) + lane (the
      // rows) and columns CW (w / 4) .. (the tile's cells; one slot per warp)
      const bool ok = tc_wait(&bar_mma, uint32_t(i - i0) & 1u);
      if (!ok) abort_flag = 1;
      tc_fence_after();
      if (ok) {
        const int count = meta[3 * i + 2];
        const int quarter = warp & 3, c0 = CW * (warp >> 2);
        const int q = c0 >> 5;  // warp-uniform slot of this warp's columns
        const float inv = 1.0f / tc_pick<SL>(ir[j], q);
        const int mycell = tc_pick<SL>(cr[j], q);
        float acc[CW];
#pragma unroll
        for (int g = 0; g < CW / 8; ++g) {
          float a8[8];
          tc_ld8(tmem + (uint32_t(32 * quarter) << 16) + uint32_t(b) * TN + uint32_t(c0 + 8 * g), a8);
#pragma unroll
          for (int e = 0; e < 8; ++e) acc[8 * g + e] = a8[e];
        }
        const int row = 32 * quarter + lane;
#pragma unroll
        for (int cc = 0; cc < CW; ++cc) {
          const int c = c0 + cc;
          const int cell = __shfl_sync(0xffffffffu, mycell, c & 31);
          const float s = __shfl_sync(0xffffffffu, inv, c & 31);
          if (c < count && row < nb) z[(long long)cell * nb + row] = acc[cc] * s;
        }
      }
    }
    tc_fence_before();
    __syncthreads();  // the next buffer is gathered, this accumulator is read
    if (abort_flag) return false;
    if (i + 1 < i1 && tid == kIssuer && !issue(i + 1, b ^ 1)) abort_flag = 1;
    // refill the slots tile i freed: its cell slot takes tile i+4, and
    // tile i+2's kappa (its cell index arrived two iterations ago)
    cell_of(i + 4, cr[j]);
    kappa_of(i + 2, cr[(j + 2) & 3], ir[(j + 2) & 3]);
    return true;
  };
  for (int i = i0; i < i1; i += 4) {
    if (!body(std::integral_constant<int, 0>(), i)) break;
    if (i + 1 >= i1 || !body(std::integral_constant<int, 1>(), i + 1)) break;
    if (i + 2 >= i1 || !body(std::integral_constant<int, 2>(), i + 2)) break;
    if (i + 3 >= i1 || !body(std::integral_constant<int, 3>(), i + 3)) break;
  }
  __syncthreads();
  if (abort_flag && tid == 0) atomicExch(status, 1);
  tc_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(S::Cols) : "memory");
}

// SMs of the current device.
static int tc_num_sms() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) ==
                                                cudaSuccess && v > 0)
    return v;
  return 152;
}

// Set-up at creation: the type images and the tiles without padding.
int sb_tc_setup(gbfem_preconditioner_s* pc, const std::vector<int>& tiles3, int nb, cudaStream_t s) {
  std::vector<int> t;
  int maxtype = 0;
  // blocks of up to 64 dofs: consecutive tiles of one type (their cells are
  // contiguous in the cell list) merge into tiles of up to 64 cells
  const bool wide = nb <= 64;
  const int cap = wide ? 64 : 32;
  for (size_t k = 0; k + 2 < tiles3.size(); k += 3)
    if (tiles3[k + 2] > 0) {
      const size_t last = t.size();
      if (last >= 3 && t[last - 3] == tiles3[k] && t[last - 2] + t[last - 1] == tiles3[k + 1] &&
          t[last - 1] + tiles3[k + 2] <= cap) {
        t[last - 1] += tiles3[k + 2];
      } else {
        t.push_back(tiles3[k]);
        t.push_back(tiles3[k + 1]);
        t.push_back(tiles3[k + 2]);
      }
      maxtype = tiles3[k] > maxtype ? tiles3[k] : maxtype;
    }
  const int ntypes = maxtype + 1;
  pc->sb_tc_wide = wide ? 1 : 0;
  GBFEM_CUDA_TRY(cudaMalloc(&pc->sb_tc_tiles, t.size() * sizeof(int)));
  GBFEM_CUDA_TRY(cudaMemcpy(pc->sb_tc_tiles, t.data(), t.size() * sizeof(int), cudaMemcpyHostToDevice));
  pc->sb_tc_ntiles = int(t.size() / 3);
  GBFEM_CUDA_TRY(cudaMalloc(&pc->sb_tc_img, size_t(ntypes) * 2 * (wide ? TcQ3::ABytes : TcQ4::ABytes)));
  GBFEM_CUDA_TRY(cudaMalloc(&pc->sb_tc_status, sizeof(int)));
  GBFEM_CUDA_TRY(cudaMemsetAsync(pc->sb_tc_status, 0, sizeof(int), s));
  if (wide)
    k_sb_tc_image<64><<<tc_num_sms() * 4, 256, 0, s>>>(static_cast<const float*>(pc->data), ntypes, nb,
                                                       static_cast<float*>(pc->sb_tc_img));
  else
    k_sb_tc_image<128><<<tc_num_sms() * 4, 256, 0, s>>>(static_cast<const float*>(pc->data), ntypes, nb,
                                                        static_cast<float*>(pc->sb_tc_img));
  GBFEM_CUDA_TRY(cudaGetLastError());
  GBFEM_CUDA_TRY(cudaStreamSynchronize(s));
  return GBFEM_OK;
}

int sb_tc_apply(const gbfem_preconditioner_s* pc, const float* kcell, const float* r, float* z, cudaStream_t s) {
  const int nb = pc->nloc;
  if (nb > kTcM) return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "tensor-core block Jacobi: blocks above 128 dofs");
  const int n = pc->sb_tc_ntiles;
  if (n <= 0) return GBFEM_OK;
  const bool wide = pc->sb_tc_wide != 0;
  if (wide && nb > 64) return set_error(GBFEM_ERR_INVALID, "tensor-core block Jacobi: wide tiles need blocks <= 64");
  auto kern = wide ? k_sb_tc_apply<64, 64> : k_sb_tc_apply<32, 128>;
  const size_t smem = wide ? TcQ3::Smem : TcQ4::Smem;
  GBFEM_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  const int sms = tc_num_sms();
  int grid = n < sms ? n : sms;
  if ((n + grid - 1) / grid > kTcMaxTilesPerCta) grid = (n + kTcMaxTilesPerCta - 1) / kTcMaxTilesPerCta;
  kern<<<grid, kTcThreads, smem, s>>>(static_cast<const float*>(pc->sb_tc_img), kcell, pc->sor_cells, pc->sb_tc_tiles,
                                      n, r, z, nb, pc->sb_tc_status);
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

}  // namespace gbfem
