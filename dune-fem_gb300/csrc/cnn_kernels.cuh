// BF16 implicit-GEMM 3-D convolution kernels (FP32 accumulate) of the
// learned preconditioner, on channels-last activations act[p][c] with
// p = x + N (y + N z) over an N^3 cell grid.
//
//   forward / backward-data : out[p][co] = sum_{t,ci} W[t][co][ci] in[nbr(p,t)][ci]
//                             (backward-data = the same kernel on flipped,
//                             transposed weights)
//   backward-weight         : dW[t][co][ci] = sum_p dout[p][co] in[nbr(p,t)][ci]
//
// The contractions run on the tensor cores with mma.sync.m16n8k16 (BF16 x
// BF16 -> FP32).  Zero padding outside the grid.  Every reduction has a fixed
// order (per-chunk partials, then a fixed-order sum), so training is bitwise
// reproducible.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace gbfem {
namespace cnn {

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi) {
  return uint32_t(__bfloat16_as_ushort(lo)) | (uint32_t(__bfloat16_as_ushort(hi)) << 16);
}

// neighbour of position p (grid N^3) through tap t (TAPS = 1 or 27), or -1
template <int TAPS>
__device__ __forceinline__ long long neighbour(long long p, int t, int N) {
  if (TAPS == 1) return p;
  const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
  const long long NN = (long long)N * N;
  const int z = int(p / NN), rem = int(p - (long long)z * NN), y = rem / N, x = rem - y * N;
  const int xx = x + dx, yy = y + dy, zz = z + dz;
  if (xx < 0 || yy < 0 || zz < 0 || xx >= N || yy >= N || zz >= N) return -1;
  return xx + (long long)N * (yy + (long long)N * zz);
}

// ---------------------------------------------------------------------------
// Convolution: one warp computes 16 output positions x COUT channels; a CTA of
// 4 warps covers 64 positions.  Weights wt[t][co][ci] (ci fastest) are staged
// in shared memory.  Epilogue: optional ReLU, output as BF16 or FP32.
// ---------------------------------------------------------------------------
template <int CIN, int COUT, int TAPS, bool RELU, typename TOUT>
__global__ void __launch_bounds__(128) conv_fwd_kernel(const bf16* __restrict__ in, const bf16* __restrict__ wt,
                                                       TOUT* __restrict__ out, int N) {
  static_assert(CIN % 16 == 0 && COUT % 8 == 0, "channel counts");
  extern __shared__ __align__(16) unsigned char smraw[];
  bf16* sw = reinterpret_cast<bf16*>(smraw);
  constexpr int WELEM = TAPS * COUT * CIN;
  {
    const uint4* src = reinterpret_cast<const uint4*>(wt);
    uint4* dst = reinterpret_cast<uint4*>(sw);
    for (int i = threadIdx.x; i < WELEM / 8; i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  const long long P = (long long)N * N * N;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, k2 = (lane & 3) * 2;
  const long long p0 = (long long)blockIdx.x * 64 + warp * 16;
  const long long r0 = p0 + g, r1 = p0 + g + 8;
  constexpr int NT = COUT / 8;
  float acc[NT][4];
#pragma unroll
  for (int j = 0; j < NT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
  const uint32_t* in32 = reinterpret_cast<const uint32_t*>(in);
  const uint32_t* sw32 = reinterpret_cast<const uint32_t*>(sw);
  for (int t = 0; t < TAPS; ++t) {
    const long long n0 = r0 < P ? neighbour<TAPS>(r0, t, N) : -1;
    const long long n1 = r1 < P ? neighbour<TAPS>(r1, t, N) : -1;
#pragma unroll
    for (int c0 = 0; c0 < CIN; c0 += 16) {
      uint32_t a[4];
      a[0] = n0 >= 0 ? __ldg(in32 + (n0 * CIN + c0 + k2) / 2) : 0u;
      a[1] = n1 >= 0 ? __ldg(in32 + (n1 * CIN + c0 + k2) / 2) : 0u;
      a[2] = n0 >= 0 ? __ldg(in32 + (n0 * CIN + c0 + k2 + 8) / 2) : 0u;
      a[3] = n1 >= 0 ? __ldg(in32 + (n1 * CIN + c0 + k2 + 8) / 2) : 0u;
#pragma unroll
      for (int j = 0; j < NT; ++j) {
        const int co = j * 8 + g;
        uint32_t b[2];
        b[0] = sw32[((t * COUT + co) * CIN + c0 + k2) / 2];
        b[1] = sw32[((t * COUT + co) * CIN + c0 + k2 + 8) / 2];
        mma_bf16(acc[j], a, b);
      }
    }
  }
#pragma unroll
  for (int j = 0; j < NT; ++j) {
    const int co = j * 8 + k2;
    float v[4] = {acc[j][0], acc[j][1], acc[j][2], acc[j][3]};
    if (RELU)
#pragma unroll
      for (int e = 0; e < 4; ++e) v[e] = v[e] > 0.f ? v[e] : 0.f;
    if (r0 < P) {
      out[r0 * COUT + co] = TOUT(v[0]);
      out[r0 * COUT + co + 1] = TOUT(v[1]);
    }
    if (r1 < P) {
      out[r1 * COUT + co] = TOUT(v[2]);
      out[r1 * COUT + co + 1] = TOUT(v[3]);
    }
  }
}

// ---------------------------------------------------------------------------
// Weight gradient partials: CTA (chunk, t) sums over positions
// [chunk*PCH, chunk*PCH + PCH) into part[chunk][t][co][ci] (FP32).
// Warps split the chunk; their tiles are added in warp order.
// A = dout^T (rows co, cols positions), B = in at neighbours (rows
// positions, cols ci): D[co][ci].
// ---------------------------------------------------------------------------
template <int CIN, int COUT, int TAPS>
__global__ void __launch_bounds__(128) conv_wgrad_kernel(const bf16* __restrict__ in, const bf16* __restrict__ dout,
                                                         float* __restrict__ part, int N, int pch) {
  constexpr int MT = COUT / 16, NT = CIN / 8;
  static_assert(COUT % 16 == 0 && CIN % 8 == 0, "channel counts");
  const int t = blockIdx.y;
  const long long P = (long long)N * N * N;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, k2 = (lane & 3) * 2;
  const long long base = (long long)blockIdx.x * pch;
  float acc[MT][NT][4];
#pragma unroll
  for (int m = 0; m < MT; ++m)
#pragma unroll
    for (int j = 0; j < NT; ++j) acc[m][j][0] = acc[m][j][1] = acc[m][j][2] = acc[m][j][3] = 0.f;
  const int per_warp = pch / 4;
  for (int ks = 0; ks < per_warp; ks += 16) {
    const long long q0 = base + warp * per_warp + ks;
    // positions of this k-step handled by the lane: q0 + k2 + {0, 1, 8, 9}
    long long pp[4] = {q0 + k2, q0 + k2 + 1, q0 + k2 + 8, q0 + k2 + 9};
    long long nb[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) nb[e] = pp[e] < P ? neighbour<TAPS>(pp[e], t, N) : -1;
    // A fragments: rows co = m*16 + g (+8), cols = the four positions
    uint32_t a[MT][4];
#pragma unroll
    for (int m = 0; m < MT; ++m) {
      const int co0 = m * 16 + g, co1 = co0 + 8;
      bf16 z = __float2bfloat16_rn(0.f);
      bf16 v00 = pp[0] < P ? dout[pp[0] * COUT + co0] : z, v01 = pp[1] < P ? dout[pp[1] * COUT + co0] : z;
      bf16 v10 = pp[0] < P ? dout[pp[0] * COUT + co1] : z, v11 = pp[1] < P ? dout[pp[1] * COUT + co1] : z;
      bf16 v02 = pp[2] < P ? dout[pp[2] * COUT + co0] : z, v03 = pp[3] < P ? dout[pp[3] * COUT + co0] : z;
      bf16 v12 = pp[2] < P ? dout[pp[2] * COUT + co1] : z, v13 = pp[3] < P ? dout[pp[3] * COUT + co1] : z;
      a[m][0] = pack2(v00, v01);
      a[m][1] = pack2(v10, v11);
      a[m][2] = pack2(v02, v03);
      a[m][3] = pack2(v12, v13);
    }
#pragma unroll
    for (int j = 0; j < NT; ++j) {
      const int ci = j * 8 + g;
      bf16 z = __float2bfloat16_rn(0.f);
      bf16 w0 = nb[0] >= 0 ? in[nb[0] * CIN + ci] : z, w1 = nb[1] >= 0 ? in[nb[1] * CIN + ci] : z;
      bf16 w2 = nb[2] >= 0 ? in[nb[2] * CIN + ci] : z, w3 = nb[3] >= 0 ? in[nb[3] * CIN + ci] : z;
      uint32_t b[2] = {pack2(w0, w1), pack2(w2, w3)};
#pragma unroll
      for (int m = 0; m < MT; ++m) mma_bf16(acc[m][j], a[m], b);
    }
  }
  // fixed-order reduction over the 4 warps: warp 0 writes, then warps 1..3 add
  __shared__ float red[COUT * CIN];
  float* out = part + ((long long)blockIdx.x * TAPS + t) * COUT * CIN;
  for (int w = 0; w < 4; ++w) {
    if (warp == w) {
#pragma unroll
      for (int m = 0; m < MT; ++m)
#pragma unroll
        for (int j = 0; j < NT; ++j) {
          const int co = m * 16 + g, ci = j * 8 + k2;
          const int e0 = co * CIN + ci, e1 = (co + 8) * CIN + ci;
          if (w == 0) {
            red[e0] = acc[m][j][0];
            red[e0 + 1] = acc[m][j][1];
            red[e1] = acc[m][j][2];
            red[e1 + 1] = acc[m][j][3];
          } else {
            red[e0] += acc[m][j][0];
            red[e0 + 1] += acc[m][j][1];
            red[e1] += acc[m][j][2];
            red[e1 + 1] += acc[m][j][3];
          }
        }
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < COUT * CIN; e += blockDim.x) out[e] = red[e];
}

// dW[t][co][ci] = sum over chunks (fixed order) of part[chunk][t][co][ci]
__global__ void wgrad_reduce_kernel(const float* __restrict__ part, float* __restrict__ dw, int nchunks, int nelem) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nelem; e += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int c = 0; c < nchunks; ++c) s += part[(long long)c * nelem + e];
    dw[e] = s;
  }
}

// ------------------------------------------------------------ elementwise --
// 32 channels per position, handled as 16 BF16 pairs; 32-bit indices (the
// network's grids hold fewer than 2^31 values, checked at creation).
constexpr int kEwC = 32, kEwPairs = kEwC / 2;
typedef __nv_bfloat162 bf162;

__device__ __forceinline__ unsigned ew_coarse(unsigned x, unsigned y, unsigned z, unsigned Nc) {
  return (x >> 1) + Nc * ((y >> 1) + Nc * (z >> 1));
}

// 2x2x2 average pooling: out[P/8][32] from in[P][32] (grid N -> N/2)
__global__ void pool_fwd_kernel(const bf16* __restrict__ in, bf16* __restrict__ out, int N, int C) {
  const unsigned Nc = unsigned(N) / 2u, total = Nc * Nc * Nc * kEwPairs;
  const bf162* in2 = reinterpret_cast<const bf162*>(in);
  bf162* out2 = reinterpret_cast<bf162*>(out);
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const unsigned c2 = e % kEwPairs, pc = e / kEwPairs;
    const unsigned x = pc % Nc, y = (pc / Nc) % Nc, z = pc / (Nc * Nc);
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const unsigned pf = (2u * x + (k & 1)) + unsigned(N) * ((2u * y + ((k >> 1) & 1)) + unsigned(N) * (2u * z + (k >> 2)));
      const float2 v = __bfloat1622float2(in2[pf * kEwPairs + c2]);
      s0 += v.x;
      s1 += v.y;
    }
    out2[e] = __floats2bfloat162_rn(0.125f * s0, 0.125f * s1);
  }
  (void)C;
}

// d_fine = (d_skip + pool_backward(d_coarse)) * (act > 0), fine grid N
__global__ void pool_bwd_add_mask_kernel(const bf16* __restrict__ dskip, const bf16* __restrict__ dcoarse,
                                         const bf16* __restrict__ act, bf16* __restrict__ dfine, int N, int C) {
  const unsigned Nn = unsigned(N), Nc = Nn / 2u, total = Nn * Nn * Nn * kEwPairs;
  const bf162* ds = reinterpret_cast<const bf162*>(dskip);
  const bf162* dc = reinterpret_cast<const bf162*>(dcoarse);
  const bf162* ac = reinterpret_cast<const bf162*>(act);
  bf162* df = reinterpret_cast<bf162*>(dfine);
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const unsigned c2 = e % kEwPairs, p = e / kEwPairs;
    const unsigned x = p % Nn, y = (p / Nn) % Nn, z = p / (Nn * Nn);
    const float2 a = __bfloat1622float2(ds[e]);
    const float2 b = __bfloat1622float2(dc[ew_coarse(x, y, z, Nc) * kEwPairs + c2]);
    const float2 m = __bfloat1622float2(ac[e]);
    float v0 = a.x + 0.125f * b.x, v1 = a.y + 0.125f * b.y;
    if (!(m.x > 0.f)) v0 = 0.f;
    if (!(m.y > 0.f)) v1 = 0.f;
    df[e] = __floats2bfloat162_rn(v0, v1);
  }
  (void)C;
}

// out_fine = upsample_nearest(coarse) + skip
__global__ void up_add_kernel(const bf16* __restrict__ coarse, const bf16* __restrict__ skip, bf16* __restrict__ out,
                              int N, int C) {
  const unsigned Nn = unsigned(N), Nc = Nn / 2u, total = Nn * Nn * Nn * kEwPairs;
  const bf162* co = reinterpret_cast<const bf162*>(coarse);
  const bf162* sk = reinterpret_cast<const bf162*>(skip);
  bf162* o = reinterpret_cast<bf162*>(out);
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const unsigned c2 = e % kEwPairs, p = e / kEwPairs;
    const unsigned x = p % Nn, y = (p / Nn) % Nn, z = p / (Nn * Nn);
    const float2 a = __bfloat1622float2(co[ew_coarse(x, y, z, Nc) * kEwPairs + c2]);
    const float2 b = __bfloat1622float2(sk[e]);
    o[e] = __floats2bfloat162_rn(a.x + b.x, a.y + b.y);
  }
  (void)C;
}

// d_coarse = (sum of the 8 children of d_fine) * (act_coarse > 0)
__global__ void up_bwd_mask_kernel(const bf16* __restrict__ dfine, const bf16* __restrict__ act,
                                   bf16* __restrict__ dcoarse, int N, int C) {
  const unsigned Nc = unsigned(N) / 2u, total = Nc * Nc * Nc * kEwPairs;
  const bf162* df = reinterpret_cast<const bf162*>(dfine);
  const bf162* ac = reinterpret_cast<const bf162*>(act);
  bf162* dc = reinterpret_cast<bf162*>(dcoarse);
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const unsigned c2 = e % kEwPairs, pc = e / kEwPairs;
    const unsigned x = pc % Nc, y = (pc / Nc) % Nc, z = pc / (Nc * Nc);
    float s0 = 0.f, s1 = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const unsigned pf = (2u * x + (k & 1)) + unsigned(N) * ((2u * y + ((k >> 1) & 1)) + unsigned(N) * (2u * z + (k >> 2)));
      const float2 v = __bfloat1622float2(df[pf * kEwPairs + c2]);
      s0 += v.x;
      s1 += v.y;
    }
    const float2 m = __bfloat1622float2(ac[e]);
    if (!(m.x > 0.f)) s0 = 0.f;
    if (!(m.y > 0.f)) s1 = 0.f;
    dc[e] = __floats2bfloat162_rn(s0, s1);
  }
  (void)C;
}

// x *= (act > 0), n values (even)
__global__ void relu_mask_kernel(bf16* __restrict__ x, const bf16* __restrict__ act, long long n) {
  bf162* x2 = reinterpret_cast<bf162*>(x);
  const bf162* a2 = reinterpret_cast<const bf162*>(act);
  const unsigned total = unsigned(n / 2);
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const float2 m = __bfloat1622float2(a2[e]);
    float2 v = __bfloat1622float2(x2[e]);
    if (!(m.x > 0.f)) v.x = 0.f;
    if (!(m.y > 0.f)) v.y = 0.f;
    x2[e] = __floats2bfloat162_rn(v.x, v.y);
  }
}

}  // namespace cnn
}  // namespace gbfem
