// One-kernel FP32 apply of the constant-coefficient closed form (the same
// operator as dg_trace_kernel + dg_const_kernel; the algebra is described in
// dg_const_kernel.cuh), without the trace buffer in HBM.
//
// Layout of the work: a CTA of 128 threads owns a brick of 8 x 4 x 4 cells,
// one cell per thread, and keeps the cell's n^3 dofs and n^3 results in
// registers (n <= 4: 128 registers at Q3).  A face's numerical flux is
// computed once and exchanged through shared memory, which holds one slot per
// face of the brick ((8+1) 4 4 + 8 (4+1) 4 + 8 4 (4+1) = 464 slots of 2 n^2
// values) plus one per face on the brick's lower boundary (80; 69.6 KB at Q3,
// three CTAs per SM).  Slots are 128-byte rows whose 16-byte chunks are
// XOR-swizzled by the slot index, so lanes at consecutive slots read
// distinct banks without padding.
//  0. every thread loads its cell's dofs (float4 loads where the cell's block
//     is 16-byte aligned).  Halo items, spread over the threads, load the
//     brick's face neighbours outside it (2 (8*4 + 8*4 + 4*4) cells per 128,
//     read through L2 -- the only traffic besides u and w) and write the
//     trace of each one's face that touches the brick into that face's slot;
//  1. every cell writes the two traces (v, P) of its lower face along each
//     axis into that face's slot, or, on the brick's lower boundary, into the
//     boundary slot;
//  2. every cell computes the flux of its upper face along each axis from its
//     own traces and the slot (its upper neighbour's traces) and overwrites
//     the slot with (Val, G) as seen from the face's lower cell; boundary items
//     do the same for the brick's lower faces from the halo and boundary
//     slots.  The upper cell of a face reads the numbers negated: the interior
//     fluxes are odd in the two sides' traces (Val(-, +) = -Val(+, -), J
//     likewise), which holds exactly in floating point because rounding is
//     symmetric; a domain-boundary face's terms are stored negated where the
//     cell is the upper one;
//  3. one pass per axis over the cell's lines applies the 1-D line operator
//     and the face expansion (the same formulas and summation order as
//     dg_const_kernel's line pass), accumulating in registers;
//  4. the results are stored once.
// Every output is one thread's fixed-order sum: deterministic, independent of
// the launch.
#pragma once
#include <cuda_runtime.h>

#include "dg_const_kernel.cuh"

namespace gbfem {

constexpr int kCellBX = 8, kCellBY = 4, kCellBZ = 4;
constexpr int kCellThreads = kCellBX * kCellBY * kCellBZ;

template <int N>
struct CellSlots {
  static constexpr int N2 = N * N;
  static constexpr int H = (N2 + 3) / 4 * 4;  // floats per half slot (v or Val | P or G), float4-aligned
  static constexpr int Q = H / 2;             // float4 chunks in use per slot
  static constexpr int QS = Q <= 2 ? 2 : (Q <= 4 ? 4 : 8);  // chunks per slot (a power of two)
  static constexpr int NX = (kCellBX + 1) * kCellBY * kCellBZ;
  static constexpr int NY = kCellBX * (kCellBY + 1) * kCellBZ;
  static constexpr int NZ = kCellBX * kCellBY * (kCellBZ + 1);
  static constexpr int NFACE = NX + NY + NZ;
  static constexpr int NBND = kCellBY * kCellBZ + kCellBX * kCellBZ + kCellBX * kCellBY;  // lower boundary
  static constexpr int FLOATS = (NFACE + NBND) * QS * 4;
  static constexpr size_t BYTES = size_t(FLOATS) * sizeof(float);
};

// Slot of the face at position f (0..B_d) along axis d; la, lb are the
// brick-local coordinates along the other two axes (in increasing axis
// order).  Consecutive x positions are consecutive slots.
template <int N>
__device__ __forceinline__ int cell_slot(int d, int f, int la, int lb) {
  using S = CellSlots<N>;
  if (d == 0) return f + (kCellBX + 1) * (la + kCellBY * lb);
  if (d == 1) return S::NX + la + kCellBX * (f + (kCellBY + 1) * lb);
  return S::NX + S::NY + la + kCellBX * (lb + kCellBY * f);
}

// Boundary slot of the brick cell's lower face along d (its lower traces).
template <int N>
__device__ __forceinline__ int cell_bnd_slot(int d, int la, int lb) {
  using S = CellSlots<N>;
  if (d == 0) return S::NFACE + la + kCellBY * lb;
  if (d == 1) return S::NFACE + kCellBY * kCellBZ + la + kCellBX * lb;
  return S::NFACE + kCellBY * kCellBZ + kCellBX * kCellBZ + la + kCellBX * lb;
}

// Address of logical chunk q of slot s (XOR swizzle within the slot).
template <int N>
__device__ __forceinline__ float4* cell_chunk(float* slots, int s, int q) {
  using S = CellSlots<N>;
  return reinterpret_cast<float4*>(slots) + s * S::QS + (q ^ (s & (S::QS - 1)));
}

// Offset of value i of tangential line jk (= j n + k) along axis D within a
// cell's n^3 block (local index i0 n^2 + i1 n + i2; the same convention as
// dg_trace_kernel).
template <int N, int D>
__host__ __device__ constexpr int cell_line_off(int jk, int i) {
  return D == 0 ? i * N * N + jk
                : (D == 1 ? (jk / N) * N * N + i * N + (jk % N) : (jk / N) * N * N + (jk % N) * N + i);
}

// Both traces of face `upper` of every line along axis D: v = sum_i L_i(s)
// x_i and P = sum_i (+-1)^i pc_i x_i, from one even and one odd partial sum.
// L_0 = 1; the constant-kappa pc_0 is 1 as well, the kappa-per-cell pc_0 is
// L_0'(1) = 0.
template <int N, bool KC, int D>
__device__ __forceinline__ void cell_traces(const float (&x)[N * N * N], bool upper, const DgConstTablesT<float>& tabs,
                                            float (&v)[N * N], float (&p)[N * N]) {
#pragma unroll
  for (int jk = 0; jk < N * N; ++jk) {
    float ev = x[cell_line_off<N, D>(jk, 0)], od = 0.f, pe = KC ? 0.f : ev, po = 0.f;
#pragma unroll
    for (int i = 1; i < N; ++i) {
      const float xi = x[cell_line_off<N, D>(jk, i)];
      if (i & 1) {
        od = fmaf(tabs.tr[N + i], xi, od);
        po = fmaf(tabs.pc[D][i], xi, po);
      } else {
        ev = fmaf(tabs.tr[N + i], xi, ev);
        pe = fmaf(tabs.pc[D][i], xi, pe);
      }
    }
    v[jk] = upper ? ev + od : ev - od;
    p[jk] = upper ? pe + po : pe - po;
  }
}

// The flux through an interior face normal to D as seen from its lower cell
// m: (Val, G) per tangential coefficient from m's upper-face traces and the
// upper cell p's lower-face traces (dg_const_kernel's formulas).
template <int N, bool ADV, bool KC, int D>
__device__ __forceinline__ void cell_interior_flux(const float (&vm)[N * N], const float (&pm)[N * N],
                                                   const float (&vp)[N * N], const float (&pp)[N * N], float km,
                                                   float kp, const DgArgsT<float>& args,
                                                   const DgConstTablesT<float>& tabs, float (&val)[N * N],
                                                   float (&G)[N * N]) {
  const bool fold_alpha = tabs.am1 != 0.f;
#pragma unroll
  for (int jk = 0; jk < N * N; ++jk) {
    const float J = vm[jk] - vp[jk];
    float vv;
    if (KC) {
      vv = fmaf(tabs.A1[D] * (0.5f * (km + kp)), J, -tabs.A2[D] * (km * pm[jk] - kp * pp[jk]));
    } else {
      vv = pm[jk] - pp[jk];
      if (fold_alpha) vv = fmaf(tabs.am1, J, vv);
      if (ADV) vv = fmaf(tabs.adv[2 * D + 1], args.b[D] >= 0.f ? vm[jk] : vp[jk], vv);
    }
    val[jk] = vv;
    G[jk] = J;
  }
}

// A domain-boundary face normal to D (the Nitsche and outflow terms) from
// the cell's own traces on it; stored negated when it is the cell's lower
// face (the slot convention: as seen from the face's lower side).
template <int N, bool ADV, bool KC, int D>
__device__ __forceinline__ void cell_boundary_flux(bool upper, const float (&vo)[N * N],
                                                   const float (&po)[N * N], float kc, const DgArgsT<float>& args,
                                                   const DgConstTablesT<float>& tabs, float (&val)[N * N],
                                                   float (&G)[N * N]) {
  const float bn = upper ? args.b[D] : -args.b[D];
#pragma unroll
  for (int jk = 0; jk < N * N; ++jk) {
    float vv = 0.f, gg = 0.f;
    if (args.weak_dirichlet) {
      if (KC) vv = fmaf(tabs.A1[D] * kc, vo[jk], -2.f * tabs.A2[D] * kc * po[jk]);
      else vv = fmaf(tabs.am2, vo[jk], po[jk] + po[jk]);
      gg = vo[jk] + vo[jk];
    }
    if (ADV && bn > 0.f) vv = fmaf(tabs.adv[2 * D + (upper ? 1 : 0)], vo[jk], vv);
    val[jk] = upper ? vv : -vv;
    G[jk] = upper ? gg : -gg;
  }
}

// Writes a[0..N2) and b[0..N2) into slot s (float4 stores, zero padding).
template <int N>
__device__ __forceinline__ void cell_store_slot(float* slots, int s, const float (&a)[N * N],
                                                const float (&b)[N * N]) {
  constexpr int N2 = N * N, H = CellSlots<N>::H;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const float* src = h ? b : a;
#pragma unroll
    for (int q = 0; q < H / 4; ++q) {
      float4 t;
      t.x = 4 * q + 0 < N2 ? src[4 * q + 0] : 0.f;
      t.y = 4 * q + 1 < N2 ? src[4 * q + 1] : 0.f;
      t.z = 4 * q + 2 < N2 ? src[4 * q + 2] : 0.f;
      t.w = 4 * q + 3 < N2 ? src[4 * q + 3] : 0.f;
      *cell_chunk<N>(slots, s, h * (H / 4) + q) = t;
    }
  }
}

template <int N>
__device__ __forceinline__ void cell_load_slot(float* slots, int s, float (&a)[N * N], float (&b)[N * N]) {
  constexpr int N2 = N * N, H = CellSlots<N>::H;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float* dst = h ? b : a;
#pragma unroll
    for (int q = 0; q < H / 4; ++q) {
      const float4 t = *cell_chunk<N>(slots, s, h * (H / 4) + q);
      if (4 * q + 0 < N2) dst[4 * q + 0] = t.x;
      if (4 * q + 1 < N2) dst[4 * q + 1] = t.y;
      if (4 * q + 2 < N2) dst[4 * q + 2] = t.z;
      if (4 * q + 3 < N2) dst[4 * q + 3] = t.w;
    }
  }
}

// Loads a cell's n^3 dofs into registers.
template <int N>
__device__ __forceinline__ void cell_load_dofs(const float* __restrict__ src, float (&x)[N * N * N]) {
  constexpr int N3 = N * N * N;
  if constexpr (N3 % 4 == 0) {
    const float4* s4 = reinterpret_cast<const float4*>(src);
#pragma unroll
    for (int q = 0; q < N3 / 4; ++q) {
      const float4 t = __ldg(s4 + q);
      x[4 * q] = t.x;
      x[4 * q + 1] = t.y;
      x[4 * q + 2] = t.z;
      x[4 * q + 3] = t.w;
    }
  } else {
#pragma unroll
    for (int e = 0; e < N3; ++e) x[e] = __ldg(src + e);
  }
}

// Brick geometry shared by the phases.
struct CellBrick {
  int nc[3];
  int o[3];  // first cell of the brick
  int e[3];  // the brick's extent inside the grid
  long long stride[3];
};

// The face neighbour of brick-boundary position (D, la, lb) below (upper =
// false) or above the brick; false where the domain ends there.
template <int D>
__device__ __forceinline__ bool cell_halo_neighbour(bool upper, int la, int lb, const CellBrick& B,
                                                    const DgArgsT<float>& args, long long* hcell, long long* bcell) {
  constexpr int A = D == 0 ? 1 : 0, Bx = D == 2 ? 1 : 2;  // the other axes, increasing
  const long long tang = (long long)(B.o[A] + la) * B.stride[A] + (long long)(B.o[Bx] + lb) * B.stride[Bx];
  *bcell = tang + (long long)(upper ? B.o[D] + B.e[D] - 1 : B.o[D]) * B.stride[D];
  int g = upper ? B.o[D] + B.e[D] : B.o[D] - 1;
  if (g < 0 || g >= B.nc[D]) {
    if (!args.periodic[D]) return false;
    g = (g + B.nc[D]) % B.nc[D];
  }
  *hcell = tang + (long long)g * B.stride[D];
  return true;
}

// Phase 0 item: the trace of the halo cell's face towards the brick (its
// upper face below the brick, into slot 0; its lower face above, into slot
// e_D).
template <int N, bool KC, int D>
__device__ __forceinline__ void cell_halo_traces(bool upper, int la, int lb, const CellBrick& B,
                                                 const DgArgsT<float>& args, const DgConstTablesT<float>& tabs,
                                                 float* slots) {
  constexpr int N2 = N * N, N3 = N2 * N;
  long long hcell, bcell;
  if (!cell_halo_neighbour<D>(upper, la, lb, B, args, &hcell, &bcell)) return;
  float x[N3], a[N2], b[N2];
  cell_load_dofs<N>(args.u + hcell * N3, x);
  cell_traces<N, KC, D>(x, !upper, tabs, a, b);
  cell_store_slot<N>(slots, cell_slot<N>(D, upper ? B.e[D] : 0, la, lb), a, b);
}

// Phase 2 item: the flux through the brick's lower face at (D, la, lb) from
// the halo cell's upper traces (slot 0) and the brick cell's lower traces
// (its boundary slot), or the domain-boundary terms; into slot 0.
template <int N, bool ADV, bool KC, int D>
__device__ __forceinline__ void cell_lower_flux(int la, int lb, const CellBrick& B, const DgArgsT<float>& args,
                                                const DgConstTablesT<float>& tabs, float* slots) {
  constexpr int N2 = N * N;
  long long hcell, bcell;
  const bool has_nb = cell_halo_neighbour<D>(false, la, lb, B, args, &hcell, &bcell);
  const int s0 = cell_slot<N>(D, 0, la, lb);
  float vo[N2], po[N2], a[N2], b[N2];
  cell_load_slot<N>(slots, cell_bnd_slot<N>(D, la, lb), vo, po);
  const float kb = KC ? __ldg(args.kcell + bcell) : 0.f;
  if (has_nb) {
    float vh[N2], ph[N2];
    cell_load_slot<N>(slots, s0, vh, ph);
    const float kh = KC ? __ldg(args.kcell + hcell) : 0.f;
    cell_interior_flux<N, ADV, KC, D>(vh, ph, vo, po, kh, kb, args, tabs, a, b);
  } else {
    cell_boundary_flux<N, ADV, KC, D>(false, vo, po, kb, args, tabs, a, b);
  }
  cell_store_slot<N>(slots, s0, a, b);
}

// The r-th face on the brick's lower (or upper) boundary: its axis D and
// brick-local coordinates (la, lb); c0, c1 are the counts of the x and y
// faces.
__device__ __forceinline__ int cell_boundary_face(int r, int c0, int c1, const CellBrick& B, int* la, int* lb) {
  if (r < c0) {
    *la = r % B.e[1];
    *lb = r / B.e[1];
    return 0;
  }
  if (r < c0 + c1) {
    r -= c0;
    *la = r % B.e[0];
    *lb = r / B.e[0];
    return 1;
  }
  r -= c0 + c1;
  *la = r % B.e[0];
  *lb = r / B.e[0];
  return 2;
}

template <int N, bool ADV, bool KC>
__global__ void __launch_bounds__(kCellThreads, 3) dg_cell_kernel(const __grid_constant__ DgArgsT<float> args,
                                                                  const __grid_constant__ DgConstTablesT<float> tabs) {
  constexpr int N2 = N * N, N3 = N2 * N;
  using S = CellSlots<N>;
  static_assert(!(KC && ADV), "cellwise kappa without advection");
  extern __shared__ __align__(16) float slots[];
  const int tid = threadIdx.x;
  CellBrick B;
  B.nc[0] = args.nc[0];
  B.nc[1] = args.nc[1];
  B.nc[2] = args.nc[2];
  const int nbx = (B.nc[0] + kCellBX - 1) / kCellBX, nby = (B.nc[1] + kCellBY - 1) / kCellBY;
  const int bidx = blockIdx.x;
  B.o[0] = (bidx % nbx) * kCellBX;
  B.o[1] = ((bidx / nbx) % nby) * kCellBY;
  B.o[2] = (bidx / (nbx * nby)) * kCellBZ;
  B.e[0] = min(kCellBX, B.nc[0] - B.o[0]);
  B.e[1] = min(kCellBY, B.nc[1] - B.o[1]);
  B.e[2] = min(kCellBZ, B.nc[2] - B.o[2]);
  B.stride[0] = 1;
  B.stride[1] = B.nc[0];
  B.stride[2] = (long long)B.nc[0] * B.nc[1];
  const int l[3] = {tid % kCellBX, (tid / kCellBX) % kCellBY, tid / (kCellBX * kCellBY)};
  const bool valid = l[0] < B.e[0] && l[1] < B.e[1] && l[2] < B.e[2];
  const long long cell = (B.o[0] + l[0]) + B.stride[1] * (B.o[1] + l[1]) + B.stride[2] * (B.o[2] + l[2]);
  // faces on the brick's lower (and upper) boundary: c0 normal to x, c1 to
  // y, c2 to z; nb <= 80
  const int c0 = B.e[1] * B.e[2], c1 = B.e[0] * B.e[2], c2 = B.e[0] * B.e[1];
  const int nb = c0 + c1 + c2;

  // ---- 0. own dofs -------------------------------------------------------------
  float u[N3];
  if (valid) {
    cell_load_dofs<N>(args.u + cell * N3, u);
  } else {
#pragma unroll
    for (int q = 0; q < N3; ++q) u[q] = 0.f;
  }

  // ---- 0. halo items: one cell each, lower side then upper side -----------------
  for (int item = tid; item < 2 * nb; item += kCellThreads) {
    const bool upper = item >= nb;
    int la, lb;
    const int D = cell_boundary_face(upper ? item - nb : item, c0, c1, B, &la, &lb);
    if (D == 0) cell_halo_traces<N, KC, 0>(upper, la, lb, B, args, tabs, slots);
    else if (D == 1) cell_halo_traces<N, KC, 1>(upper, la, lb, B, args, tabs, slots);
    else cell_halo_traces<N, KC, 2>(upper, la, lb, B, args, tabs, slots);
  }

  // ---- 1. own lower-face traces --------------------------------------------------
  if (valid) {
    float a[N2], b[N2];
    cell_traces<N, KC, 0>(u, false, tabs, a, b);
    cell_store_slot<N>(slots, l[0] > 0 ? cell_slot<N>(0, l[0], l[1], l[2]) : cell_bnd_slot<N>(0, l[1], l[2]), a, b);
    cell_traces<N, KC, 1>(u, false, tabs, a, b);
    cell_store_slot<N>(slots, l[1] > 0 ? cell_slot<N>(1, l[1], l[0], l[2]) : cell_bnd_slot<N>(1, l[0], l[2]), a, b);
    cell_traces<N, KC, 2>(u, false, tabs, a, b);
    cell_store_slot<N>(slots, l[2] > 0 ? cell_slot<N>(2, l[2], l[0], l[1]) : cell_bnd_slot<N>(2, l[0], l[1]), a, b);
  }
  __syncthreads();

  // ---- 2. fluxes of the upper faces, and of the brick's lower faces ---------------
  const float kc = KC && valid ? __ldg(args.kcell + cell) : 0.f;
  if (valid) {
    auto upper_face = [&](auto dc) {
      constexpr int D = decltype(dc)::value;
      const int la = l[D == 0 ? 1 : 0], lb = l[D == 2 ? 1 : 2];
      const int sl = cell_slot<N>(D, l[D] + 1, la, lb);
      const int cd = B.o[D] + l[D];
      int nd = cd + 1;
      bool has_nb = true;
      if (nd >= B.nc[D]) {
        if (args.periodic[D]) nd = 0;
        else has_nb = false;
      }
      float vo[N2], po[N2], a[N2], b[N2];
      cell_traces<N, KC, D>(u, true, tabs, vo, po);
      if (has_nb) {
        float vn[N2], pn[N2];
        cell_load_slot<N>(slots, sl, vn, pn);
        const float kn = KC ? __ldg(args.kcell + cell + (long long)(nd - cd) * B.stride[D]) : 0.f;
        cell_interior_flux<N, ADV, KC, D>(vo, po, vn, pn, kc, kn, args, tabs, a, b);
      } else {
        cell_boundary_flux<N, ADV, KC, D>(true, vo, po, kc, args, tabs, a, b);
      }
      cell_store_slot<N>(slots, sl, a, b);
    };
    upper_face(std::integral_constant<int, 0>());
    upper_face(std::integral_constant<int, 1>());
    upper_face(std::integral_constant<int, 2>());
  }
  // the lower-boundary faces on the threads that had one halo item in phase 0
  {
    const int first = 2 * nb > kCellThreads ? 2 * nb - kCellThreads : 0;
    for (int r = tid - first; r >= 0 && r < nb; r += kCellThreads) {
      int la, lb;
      const int D = cell_boundary_face(r, c0, c1, B, &la, &lb);
      if (D == 0) cell_lower_flux<N, ADV, KC, 0>(la, lb, B, args, tabs, slots);
      else if (D == 1) cell_lower_flux<N, ADV, KC, 1>(la, lb, B, args, tabs, slots);
      else cell_lower_flux<N, ADV, KC, 2>(la, lb, B, args, tabs, slots);
    }
  }
  __syncthreads();
  if (!valid) return;

  // ---- 3. line operator + face expansion, one pass per axis ----------------------
  float w[N3];
  const bool has_massK = KC && tabs.massK != 0.f;
  const bool has_mass = tabs.M[0][0] != 0.f;
  auto line_pass = [&](auto dc) {
    constexpr int D = decltype(dc)::value;
    const int la = l[D == 0 ? 1 : 0], lb = l[D == 2 ? 1 : 2];
    const int s0 = cell_slot<N>(D, l[D], la, lb);      // lower face
    const int s1 = cell_slot<N>(D, l[D] + 1, la, lb);  // upper face
    const float gscale = KC ? -tabs.A2[D] * kc : 1.f;
#pragma unroll
    for (int q = 0; q < S::H / 4; ++q) {
      const float4 V0 = *cell_chunk<N>(slots, s0, q);
      const float4 G0 = *cell_chunk<N>(slots, s0, S::H / 4 + q);
      const float4 V1 = *cell_chunk<N>(slots, s1, q);
      const float4 G1 = *cell_chunk<N>(slots, s1, S::H / 4 + q);
      const float v0a[4] = {V0.x, V0.y, V0.z, V0.w}, g0a[4] = {G0.x, G0.y, G0.z, G0.w};
      const float v1a[4] = {V1.x, V1.y, V1.z, V1.w}, g1a[4] = {G1.x, G1.y, G1.z, G1.w};
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const int jk = 4 * q + t;
        if (jk >= N2) continue;
        // own view: Val_0 = -slot0, Val_1 = slot1 (G likewise)
        const float vs = v1a[t] - v0a[t], vd = v1a[t] + v0a[t];
        float gs = g1a[t] - g0a[t], gd = g1a[t] + g0a[t];
        if (KC) {
          gs *= gscale;
          gd *= gscale;
        }
        float x[N];
#pragma unroll
        for (int i = 0; i < N; ++i) x[i] = u[cell_line_off<N, D>(jk, i)];
#pragma unroll
        for (int i = 0; i < N; ++i) {
          float& out = w[cell_line_off<N, D>(jk, i)];
          float acc = D == 0 ? 0.f : out;
          if (KC) {
            float tt = 0.f;
#pragma unroll
            for (int jj = 0; jj < N; ++jj)
              if (i != 0 && jj != 0 && !((i + jj) & 1)) tt = fmaf(tabs.M[D][i * N + jj], x[jj], tt);
            acc = fmaf(kc, tt, acc);
            if (D == 0 && has_massK) acc = fmaf(tabs.massK, x[i], acc);
            acc = fmaf(tabs.tr[N + i], (i & 1) ? vd : vs, acc);
            if (i > 0) acc = fmaf(tabs.dtr[N + i], (i & 1) ? gd : gs, acc);
          } else {
#pragma unroll
            for (int jj = 0; jj < N; ++jj) {
              const bool mass00 = D == 0 && i == 0 && jj == 0 && has_mass;
              const bool k1 = i != 0 && jj != 0 && !((i + jj) & 1);
              const bool d1 = jj < i && ((i + jj) & 1);
              if (k1 || mass00 || (ADV && d1)) acc = fmaf(tabs.M[D][i * N + jj], x[jj], acc);
            }
            acc = fmaf(tabs.etr[D][i], (i & 1) ? vd : vs, acc);
            if (i > 0) acc = fmaf(tabs.edtr[D][i], (i & 1) ? gd : gs, acc);
          }
          out = acc;
        }
      }
    }
  };
  line_pass(std::integral_constant<int, 0>());
  line_pass(std::integral_constant<int, 1>());
  line_pass(std::integral_constant<int, 2>());

  // ---- 4. store ------------------------------------------------------------------
  float* dst = args.w + cell * N3;
  if constexpr (N3 % 4 == 0) {
    float4* d4 = reinterpret_cast<float4*>(dst);
#pragma unroll
    for (int q = 0; q < N3 / 4; ++q) __stcs(d4 + q, make_float4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]));
  } else {
#pragma unroll
    for (int q = 0; q < N3; ++q) __stcs(dst + q, w[q]);
  }
}

}  // namespace gbfem
