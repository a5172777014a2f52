// Host side of the operator handles: creation from the descriptor, the
// 1-D tables, dispatch of apply / diagonal / block-diagonal, and the
// continuous Lagrange Q1 operator of the 2-D Poisson-type problem.
#include <cuda_runtime.h>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "blas.cuh"
#include "dg_kernel.cuh"
#include "gbfem_internal.cuh"
#include "operator_impl.hpp"
#include "tables.hpp"

namespace gbfem {

int dg_launch_f64(const DgArgsT<double>&, const DgTablesT<double>&, int, int, bool, cudaStream_t);
int dg_launch_f32(const DgArgsT<float>&, const DgTablesT<float>&, int, int, bool, cudaStream_t);
int dg_const_launch_f64(const DgArgsT<double>&, const DgConstTablesT<double>&, int, double*, int, cudaStream_t,
                        double* ucopy = nullptr);
int dg_const_launch_f32(const DgArgsT<float>&, const DgConstTablesT<float>&, int, float*, int, cudaStream_t,
                        float* ucopy = nullptr);
int dg_cell_launch_f32(const DgArgsT<float>&, const DgConstTablesT<float>&, int, cudaStream_t);
bool dg_cell_supported(int n);
int dg_kappa_points_f64(const double*, double*, double*, long long, const DgTablesT<double>&, int, int, cudaStream_t);
int dg_kappa_points_f32(const float*, float*, float*, long long, const DgTablesT<float>&, int, int, cudaStream_t);

template <typename T>
__global__ void k_kappa_field(long long ncells, int nloc, const T* __restrict__ kcell, T* __restrict__ field) {
  const long long n = ncells * nloc;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const long long c = e / nloc;
    field[e] = e - c * nloc == 0 ? kcell[c] : T(0);
  }
}

int dg_kappa_cache(gbfem_operator_s* op) {
  if (op->dg.kappa_cell) {
    // the cellwise kappa as a DG field: mean = kappa_c, higher coefficients 0
    const size_t es = op->precision == GBFEM_F64 ? 8 : 4;
    if (!op->kappa_field) {
      GBFEM_CUDA_TRY(cudaMalloc(&op->kappa_field, size_t(op->ndofs) * es));
      op->owns_kfield = true;
    }
    if (op->precision == GBFEM_F64)
      k_kappa_field<double><<<stream_grid(op->ndofs), 256>>>(op->ncells, op->nloc,
                                                             static_cast<const double*>(op->dg.kappa_cell),
                                                             static_cast<double*>(op->kappa_field));
    else
      k_kappa_field<float><<<stream_grid(op->ndofs), 256>>>(op->ncells, op->nloc,
                                                            static_cast<const float*>(op->dg.kappa_cell),
                                                            static_cast<float*>(op->kappa_field));
    GBFEM_CUDA_TRY(cudaGetLastError());
    op->dg.kappa = op->kappa_field;
  }
  if (!op->dg.kappa) return GBFEM_OK;
  const size_t es = op->precision == GBFEM_F64 ? 8 : 4;
  const size_t q2 = size_t(op->q) * op->q;
  if (!op->kq_cache) {
    GBFEM_CUDA_TRY(cudaMalloc(&op->kq_cache, size_t(op->ncells) * q2 * op->q * es));
    op->owns_kcache = true;
    GBFEM_CUDA_TRY(cudaMalloc(&op->kf_cache, size_t(op->ncells) * 6 * q2 * es));
  }
  if (op->precision == GBFEM_F64)
    GBFEM_TRY(dg_kappa_points_f64(static_cast<const double*>(op->dg.kappa), static_cast<double*>(op->kq_cache),
                                  static_cast<double*>(op->kf_cache), op->ncells, op->tab64, op->n, op->q, nullptr));
  else
    GBFEM_TRY(dg_kappa_points_f32(static_cast<const float*>(op->dg.kappa), static_cast<float*>(op->kq_cache),
                                  static_cast<float*>(op->kf_cache), op->ncells, op->tab32, op->n, op->q, nullptr));
  GBFEM_CUDA_TRY(cudaDeviceSynchronize());
  return GBFEM_OK;
}

// Trace buffer of the closed-form kernel: [cell][6 faces][v|P][n^2], allocated
// on the first apply of an operator.
static int trace_buffer(const gbfem_operator_s* op, void** buf) {
  auto* mop = const_cast<gbfem_operator_s*>(op);
  if (!mop->trace_buf) {
    const size_t bytes = size_t(op->ncells) * 12 * op->n * op->n * (op->precision == GBFEM_F64 ? 8 : 4);
    GBFEM_CUDA_TRY(cudaMalloc(&mop->trace_buf, bytes));
  }
  *buf = mop->trace_buf;
  return GBFEM_OK;
}

template <typename T>
static void fill_const_tables(const Tables1D& t, const ConstTables1D& c, DgConstTablesT<T>* out) {
  std::memset(out, 0, sizeof(*out));
  for (int i = 0; i < t.n; ++i)
    for (int j = 0; j < t.n; ++j) {
      out->K1[i * t.n + j] = T(c.K1[i][j]);
      out->D1[i * t.n + j] = T(c.D1[i][j]);
    }
  for (int s = 0; s < 2; ++s)
    for (int i = 0; i < t.n; ++i) {
      out->tr[s * t.n + i] = T(t.tr[s][i]);
      out->dtr[s * t.n + i] = T(t.dtr[s][i]);
    }
}

template <typename T>
static void fill_dg_tables(const Tables1D& t, DgTablesT<T>* out) {
  std::memset(out, 0, sizeof(*out));
  for (int a = 0; a < t.q; ++a)
    for (int i = 0; i < t.n; ++i) out->B[a * t.n + i] = T(t.B[a][i]);
  for (int a = 0; a < t.q; ++a)
    for (int b = 0; b < t.q; ++b) out->Dc[a * t.q + b] = T(t.Dc[a][b]);
  for (int a = 0; a < t.q; ++a) out->w[a] = T(t.wts[a]);
  for (int a = 0; a < t.q; ++a) out->x[a] = T(t.pts[a]);
  for (int s = 0; s < 2; ++s)
    for (int i = 0; i < t.n; ++i) {
      out->tr[s * t.n + i] = T(t.tr[s][i]);
      out->dtr[s * t.n + i] = T(t.dtr[s][i]);
    }
}

template <typename T>
static void fill_dg_args(const gbfem_operator_s* op, DgArgsT<T>* a) {
  std::memset(a, 0, sizeof(*a));
  const gbfem_dg_desc& d = op->dg;
  double h[3], vol = 1.0;
  for (int k = 0; k < 3; ++k) {
    a->nc[k] = d.grid.cells[k];
    a->periodic[k] = d.grid.periodic[k];
    h[k] = (d.grid.upper[k] - d.grid.lower[k]) / d.grid.cells[k];
    vol *= h[k];
  }
  a->ncells = op->ncells;
  a->detK = T(vol);
  for (int k = 0; k < 3; ++k) {
    a->invh[k] = T(1.0 / h[k]);
    const double area = vol / h[k];
    a->faceA[k] = T(area);
    a->sigma[k] = T(d.penalty / (vol / area));  // h_F = avg|K| / |F|
  }
  a->eps = T(d.diffusion);
  a->mass = T(d.mass);
  for (int k = 0; k < 3; ++k) a->b[k] = T(d.velocity[k]);
  a->advect = (d.velocity[0] != 0.0 || d.velocity[1] != 0.0 || d.velocity[2] != 0.0) ? 1 : 0;
  a->weak_dirichlet = d.weak_dirichlet;
  a->kappa = static_cast<const T*>(d.kappa);
  a->kq = static_cast<const T*>(op->kq_cache);
  a->kf = static_cast<const T*>(op->kf_cache);
  a->kcell = static_cast<const T*>(d.kappa_cell);
}

// M_d = eps |K|/h_d^2 K1 - b_d |K|/h_d D1 (+ c |K| I on axis 0), rounded once.
template <typename T>
static void fill_line_operators(const gbfem_operator_s* op, DgConstTablesT<T>* ct) {
  const gbfem_dg_desc& d = op->dg;
  double h[3], vol = 1.0;
  for (int k = 0; k < 3; ++k) {
    h[k] = (d.grid.upper[k] - d.grid.lower[k]) / d.grid.cells[k];
    vol *= h[k];
  }
  const int n = op->n;
  const bool kc = d.kappa_cell != nullptr;  // M: the diffusion part only, scaled per cell in the kernel
  for (int ax = 0; ax < 3; ++ax)
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double m = d.diffusion * vol / (h[ax] * h[ax]) * op->cK1[i * n + j] -
                   d.velocity[ax] * vol / h[ax] * op->cD1[i * n + j];
        if (!kc && ax == 0 && i == j) m += d.mass * vol;
        ct->M[ax][i * n + j] = T(m);
      }
  ct->massK = T(kc ? d.mass * vol : 0.0);
  // Folded flux constants of the closed-form kernel: the second trace P and
  // the expansion factors (kappa per cell: P is the outward normal derivative
  // and the expansion uses L_i(1), L_i'(1) unscaled).  C = A1, or 1 where A1
  // vanishes (no diffusion or no penalty); A1 / C is then the same on every
  // axis.
  const double aC = d.diffusion * d.penalty != 0.0 ? 1.0 : 0.0;
  ct->am1 = T(aC - 1.0);
  ct->am2 = T(aC - 2.0);
  for (int ax = 0; ax < 3; ++ax) {
    const double area = vol / h[ax];
    const double A1 = area * d.diffusion * d.penalty / h[ax];  // sigma = beta / h_F, h_F = |K| / |F| = h
    const double A2 = area * d.diffusion * 0.5 / h[ax];
    ct->A1[ax] = T(A1);
    ct->A2[ax] = T(A2);
    const double C = aC != 0.0 ? A1 : 1.0, r = A2 / C;
    for (int i = 0; i < n; ++i) {
      const double L1 = op->ctab64.tr[n + i], dL1 = op->ctab64.dtr[n + i];
      ct->pc[ax][i] = T(kc ? dL1 : L1 - r * dL1);
      ct->etr[ax][i] = T(C * L1);
      ct->edtr[ax][i] = T(-A2 * dL1);
    }
    for (int side = 0; side < 2; ++side) {
      const double bn = side ? d.velocity[ax] : -d.velocity[ax];
      ct->adv[2 * ax + side] = T(area * bn / C);
    }
  }
}

static int dg_apply_linear(const gbfem_operator_s* op, const void* u, void* w, cudaStream_t s, int unit_mode,
                           void* blocks, long long cell_begin, long long cell_count, int phase, void* ucopy);

int dg_apply(const gbfem_operator_s* op, const void* u, void* w, cudaStream_t s, int unit_mode,
             void* blocks, long long cell_begin, long long cell_count, int phase, void* ucopy) {
  if (op->nonlinear && unit_mode != 0)
    return set_error(GBFEM_ERR_INVALID, "nonlinear operator: diagonal and blocks belong to its Jacobian");
  if (op->form) return form_apply(op, u, w, s, unit_mode, blocks, cell_begin, cell_count);
  GBFEM_TRY(dg_apply_linear(op, u, w, s, unit_mode, blocks, cell_begin, cell_count, phase, ucopy));
  const long long count = cell_count > 0 ? cell_count : op->ncells - cell_begin;
  if (unit_mode == 0 && (phase & 2)) {
    if (op->nonlinear) return reaction_launch(op, 0, u, w, nullptr, cell_begin, count, 0, s);
    if (op->jac_points) return reaction_launch(op, 2, u, w, op->jac_points, cell_begin, count, 0, s);
  } else if (op->jac_points && unit_mode == 1) {
    return reaction_launch(op, 0, nullptr, blocks, op->jac_points, cell_begin, count, 1, s);
  } else if (op->jac_points && unit_mode == 2) {
    return reaction_launch(op, 0, nullptr, blocks, op->jac_points, 0, op->ncells, 2, s);
  }
  return GBFEM_OK;
}

static int dg_apply_linear(const gbfem_operator_s* op, const void* u, void* w, cudaStream_t s, int unit_mode,
                           void* blocks, long long cell_begin, long long cell_count, int phase, void* ucopy) {
  if (op->precision == GBFEM_F64) {
    DgArgsT<double> a;
    fill_dg_args(op, &a);
    a.cell_begin = cell_begin;
    a.cell_count = cell_count;
    a.u = static_cast<const double*>(u);
    a.w = static_cast<double*>(w);
    a.unit_mode = unit_mode;
    a.blocks = static_cast<double*>(blocks);
    if (unit_mode == 0 && op->coefficient_space) {
      DgConstTablesT<double> ct = op->ctab64;
      fill_line_operators(op, &ct);
      void* tb = nullptr;
      GBFEM_TRY(trace_buffer(op, &tb));
      return dg_const_launch_f64(a, ct, op->n, static_cast<double*>(tb), phase, s, static_cast<double*>(ucopy));
    }
    return dg_launch_f64(a, op->tab64, op->n, op->q, op->dg.kappa != nullptr, s);
  } else {
    DgArgsT<float> a;
    fill_dg_args(op, &a);
    a.cell_begin = cell_begin;
    a.cell_count = cell_count;
    a.u = static_cast<const float*>(u);
    a.w = static_cast<float*>(w);
    a.unit_mode = unit_mode;
    a.blocks = static_cast<float*>(blocks);
    if (unit_mode == 0 && op->coefficient_space) {
      DgConstTablesT<float> ct = op->ctab32;
      fill_line_operators(op, &ct);
      // the whole grid in one kernel (no trace buffer) where the cell's dofs
      // and results fit in registers; slabs of the host pipeline and p = 4
      // take the two-kernel form
      if (phase == 3 && cell_begin == 0 && (cell_count == 0 || cell_count == op->ncells) && !ucopy &&
          dg_cell_supported(op->n) && !op->two_kernel_f32)
        return dg_cell_launch_f32(a, ct, op->n, s);
      void* tb = nullptr;
      GBFEM_TRY(trace_buffer(op, &tb));
      return dg_const_launch_f32(a, ct, op->n, static_cast<float*>(tb), phase, s, static_cast<float*>(ucopy));
    }
    return dg_launch_f32(a, op->tab32, op->n, op->q, op->dg.kappa != nullptr, s);
  }
}

// ---- continuous Q1 (2-D) ---------------------------------------------------
// Vertex-owner gather: each thread owns one vertex and sums the rows of the
// element matrices of the (up to) four cells around it.  Dirichlet rows are
// w_D = u_D (g = 0), as DirichletWrapperOperator::operator() produces
// (schemes/dirichletwrapper.hh:101-105, dirichletconstraints.hh:396-430).
template <typename T>
__global__ void q1_apply_kernel(const T* __restrict__ u, T* __restrict__ w, int nx, int ny, Q1Element e,
                                int diag_only) {
  const int vx_n = nx + 1, vy_n = ny + 1;
  const long long nv = (long long)vx_n * vy_n;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nv;
       v += (long long)gridDim.x * blockDim.x) {
    const int vx = int(v % vx_n), vy = int(v / vx_n);
    if (vx == 0 || vy == 0 || vx == nx || vy == ny) {
      w[v] = diag_only ? T(1) : u[v];
      continue;
    }
    double acc = 0.0;
    // cells (vx-1+cx, vy-1+cy), cx,cy in {0,1}; local index of v in that cell = (1-cx) + 2*(1-cy)
#pragma unroll
    for (int cy = 0; cy < 2; ++cy)
#pragma unroll
      for (int cx = 0; cx < 2; ++cx) {
        const int ex = vx - 1 + cx, ey = vy - 1 + cy;
        const int a = (1 - cx) + 2 * (1 - cy);
        if (diag_only) {
          acc += e.K[a * 4 + a];
          continue;
        }
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const int bx = ex + (b & 1), by = ey + (b >> 1);
          acc += e.K[a * 4 + b] * double(u[(long long)by * vx_n + bx]);
        }
      }
    w[v] = T(acc);
  }
}

int q1_apply(const gbfem_operator_s* op, const void* u, void* w, cudaStream_t s, int diag_only) {
  const long long nv = op->ndofs;
  const int threads = 256;
  const int blocks = int((nv + threads - 1) / threads);
  if (op->precision == GBFEM_F64)
    q1_apply_kernel<double><<<blocks, threads, 0, s>>>(static_cast<const double*>(u), static_cast<double*>(w),
                                                        op->grid.cells[0], op->grid.cells[1], op->q1, diag_only);
  else
    q1_apply_kernel<float><<<blocks, threads, 0, s>>>(static_cast<const float*>(u), static_cast<float*>(w),
                                                       op->grid.cells[0], op->grid.cells[1], op->q1, diag_only);
  GBFEM_CUDA_TRY(cudaGetLastError());
  return GBFEM_OK;
}

// Element matrix of eps*grad.grad + c*mass for bilinear Q1 on an hx x hy
// rectangle, 2x2 Gauss (the reference's default interior order 2p = 2,
// schemes/galerkin.hh:131).
static Q1Element make_q1_element(double hx, double hy, double eps, double c) {
  Q1Element e;
  long double p[2], wq[2];
  gauss01(2, p, wq);
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b) {
      long double s = 0.0L;
      for (int qy = 0; qy < 2; ++qy)
        for (int qx = 0; qx < 2; ++qx) {
          auto phi = [&](int k, long double x, long double y, long double* v, long double* dx, long double* dy) {
            const int kx = k & 1, ky = k >> 1;
            long double fx = kx ? x : 1.0L - x, fy = ky ? y : 1.0L - y;
            long double gx = kx ? 1.0L : -1.0L, gy = ky ? 1.0L : -1.0L;
            *v = fx * fy;
            *dx = gx * fy / hx;
            *dy = fx * gy / hy;
          };
          long double va, dxa, dya, vb, dxb, dyb;
          phi(a, p[qx], p[qy], &va, &dxa, &dya);
          phi(b, p[qx], p[qy], &vb, &dxb, &dyb);
          s += wq[qx] * wq[qy] * hx * hy * (eps * (dxa * dxb + dya * dyb) + c * va * vb);
        }
      e.K[a * 4 + b] = double(s);
    }
  return e;
}

}  // namespace gbfem

using namespace gbfem;

static int check_grid(const gbfem_grid_desc* g, int want_dim) {
  if (!g) return set_error(GBFEM_ERR_INVALID, "grid descriptor is null");
  if (g->dim != want_dim) return set_error(GBFEM_ERR_INVALID, "grid dim " + std::to_string(g->dim) +
                                                                  " not supported here (want " +
                                                                  std::to_string(want_dim) + ")");
  for (int k = 0; k < want_dim; ++k) {
    if (g->cells[k] <= 0) return set_error(GBFEM_ERR_INVALID, "grid: cells must be positive");
    if (!(g->upper[k] > g->lower[k])) return set_error(GBFEM_ERR_INVALID, "grid: upper must exceed lower");
  }
  return GBFEM_OK;
}

namespace gbfem {

// Streams and events of the pipelined host-buffer apply.
struct HostPipe {
  cudaStream_t in = nullptr, comp = nullptr, out = nullptr, tr = nullptr;
  cudaEvent_t start = nullptr;
  std::vector<cudaEvent_t> ev_in, ev_comp, ev_tr;
  // the copy pipeline captured as a graph, for one pair of page-locked buffers
  cudaGraphExec_t gexec = nullptr;
  const void* g_u = nullptr;
  void* g_w = nullptr;
  int g_chunks = 0;
  cudaEvent_t join[3] = {nullptr, nullptr, nullptr};
};

static void drop_host_graph(HostPipe* p) {
  if (p && p->gexec) {
    cudaGraphExecDestroy(p->gexec);
    p->gexec = nullptr;
    p->g_u = nullptr;
    p->g_w = nullptr;
    p->g_chunks = 0;
  }
}

void destroy_host_pipe(HostPipe* p) {
  if (!p) return;
  drop_host_graph(p);
  for (cudaEvent_t e : p->join)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : p->ev_in) cudaEventDestroy(e);
  for (cudaEvent_t e : p->ev_comp) cudaEventDestroy(e);
  for (cudaEvent_t e : p->ev_tr) cudaEventDestroy(e);
  if (p->start) cudaEventDestroy(p->start);
  if (p->in) cudaStreamDestroy(p->in);
  if (p->comp) cudaStreamDestroy(p->comp);
  if (p->out) cudaStreamDestroy(p->out);
  if (p->tr) cudaStreamDestroy(p->tr);
  delete p;
}

static int host_pipe(gbfem_operator_s* op, int nchunks, HostPipe** out) {
  if (!op->pipe) {
    // built in full before the operator keeps it
    HostPipe* np = new (std::nothrow) HostPipe();
    if (!np) return set_error(GBFEM_ERR_INVALID, "out of host memory");
    cudaError_t e = cudaStreamCreateWithFlags(&np->in, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&np->comp, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&np->out, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&np->tr, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&np->start, cudaEventDisableTiming);
    for (cudaEvent_t& j : np->join)
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&j, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      destroy_host_pipe(np);
      return set_cuda_error(e, "gbfem_operator_apply_host: streams");
    }
    op->pipe = np;
  }
  HostPipe* p = op->pipe;
  while (int(p->ev_in.size()) < nchunks) {  // the three lists grow together
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    cudaError_t e = cudaSuccess;
    for (cudaEvent_t& x : ev)
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&x, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      for (cudaEvent_t x : ev)
        if (x) cudaEventDestroy(x);
      return set_cuda_error(e, "gbfem_operator_apply_host: events");
    }
    p->ev_in.push_back(ev[0]);
    p->ev_comp.push_back(ev[1]);
    p->ev_tr.push_back(ev[2]);
  }
  *out = p;
  return GBFEM_OK;
}

// Host-buffer apply of a DG operator, pipelined over slabs of whole z-planes
// (a slab is a contiguous range of cells and dofs): the host-to-device copy
// of slab k+1, the trace pass of slab k+1, the apply of slab k and the
// device-to-host copy of slab k-1 run at the same time on four streams.  The
// apply of a slab needs its z-neighbours' data (their traces for the
// closed-form kernel, their dofs for the quadrature kernel), so it is issued
// once the next slab's traces exist (or it has arrived); with periodic z,
// slab 0 also needs the last slab and is applied last.  Each cell is computed
// by the same kernel code as the one-shot apply, so the result is bitwise the
// same.

// The device address of page-locked (registered or cudaHostAlloc'ed) host
// memory, or nullptr for anything else.  Only such memory is ever read or
// written by a kernel.
static void* mapped_device_pointer(const void* host) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost) return nullptr;
  return a.devicePointer;
}

// Host-buffer apply of the closed-form kernel on page-locked buffers: the
// trace pass reads u straight from host memory over NVLink-C2C (and leaves a
// device copy for the main kernel), the main kernel writes w straight to host
// memory.  Slabs of z-planes as in the copy pipeline: traces of slab k on one
// stream, the apply of slab k-1 on another once slab k's traces exist, so the
// C2C reads overlap the FP64 work.  Same kernels and arithmetic as the
// device apply.
static int dg_apply_host_mapped(gbfem_operator_s* op, const void* du, void* dw) {
  const int nz = op->dg.grid.cells[2];
  const long long plane = (long long)op->dg.grid.cells[0] * op->dg.grid.cells[1];
  int nchunks = op->host_chunks;
  if (nchunks <= 0) {
    const long long by_size = op->ncells / 8192;
    nchunks = int(by_size < 16 ? (by_size < 1 ? 1 : by_size) : 16);
  }
  if (nchunks > nz) nchunks = nz;
  if (nchunks > 64) nchunks = 64;
  const int zper = (nz + nchunks - 1) / nchunks;
  nchunks = (nz + zper - 1) / zper;
  HostPipe* p = nullptr;
  GBFEM_TRY(host_pipe(op, nchunks, &p));
  auto first_cell = [&](int k) { return (long long)k * zper * plane; };
  auto cell_count = [&](int k) {
    const long long z1 = (long long)(k + 1) * zper < nz ? (long long)(k + 1) * zper : nz;
    return (z1 - (long long)k * zper) * plane;
  };
  GBFEM_CUDA_TRY(cudaEventRecord(p->start, 0));
  GBFEM_CUDA_TRY(cudaStreamWaitEvent(p->in, p->start, 0));
  GBFEM_CUDA_TRY(cudaStreamWaitEvent(p->comp, p->start, 0));
  for (int k = 0; k < nchunks; ++k) {
    GBFEM_TRY(dg_apply(op, du, nullptr, p->in, 0, nullptr, first_cell(k), cell_count(k), 1, op->host_u));
    GBFEM_CUDA_TRY(cudaEventRecord(p->ev_in[k], p->in));
  }
  const bool defer0 = op->dg.grid.periodic[2] && nchunks > 1;
  auto apply = [&](int j) -> int {
    // slab j reads the traces of slabs j-1, j, j+1 (and wraps with periodic z)
    const int need = j + 1 < nchunks ? j + 1 : nchunks - 1;
    GBFEM_CUDA_TRY(cudaStreamWaitEvent(p->comp, p->ev_in[defer0 && j == 0 ? nchunks - 1 : need], 0));
    return dg_apply(op, op->host_u, dw, p->comp, 0, nullptr, first_cell(j), cell_count(j), 2);
  };
  int rc = GBFEM_OK;
  for (int j = defer0 ? 1 : 0; j < nchunks && rc == GBFEM_OK; ++j) rc = apply(j);
  if (rc == GBFEM_OK && defer0) rc = apply(0);
  const cudaError_t e1 = cudaStreamSynchronize(p->comp);
  const cudaError_t e2 = cudaStreamSynchronize(p->in);
  GBFEM_TRY(rc);
  if (e1 != cudaSuccess) return set_cuda_error(e1, "gbfem_operator_apply_host");
  if (e2 != cudaSuccess) return set_cuda_error(e2, "gbfem_operator_apply_host");
  return GBFEM_OK;
}

// z-plane boundaries of the copy pipeline's slabs: slab k holds the planes
// [zb[k], zb[k+1]).  About nchunks slabs of zper planes; with zper >= 3 the
// first two and the last two slabs are single planes instead.  The first
// apply waits for its upper neighbour slab, so it can then start once two
// planes have arrived, and the last apply and copy-out are one plane each:
// a shorter fill and drain around the same steady state.
static std::vector<int> slab_bounds(int nz, int nchunks) {
  const int zper = (nz + nchunks - 1) / nchunks;
  std::vector<int> zb{0};
  int z = 0;
  if (zper >= 3 && nchunks >= 4) {  // then nz >= 9
    zb.push_back(1);
    zb.push_back(2);
    z = 2;
    while (z < nz - 2) {
      z = z + zper < nz - 2 ? z + zper : nz - 2;
      zb.push_back(z);
    }
    zb.push_back(nz - 1);
    zb.push_back(nz);
  } else {
    while (z < nz) {
      z = z + zper < nz ? z + zper : nz;
      zb.push_back(z);
    }
  }
  return zb;
}

// Enqueues the copy pipeline over the slabs zb after the work already queued
// on `origin`.
static int enqueue_copy_pipeline(gbfem_operator_s* op, HostPipe* p, const void* u_host, void* w_host,
                                 const std::vector<int>& zb, cudaStream_t origin) {
  const size_t es = op->precision == GBFEM_F64 ? 8 : 4;
  const long long plane = (long long)op->dg.grid.cells[0] * op->dg.grid.cells[1];
  const size_t cell_bytes = size_t(op->nloc) * es;
  const int nchunks = int(zb.size()) - 1;
  auto first_cell = [&](int k) { return (long long)zb[k] * plane; };
  auto cell_count = [&](int k) { return (long long)(zb[k + 1] - zb[k]) * plane; };
  GBFEM_CUDA_TRY(cudaEventRecord(p->start, origin));
  GBFEM_CUDA_TRY(cudaStreamWaitEvent(p->in, p->start, 0));
  GBFEM_CUDA_TRY(cudaStreamWaitEvent(p->comp, p->start, 0));
  GBFEM_CUDA_TRY(cudaStreamWaitEvent(p->out, p->start, 0));
  for (int k = 0; k < nchunks; ++k) {
    const size_t off = size_t(first_cell(k)) * cell_bytes;
    GBFEM_CUDA_TRY(cudaMemcpyAsync(static_cast<char*>(op->host_u) + off, static_cast<const char*>(u_host) + off,
                                   size_t(cell_count(k)) * cell_bytes, cudaMemcpyHostToDevice, p->in));
    GBFEM_CUDA_TRY(cudaEventRecord(p->ev_in[k], p->in));
  }
  // The closed form's trace pass of slab k runs on its own stream as soon as
  // slab k has arrived, so it fills the SMs left idle by the tail of the apply
  // of slab k-1 (a slab is only a wave or two of CTAs).  The apply of slab j
  // reads the traces (or, for the quadrature kernel, the dofs) of slabs j-1,
  // j and j+1, so it waits for slab j+1's traces (or arrival).
  const bool traces = op->coefficient_space;
  if (traces) {
    GBFEM_CUDA_TRY(cudaStreamWaitEvent(p->tr, p->start, 0));
    for (int k = 0; k < nchunks; ++k) {
      GBFEM_CUDA_TRY(cudaStreamWaitEvent(p->tr, p->ev_in[k], 0));
      GBFEM_TRY(dg_apply(op, op->host_u, nullptr, p->tr, 0, nullptr, first_cell(k), cell_count(k), 1));
      GBFEM_CUDA_TRY(cudaEventRecord(p->ev_tr[k], p->tr));
    }
  }
  const std::vector<cudaEvent_t>& ready = traces ? p->ev_tr : p->ev_in;
  auto apply = [&](int j) -> int {
    const int need = j + 1 < nchunks ? j + 1 : nchunks - 1;
    GBFEM_CUDA_TRY(cudaStreamWaitEvent(p->comp, ready[need], 0));
    GBFEM_TRY(dg_apply(op, op->host_u, op->host_w, p->comp, 0, nullptr, first_cell(j), cell_count(j), 2));
    GBFEM_CUDA_TRY(cudaEventRecord(p->ev_comp[j], p->comp));
    GBFEM_CUDA_TRY(cudaStreamWaitEvent(p->out, p->ev_comp[j], 0));
    const size_t off = size_t(first_cell(j)) * cell_bytes;
    GBFEM_CUDA_TRY(cudaMemcpyAsync(static_cast<char*>(w_host) + off, static_cast<const char*>(op->host_w) + off,
                                   size_t(cell_count(j)) * cell_bytes, cudaMemcpyDeviceToHost, p->out));
    return GBFEM_OK;
  };
  // with periodic z, slab 0 also reads the last slab: it is applied last
  const bool defer0 = op->dg.grid.periodic[2] && nchunks > 1;
  for (int j = defer0 ? 1 : 0; j < nchunks; ++j) GBFEM_TRY(apply(j));
  if (defer0) {
    GBFEM_CUDA_TRY(cudaStreamWaitEvent(p->comp, ready[nchunks - 1], 0));
    GBFEM_TRY(apply(0));
  }
  return GBFEM_OK;
}

// Captures the copy pipeline for (u_host, w_host, nchunks) into a graph:
// one launch then replaces the ~10 API calls and cross-stream waits per slab.
// Every buffer the graph touches exists before the capture starts.
static int capture_copy_pipeline(gbfem_operator_s* op, HostPipe* p, const void* u_host, void* w_host, int nchunks,
                                 const std::vector<int>& zb) {
  drop_host_graph(p);
  if (op->coefficient_space) {
    void* tb = nullptr;
    GBFEM_TRY(trace_buffer(op, &tb));
  }
  GBFEM_CUDA_TRY(cudaStreamBeginCapture(p->in, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_copy_pipeline(op, p, u_host, w_host, zb, p->in);
  if (rc == GBFEM_OK) {
    // join every forked stream back into the origin
    cudaStream_t forked[3] = {p->comp, p->out, op->coefficient_space ? p->tr : nullptr};
    for (int i = 0; i < 3 && rc == GBFEM_OK; ++i) {
      if (!forked[i]) continue;
      cudaError_t e = cudaEventRecord(p->join[i], forked[i]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(p->in, p->join[i], 0);
      if (e != cudaSuccess) rc = set_cuda_error(e, "gbfem_operator_apply_host: graph capture");
    }
  }
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(p->in, &g);
  if (rc != GBFEM_OK || ce != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    if (rc != GBFEM_OK) return rc;
    return set_cuda_error(ce, "gbfem_operator_apply_host: graph capture");
  }
  cudaGraphExec_t ex = nullptr;
  const cudaError_t ie = cudaGraphInstantiate(&ex, g, 0);
  cudaGraphDestroy(g);
  if (ie != cudaSuccess) return set_cuda_error(ie, "gbfem_operator_apply_host: graph instantiate");
  p->gexec = ex;
  p->g_u = u_host;
  p->g_w = w_host;
  p->g_chunks = nchunks;
  return GBFEM_OK;
}

int dg_apply_host_pipelined(gbfem_operator_s* op, const void* u_host, void* w_host) {
  const bool pinned = mapped_device_pointer(u_host) && mapped_device_pointer(w_host);
  if (op->coefficient_space && op->host_in_place && pinned) {
    void* du = mapped_device_pointer(u_host);
    void* dw = mapped_device_pointer(w_host);
    return dg_apply_host_mapped(op, du, dw);
  }
  const int nz = op->dg.grid.cells[2];
  int nchunks = op->host_chunks;
  if (nchunks <= 0) {
    // about 16 slabs, each large enough to fill the GPU (>= 8192 cells)
    const long long by_size = op->ncells / 8192;
    nchunks = int(by_size < 16 ? (by_size < 1 ? 1 : by_size) : 16);
  }
  if (nchunks > nz) nchunks = nz;
  if (nchunks > 64) nchunks = 64;
  const std::vector<int> zb = slab_bounds(nz, nchunks);
  HostPipe* p = nullptr;
  GBFEM_TRY(host_pipe(op, int(zb.size()) - 1, &p));
  // A graph needs page-locked buffers (asynchronous copies) and kernel
  // arguments that stay valid: the plain linear operators.  The graph is
  // kept for the last pair of buffers (and slab count).
  if (pinned && !op->nonlinear && !op->jac_points) {
    if (!(p->gexec && p->g_u == u_host && p->g_w == w_host && p->g_chunks == nchunks))
      GBFEM_TRY(capture_copy_pipeline(op, p, u_host, w_host, nchunks, zb));
    // on the legacy default stream: after the work already queued there
    GBFEM_CUDA_TRY(cudaGraphLaunch(p->gexec, 0));
    GBFEM_CUDA_TRY(cudaStreamSynchronize(0));
    return GBFEM_OK;
  }
  const int rc = enqueue_copy_pipeline(op, p, u_host, w_host, zb, 0);
  // every slab's copy-out waited on its apply: the out stream ends last
  const cudaError_t e = cudaStreamSynchronize(p->out);
  GBFEM_TRY(rc);
  if (e != cudaSuccess) return set_cuda_error(e, "gbfem_operator_apply_host");
  return GBFEM_OK;
}

}  // namespace gbfem

extern "C" {

int gbfem_dg_operator_create(const gbfem_dg_desc* desc, gbfem_operator* out) {
  if (!desc || !out) return set_error(GBFEM_ERR_INVALID, "gbfem_dg_operator_create: null argument");
  *out = nullptr;
  GBFEM_TRY(check_grid(&desc->grid, 3));
  const int p = desc->order;
  if (p < 1 || p > 4) return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "DG order must be 1..4");
  int q = desc->quad_points == 0 ? p + 2 : desc->quad_points;
  if (q != p + 1 && q != p + 2)
    return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "quad_points must be p+1 or p+2 (or 0 for p+2)");
  if (desc->precision != GBFEM_F64 && desc->precision != GBFEM_F32)
    return set_error(GBFEM_ERR_INVALID, "precision must be GBFEM_F64 or GBFEM_F32");
  if (desc->kappa_cell && desc->kappa)
    return set_error(GBFEM_ERR_INVALID, "give either kappa or kappa_cell, not both");
  if (desc->kappa_cell && (desc->velocity[0] != 0.0 || desc->velocity[1] != 0.0 || desc->velocity[2] != 0.0))
    return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "kappa_cell with advection");
  auto* op = new (std::nothrow) gbfem_operator_s();
  if (!op) return set_error(GBFEM_ERR_INVALID, "out of host memory");
  op->kind = OpKind::DG;
  op->precision = desc->precision;
  op->dg = *desc;
  op->dg.quad_points = q;
  op->grid = desc->grid;
  op->n = p + 1;
  op->q = q;
  op->nloc = op->n * op->n * op->n;
  op->ncells = (long long)desc->grid.cells[0] * desc->grid.cells[1] * desc->grid.cells[2];
  op->ndofs = op->ncells * op->nloc;
  for (int k = 0; k < 3; ++k)
    if (desc->grid.periodic[k] && desc->grid.cells[k] < 2) {
      delete op;
      return set_error(GBFEM_ERR_INVALID, "a periodic direction needs at least 2 cells");
    }
  Tables1D t = make_tables(op->n, q);
  fill_dg_tables(t, &op->tab64);
  fill_dg_tables(t, &op->tab32);
  ConstTables1D ct = make_const_tables(op->n);
  fill_const_tables(t, ct, &op->ctab64);
  fill_const_tables(t, ct, &op->ctab32);
  for (int i = 0; i < op->n; ++i)
    for (int j = 0; j < op->n; ++j) {
      op->cK1[i * op->n + j] = double(ct.K1[i][j]);
      op->cD1[i * op->n + j] = double(ct.D1[i][j]);
    }
  // q >= p+1 always holds here, so the quadrature is exact for constant kappa
  if (desc->algorithm < GBFEM_ALGO_AUTO || desc->algorithm > GBFEM_ALGO_TRACE_PASS) {
    delete op;
    return set_error(GBFEM_ERR_INVALID, "gbfem_dg_operator_create: unknown algorithm");
  }
  op->coefficient_space = desc->kappa == nullptr && desc->algorithm != GBFEM_ALGO_QUADRATURE;
  op->two_kernel_f32 = desc->algorithm == GBFEM_ALGO_TRACE_PASS;
  const int rc = dg_kappa_cache(op);
  if (rc) {
    gbfem_operator_destroy(op);
    return rc;
  }
  *out = op;
  return GBFEM_OK;
}

int gbfem_operator_update_coefficients(gbfem_operator op) {
  if (!op) return set_error(GBFEM_ERR_INVALID, "gbfem_operator_update_coefficients: null argument");
  if (op->kind != OpKind::DG) return GBFEM_OK;
  drop_host_graph(op->pipe);
  return dg_kappa_cache(op);
}

int gbfem_q1_operator_create(const gbfem_grid_desc* grid, int precision, double diffusion, double mass,
                             gbfem_operator* out) {
  if (!out) return set_error(GBFEM_ERR_INVALID, "gbfem_q1_operator_create: null out");
  *out = nullptr;
  GBFEM_TRY(check_grid(grid, 2));
  if (precision != GBFEM_F64 && precision != GBFEM_F32)
    return set_error(GBFEM_ERR_INVALID, "precision must be GBFEM_F64 or GBFEM_F32");
  auto* op = new (std::nothrow) gbfem_operator_s();
  if (!op) return set_error(GBFEM_ERR_INVALID, "out of host memory");
  op->kind = OpKind::Q1;
  op->precision = precision;
  op->grid = *grid;
  op->n = 2;
  op->q = 2;
  op->nloc = 1;
  op->ncells = (long long)grid->cells[0] * grid->cells[1];
  op->ndofs = (long long)(grid->cells[0] + 1) * (grid->cells[1] + 1);
  const double hx = (grid->upper[0] - grid->lower[0]) / grid->cells[0];
  const double hy = (grid->upper[1] - grid->lower[1]) / grid->cells[1];
  op->q1 = make_q1_element(hx, hy, diffusion, mass);
  *out = op;
  return GBFEM_OK;
}

int gbfem_operator_destroy(gbfem_operator op) {
  if (!op) return GBFEM_OK;
  if (op->pipe) destroy_host_pipe(op->pipe);
  if (op->jac_points) cudaFree(op->jac_points);
  if (op->owns_kcache) {
    if (op->kq_cache) cudaFree(op->kq_cache);
    if (op->kf_cache) cudaFree(op->kf_cache);
  }
  if (op->jit_lib) cudaLibraryUnload(static_cast<cudaLibrary_t>(op->jit_lib));
  if (op->owns_form_u0 && op->form_u0) cudaFree(op->form_u0);
  if (op->owns_kfield && op->kappa_field) cudaFree(op->kappa_field);
  if (op->host_u) cudaFree(op->host_u);
  if (op->host_w) cudaFree(op->host_w);
  if (op->bsr_blocks) cudaFree(op->bsr_blocks);
  if (op->trace_buf) cudaFree(op->trace_buf);
  if (op->bsr_col) cudaFree(op->bsr_col);
  delete op;
  return GBFEM_OK;
}

int gbfem_operator_size(gbfem_operator op, int64_t* ndofs) {
  if (!op || !ndofs) return set_error(GBFEM_ERR_INVALID, "gbfem_operator_size: null argument");
  *ndofs = op->ndofs;
  return GBFEM_OK;
}

int gbfem_operator_precision(gbfem_operator op, int* precision) {
  if (!op || !precision) return set_error(GBFEM_ERR_INVALID, "gbfem_operator_precision: null argument");
  *precision = op->precision;
  return GBFEM_OK;
}

int gbfem_operator_apply(gbfem_operator op, const void* u, void* w, void* stream) {
  if (!op || !u || !w) return set_error(GBFEM_ERR_INVALID, "gbfem_operator_apply: null argument");
  if (u == w) return set_error(GBFEM_ERR_INVALID, "gbfem_operator_apply: u and w must not alias");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (op->kind == OpKind::DG) return dg_apply(op, u, w, s, 0, nullptr);
  if (op->kind == OpKind::BSR) return bsr_apply(op, u, w, s, 0);
  return q1_apply(op, u, w, s, 0);
}

int gbfem_operator_apply_host(gbfem_operator op, const void* u_host, void* w_host) {
  if (!op || !u_host || !w_host) return set_error(GBFEM_ERR_INVALID, "gbfem_operator_apply_host: null argument");
  const size_t bytes = size_t(op->ndofs) * (op->precision == GBFEM_F64 ? 8 : 4);
  if (!op->host_u) {
    GBFEM_CUDA_TRY(cudaMalloc(&op->host_u, bytes));
    GBFEM_CUDA_TRY(cudaMalloc(&op->host_w, bytes));
  }
  if (op->kind == OpKind::DG && !op->form) return dg_apply_host_pipelined(op, u_host, w_host);
  GBFEM_CUDA_TRY(cudaMemcpyAsync(op->host_u, u_host, bytes, cudaMemcpyHostToDevice, 0));
  GBFEM_TRY(gbfem_operator_apply(op, op->host_u, op->host_w, nullptr));
  GBFEM_CUDA_TRY(cudaMemcpyAsync(w_host, op->host_w, bytes, cudaMemcpyDeviceToHost, 0));
  GBFEM_CUDA_TRY(cudaStreamSynchronize(0));
  return GBFEM_OK;
}

int gbfem_operator_set_host_transfer(gbfem_operator op, int mode) {
  if (!op || mode < 0 || mode > 1) return set_error(GBFEM_ERR_INVALID, "gbfem_operator_set_host_transfer: invalid argument");
  op->host_in_place = mode;
  return GBFEM_OK;
}

int gbfem_operator_set_host_chunks(gbfem_operator op, int nchunks) {
  if (!op || nchunks < 0) return set_error(GBFEM_ERR_INVALID, "gbfem_operator_set_host_chunks: invalid argument");
  op->host_chunks = nchunks;
  return GBFEM_OK;
}

int gbfem_operator_block_diagonal(gbfem_operator op, void* blocks, void* stream) {
  if (!op || !blocks) return set_error(GBFEM_ERR_INVALID, "gbfem_operator_block_diagonal: null argument");
  if (op->kind == OpKind::BSR) {
    const size_t bsz = size_t(op->nloc) * op->nloc * (op->precision == GBFEM_F64 ? 8 : 4);
    GBFEM_CUDA_TRY(cudaMemcpy2DAsync(blocks, bsz, op->bsr_blocks, 7 * bsz, bsz, size_t(op->ncells),
                                     cudaMemcpyDeviceToDevice, static_cast<cudaStream_t>(stream)));
    return GBFEM_OK;
  }
  if (op->kind != OpKind::DG)
    return set_error(GBFEM_ERR_NOT_IMPLEMENTED, "block diagonal is defined for DG operators only");
  return dg_apply(op, nullptr, nullptr, static_cast<cudaStream_t>(stream), 1, blocks);
}

}  // extern "C"

extern "C" int gbfem_operator_diagonal(gbfem_operator op, void* diag, void* stream) {
  if (!op || !diag) return set_error(GBFEM_ERR_INVALID, "gbfem_operator_diagonal: null argument");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (op->kind == OpKind::DG) return dg_apply(op, nullptr, nullptr, s, 2, diag);
  if (op->kind == OpKind::BSR) return bsr_apply(op, nullptr, diag, s, 1);
  return q1_apply(op, nullptr, diag, s, 1);
}
