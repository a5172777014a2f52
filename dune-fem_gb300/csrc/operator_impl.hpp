// Definition of the opaque operator handle.
#pragma once
#include <cuda_runtime.h>

#include "../../include/gbfem.h"
#include "dg_const_kernel.cuh"
#include "dg_kernel.cuh"

namespace gbfem {

enum class OpKind { DG = 1, Q1 = 2, BSR = 3 };

// Element matrix of the continuous Q1 operator; local vertex k = kx + 2*ky.
struct Q1Element {
  double K[16];
};

// unit_mode 0: w = A u on the cells [cell_begin, cell_begin+cell_count)
// (cell_count 0 = all); 1: diagonal blocks of those cells into blocks; 2: the
// diagonal into blocks.  phase (unit mode 0 of the closed-form kernel): bit 1
// computes the face traces of the cells, bit 2 the apply (which reads the
// traces of the neighbours); the other kernels ignore it.
int dg_apply(const struct ::gbfem_operator_s* op, const void* u, void* w, cudaStream_t s, int unit_mode,
             void* blocks, long long cell_begin = 0, long long cell_count = 0, int phase = 3,
             void* ucopy = nullptr);  // closed form, phase 1: also copy the dofs read to ucopy
int q1_apply(const struct ::gbfem_operator_s* op, const void* u, void* w, cudaStream_t s, int diag_only);
// assembled operator: y = A x (diag_only: the diagonal into y)
int bsr_apply(const struct ::gbfem_operator_s* op, const void* x, void* y, cudaStream_t s, int diag_only);
// reaction term of a nonlinear DG operator / linearised term of a Jacobian
// (reaction_kernel.cuh): mode 0 w += R(u), 1 pts = linearisation at u, 2 w +=
// R'(u0) u; blocks_mode 1/2 add the linearised cell blocks / their diagonal.
int reaction_launch(const struct ::gbfem_operator_s* op, int mode, const void* u, void* w, void* pts,
                    long long cell_begin, long long count, int blocks_mode, cudaStream_t s);
// general form operators (form.cu): unit_mode as dg_apply; a form's Jacobian
// applies S'(u0) in unit mode 0
int form_apply(const struct ::gbfem_operator_s* op, const void* u, void* w, cudaStream_t s, int unit_mode,
               void* blocks, long long cell_begin, long long cell_count);
struct HostPipe;
void destroy_host_pipe(HostPipe* p);
int dg_apply_host_pipelined(struct ::gbfem_operator_s* op, const void* u_host, void* w_host);
// (re)computes kq_cache / kf_cache from the operator's kappa vector
int dg_kappa_cache(struct ::gbfem_operator_s* op);

}  // namespace gbfem

struct gbfem_operator_s {
  gbfem::OpKind kind = gbfem::OpKind::DG;
  int precision = GBFEM_F64;
  gbfem_dg_desc dg{};
  gbfem_grid_desc grid{};
  int n = 0, q = 0, nloc = 0;
  long long ncells = 0, ndofs = 0;
  gbfem::DgTablesT<double> tab64{};
  gbfem::DgTablesT<float> tab32{};
  gbfem::DgConstTablesT<double> ctab64{};
  gbfem::DgConstTablesT<float> ctab32{};
  bool coefficient_space = false;  // constant-coefficient closed form (exact quadrature)
  bool two_kernel_f32 = false;     // FP32 closed form: trace pass + apply even where one kernel applies
  double cK1[gbfem::kDgMaxN * gbfem::kDgMaxN] = {};  // 1-D stiffness int L_i' L_j'
  double cD1[gbfem::kDgMaxN * gbfem::kDgMaxN] = {};  // 1-D advection int L_i' L_j
  gbfem::Q1Element q1{};
  void* bsr_blocks = nullptr;   // assembled: [cell][7][nloc][nloc]
  long long* bsr_col = nullptr; // assembled: [cell][7] column cell (-1 = none)
  void* trace_buf = nullptr;    // closed-form kernel: face traces [cell][6][2][n^2]
  void* host_u = nullptr;  // device staging of gbfem_operator_apply_host
  void* host_w = nullptr;
  int host_chunks = 0;     // z-slab chunks of the pipelined host apply (0 = automatic)
  int host_in_place = 0;   // 1: page-locked host buffers are read / written by the kernels over C2C
  int nonlinear = 0;       // DG: adds the reaction R(u) = int r(u) v (react = c1, c3, ce)
  double react[3] = {0.0, 0.0, 0.0};
  void* jac_points = nullptr;  // Jacobian of a nonlinear DG operator: [cell][q^3] w |K| r'(u0)
  void* kq_cache = nullptr;    // variable kappa at the volume Gauss points [cell][q^3]
  void* kf_cache = nullptr;    // variable kappa at the face Gauss points [cell][6][q^2]
  bool owns_kcache = false;    // false in copies (Jacobian) that share the operator's caches
  void* kappa_field = nullptr; // cellwise kappa as a DG field (the mean only), for the Gauss-point paths
  bool owns_kfield = false;
  void* jit_lib = nullptr;     // run-time compiled reaction (cudaLibrary_t), owned by the operator
  void* jit_kernel = nullptr;  // its kernel (cudaKernel_t): modes 0 and 1 of the reaction
  // run-time compiled general form (form.cu): kind DG, nonlinear, M components
  int form = 0;
  int form_m = 1;
  void* form_val = nullptr;    // cudaKernel_t: w = S(u)
  void* form_lin = nullptr;    // cudaKernel_t: the dual-number linearisation (Jacobian modes)
  int form_jacobian = 0;       // this operator is S'(form_u0) of a form
  void* form_u0 = nullptr;     // its linearisation point (owned by the Jacobian)
  bool owns_form_u0 = false;
  gbfem::HostPipe* pipe = nullptr;  // its streams and events
};
