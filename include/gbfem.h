/*
 * gbfem.h -- C-ABI of the GB300-native matrix-free operator apply and Krylov
 * solve of dune-fem.
 *
 * Every entry point is `extern "C"`, takes opaque handles, plain pointers and
 * sizes, and returns an int status (GBFEM_OK = 0, negative on error; the
 * message is in gbfem_last_error()).  Dof vectors are device pointers unless
 * a function name ends in `_host`.  A `stream` argument is a cudaStream_t
 * passed as void* (NULL = the legacy default stream).
 *
 * Each declaration names the dune-fem interface it replaces (paths are
 * relative to the dune-fem source tree).
 */
#ifndef GBFEM_H
#define GBFEM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define GBFEM_OK 0
#define GBFEM_ERR_INVALID (-1)         /* bad argument: DUNE_THROW(InvalidStateException/RangeError) */
#define GBFEM_ERR_NOT_IMPLEMENTED (-2) /* DUNE_THROW(NotImplemented) */
#define GBFEM_ERR_CUDA (-3)            /* CUDA runtime error (message holds cudaGetErrorString) */
#define GBFEM_ERR_NO_DEVICE (-4)       /* no CUDA device visible */
#define GBFEM_ERR_NONFINITE (-5)       /* NaN/Inf met in a solver (the reference asserts) */

/* precisions of dof vectors and of the arithmetic of an operator */
#define GBFEM_F64 0
#define GBFEM_F32 1
/* block-Jacobi storage only: FP16 inverse blocks scaled by one FP32 factor per
 * block (max |entry|), applied to FP32 vectors (half the FP32 traffic) */
#define GBFEM_F16 2

/* Returns the calling thread's last error message ("" if none). */
const char* gbfem_last_error(void);
/* Library version, major*10000 + minor*100 + patch. */
int gbfem_version(void);

/* ---- device memory (stands in for the DofManager-owned storage of
 *      AdaptiveDiscreteFunction, function/adaptivefunction/adaptivefunction.hh:45-203)
 * ----------------------------------------------------------------------- */
int gbfem_malloc(void** ptr, size_t bytes);
int gbfem_free(void* ptr);
int gbfem_memcpy_h2d(void* dst, const void* src, size_t bytes);
int gbfem_memcpy_d2h(void* dst, const void* src, size_t bytes);
int gbfem_memset(void* ptr, int value, size_t bytes);
int gbfem_synchronize(void);

/* ---- structured Cartesian grid (replaces the YaspGrid leaf grid part the
 *      reference tests build, e.g. solver/test/inverseoperatortest.cc:74) -- */
typedef struct {
  int dim;            /* 2 or 3 */
  int cells[3];       /* cells per direction; cell index = ix + Nx*(iy + Ny*iz) */
  double lower[3];    /* lower-left corner */
  double upper[3];    /* upper-right corner */
  int periodic[3];    /* 1 = periodic in that direction */
} gbfem_grid_desc;

/* ---- DG operator on a Q_p tensor Legendre space --------------------------
 * Replaces GalerkinOperator<DGConservationLawModelIntegrands> for the SIPG
 * diffusion + upwind advection + mass form (schemes/galerkin.hh:1383-1504,
 * schemes/integrands.hh:748-967, UFL form pydemo/advectiondiffusion.py:33-55).
 * Dof layout = the reference's DG block layout (space/discontinuousgalerkin/
 * generic.hh:51-124): dof = cell*(p+1)^d + local, local = i0*(p+1)^2 + i1*(p+1)
 * + i2 with i0 the x-degree (space/shapefunctionset/legendre.hh:168-193).
 * ----------------------------------------------------------------------- */
typedef struct {
  gbfem_grid_desc grid;
  int order;            /* p, 1..4 */
  int quad_points;      /* Gauss points per direction q (volume and faces), p+1..p+3; 0 = p+2 */
  int precision;        /* GBFEM_F64 or GBFEM_F32: dof vectors and arithmetic */
  double diffusion;     /* eps in eps*kappa*grad u.grad v (0 = no diffusion) */
  double penalty;       /* SIPG beta; face weight beta*avg(kappa)/h_F, h_F = avg|K|/|F| */
  double mass;          /* c in c*u*v */
  double velocity[3];   /* constant advection b, upwind flux; all zero = no advection */
  int weak_dirichlet;   /* 1 = Nitsche weak u=0 on non-periodic boundary faces, 0 = do-nothing */
  const void* kappa;    /* device DG coefficients of kappa (same layout/precision) or NULL = 1 */
  int algorithm;        /* GBFEM_ALGO_AUTO, GBFEM_ALGO_QUADRATURE or GBFEM_ALGO_TRACE_PASS (see below) */
  const void* kappa_cell; /* device array of one kappa per cell (same precision), or NULL; excludes
                             kappa and velocity.  A cellwise-constant coefficient: the closed form
                             applies it exactly (as a DG kappa field with only the mean) */
} gbfem_dg_desc;

/* GBFEM_ALGO_AUTO: with kappa == NULL the apply uses the closed form of the
 * same integrals (orthonormal basis, affine cells, exact Gauss quadrature:
 * 1-D stiffness/advection matrices along lines, identity tangential face
 * mass), which equals the quadrature result up to rounding; otherwise the
 * sum-factorised quadrature kernel.  The closed form runs as a trace pass
 * into an operator-owned buffer followed by the apply, except FP32 with
 * p <= 3 over the whole grid, which is one kernel without the buffer.
 * GBFEM_ALGO_QUADRATURE always evaluates at the q^3 volume / q^2 face Gauss
 * points.  GBFEM_ALGO_TRACE_PASS is the closed form always in its trace-pass
 * form. */
#define GBFEM_ALGO_AUTO 0
#define GBFEM_ALGO_QUADRATURE 1
#define GBFEM_ALGO_TRACE_PASS 2

typedef struct gbfem_operator_s* gbfem_operator;

/* Creates the SIPG/upwind DG operator.  ≙ constructing GalerkinOperator +
 * DGConservationLawModelIntegrands (schemes/galerkin.hh:1383-1430). */
int gbfem_dg_operator_create(const gbfem_dg_desc* desc, gbfem_operator* op);
/* A variable kappa is evaluated at the operator's Gauss points once, when the
 * operator is created (kept on the device: q^3 + 6 q^2 values per cell).
 * After changing the contents of the kappa vector, call this to re-evaluate.
 * (The reference's integrands read their coefficient function at every
 * evaluation.)  A Jacobian shares its operator's cache and must not outlive it. */
int gbfem_operator_update_coefficients(gbfem_operator op);
/* Continuous Lagrange Q1 operator for -div(eps grad u) + c u on a 2-D grid
 * with strong Dirichlet rows on the whole boundary: w = A u, w_D = u_D.
 * ≙ DirichletWrapperOperator over GalerkinOperator (schemes/dirichletwrapper.hh:
 * 101-105, schemes/dirichletconstraints.hh:396-430).  Vertex dof numbering
 * = ix + (Nx+1)*iy. */
int gbfem_q1_operator_create(const gbfem_grid_desc* grid, int precision, double diffusion,
                             double mass, gbfem_operator* op);
int gbfem_operator_destroy(gbfem_operator op);
/* Number of dofs of the domain/range space. */
int gbfem_operator_size(gbfem_operator op, int64_t* ndofs);
int gbfem_operator_precision(gbfem_operator op, int* precision);

/* w = op(u).  ≙ Operator<D,R>::operator()(const D& u, R& w) const
 * (operator/common/operator.hh:55); the reference clears w and rebuilds it
 * (schemes/galerkin.hh:1459-1496), as this does.  u and w: device arrays of
 * gbfem_operator_size elements of the operator's precision; must not alias. */
int gbfem_operator_apply(gbfem_operator op, const void* u, void* w, void* stream);
/* Same as gbfem_operator_apply with host arrays: copies u to the device,
 * applies, copies w back, synchronously.  Device buffers are cached in op.
 * DG operators pipeline the call over slabs of z-planes (copy in, trace pass,
 * apply and copy out of successive slabs overlap on four streams; page-locked
 * host arrays let the copies run asynchronously; see also
 * gbfem_operator_set_host_transfer).  For page-locked arrays and a linear
 * operator the pipeline is captured once as a CUDA graph for that pair of
 * arrays and slab count, and replayed while they stay the same (the arrays'
 * contents are read at each call).  The result is bitwise that of
 * gbfem_operator_apply. */
int gbfem_operator_apply_host(gbfem_operator op, const void* u_host, void* w_host);
/* Number of slabs of the pipelined gbfem_operator_apply_host (0 = automatic:
 * up to 16, each >= 8192 cells; capped at the number of z-planes and 64).
 * With three or more z-planes per slab the first two and the last two slabs
 * become single planes (a shorter pipeline fill and drain). */
int gbfem_operator_set_host_chunks(gbfem_operator op, int nchunks);
/* How gbfem_operator_apply_host moves page-locked host buffers of the
 * constant-coefficient DG kernel: 0 (default) = the slab copy pipeline;
 * 1 = the kernels read u and write w in host memory directly over NVLink-C2C
 * (only for buffers cudaPointerGetAttributes reports as page-locked; pageable
 * ones always take the copy pipeline).  On GB300 the copy pipeline is the
 * faster of the two at 8-16 slabs; in place wins without slabs. */
int gbfem_operator_set_host_transfer(gbfem_operator op, int mode);

/* Diagonal of the operator's matrix.  ≙ DifferentiableOperator::jacobian
 * (operator/common/differentiableoperator.hh:54) followed by
 * SparseRowMatrix::extractDiagonal / DiagonalPreconditioner's setup
 * (solver/diagonalpreconditioner.hh:60-99), without assembling the matrix. */
int gbfem_operator_diagonal(gbfem_operator op, void* diag, void* stream);
/* Dense element-diagonal blocks, row-major nloc x nloc per cell
 * (nloc = (p+1)^d).  ≙ jacobian into BlockDiagonalLinearOperator
 * (operator/linear/blockdiagonal.hh:24-135). */
int gbfem_operator_block_diagonal(gbfem_operator op, void* blocks, void* stream);

/* Assembled copy of a DG operator: the full Jacobian in block-sparse-row form
 * (per cell 7 dense nloc x nloc blocks: itself and the six face neighbours),
 * returned as another gbfem_operator whose apply is the block SpMV.
 * ≙ DifferentiableGalerkinOperator::jacobian/assemble into a
 * SparseRowLinearOperator (schemes/galerkin.hh:1548-1643, 1195-1314;
 * operator/linear/spoperator.hh:17-55, operator/matrix/spmatrix.hh:148-180).
 * Memory: ncells * 7 * nloc^2 values. */
int gbfem_operator_assemble(gbfem_operator op, gbfem_operator* assembled);

/* ---- preconditioners ------------------------------------------------------
 * A preconditioner is any map z = P(r) on dof vectors (the reference takes
 * any Operator<D,D>, solver/krylovinverseoperators.hh:36).
 * ----------------------------------------------------------------------- */
typedef struct gbfem_preconditioner_s* gbfem_preconditioner;
/* z = r / diag(A), entries with |diag| < 16 eps set to 1.
 * ≙ DiagonalPreconditioner (solver/diagonalpreconditioner.hh:80-142). */
int gbfem_preconditioner_diagonal_create(gbfem_operator op, gbfem_preconditioner* pc);
/* z_K = (A_KK)^{-1} r_K with the exact element-diagonal blocks of op, inverted
 * by Gauss-Jordan with partial pivoting, stored in `precision` (GBFEM_F16:
 * scaled FP16 blocks for FP32 vectors; the preconditioner's precision is then
 * GBFEM_F32).
 * ≙ BlockDiagonalLinearOperator::invert + multiply
 * (operator/linear/blockdiagonal.hh:102-135).  op must be a DG operator. */
int gbfem_preconditioner_block_jacobi_create(gbfem_operator op, int precision, gbfem_preconditioner* pc);
/* Stationary-iteration preconditioners of an assembled operator (from
 * gbfem_operator_assemble; it must outlive pc): FemPreconditioning with
 * fem.solver.preconditioning.method jacobi / gauss-seidel / sor / ssor
 * (solver/fempreconditioning.hh:59-161, built as in krylovinverseoperators.hh:
 * 226-250), sweeping x_i = w (b_i - sum_{j!=i} a_ij x_j) / a_ii in natural row
 * order (operator/matrix/spmatrix.hh:376-480; SSOR adds the backward sweep),
 * from x = 0, `iterations` times.  The reference's FemPreconditioning
 * constructor drops its n and w arguments (fempreconditioning.hh:184-186), so
 * iterations = 1 and relaxation = 1 reproduce it; Gauss-Seidel always relaxes
 * with 1.  Method ids are the reference's SolverParameter ids. */
#define GBFEM_SMOOTHER_SSOR 2
#define GBFEM_SMOOTHER_SOR 3
#define GBFEM_SMOOTHER_GAUSS_SEIDEL 5
#define GBFEM_SMOOTHER_JACOBI 6
int gbfem_preconditioner_sor_create(gbfem_operator assembled, int method, int iterations, double relaxation,
                                    gbfem_preconditioner* pc);
/* For an FP32 DG operator with kappa_cell (no mass): z_c = H_t^{-1} r_c /
 * kappa_c, H_t the diagonal block of the kappa = 1 operator for the cell's
 * boundary type t (at most 27 inverses kept, instead of one block per cell).
 * It equals block Jacobi where kappa is constant across a cell's faces and
 * approximates it (the penalty's face average) elsewhere.  No counterpart in
 * the reference.  op must outlive pc. */
int gbfem_preconditioner_scaled_block_jacobi_create(gbfem_operator op, gbfem_preconditioner* pc);
/* The same with the engine of the tile product chosen: for blocks of 33 to
 * 128 dofs (p = 3, 4) the cells are cut into tiles of <= 32 cells of one
 * boundary type and each tile is the dense product H_t^{-1} R_tile.
 * GBFEM_SB_ENGINE_TENSOR (the default of the create call above): tcgen05
 * tensor cores, TF32 with the 3xTF32 split (FP32 accuracy), the inverse
 * staged by TMA; GBFEM_SB_ENGINE_FMA: FP32 FMA in registers. */
#define GBFEM_SB_ENGINE_TENSOR 0
#define GBFEM_SB_ENGINE_FMA 1
int gbfem_preconditioner_scaled_block_jacobi_create_engine(gbfem_operator op, int engine, gbfem_preconditioner* pc);
/* Device-side status of a preconditioner's kernels: 0, or 1 if a bounded
 * wait inside the tensor-core kernel gave up (its result is then invalid).
 * Synchronises the device. */
int gbfem_preconditioner_status(gbfem_preconditioner pc, int* status);
int gbfem_preconditioner_apply(gbfem_preconditioner pc, const void* r, void* z, void* stream);
int gbfem_preconditioner_precision(gbfem_preconditioner pc, int* precision);
int gbfem_preconditioner_destroy(gbfem_preconditioner pc);

/* ---- Krylov inverse operators ---------------------------------------------
 * ≙ KrylovInverseOperator::operator()(f,u) -> LinearSolver::cg/gmres/bicgstab
 * (solver/krylovinverseoperators.hh:118-208, solver/linear/cg.hh:18-117,
 * solver/linear/gmres.hh:116-299, solver/linear/bicgstab.hh), plus flexible
 * CG (Notay, SIAM J. Sci. Comput. 22, 2000) and flexible GMRES (Saad, SIAM J.
 * Sci. Comput. 14, 1993), which the reference only has through dune-istl
 * (solver/istl.hh:688-696).  u is the initial guess on entry.
 * ----------------------------------------------------------------------- */
#define GBFEM_SOLVER_CG 0
#define GBFEM_SOLVER_GMRES 1
#define GBFEM_SOLVER_BICGSTAB 2
#define GBFEM_SOLVER_FCG 3
#define GBFEM_SOLVER_FGMRES 4

/* LinearSolver::ToleranceCriteria (solver/parameter.hh:14-17).  As in the
 * reference, preconditioned CG measures the residual in the preconditioner's
 * norm <r, B r> (solver/linear/cg.hh:62-67); GBFEM_TOL_RELATIVE_RESIDUAL (an
 * addition, no counterpart in the reference) makes CG stop on the
 * unpreconditioned ||b - A x|| <= tolerance ||b|| instead (one more dot
 * product per iteration, same iterates; host loop).  The other methods
 * measure the unpreconditioned residual already and treat it as
 * GBFEM_TOL_RELATIVE. */
#define GBFEM_TOL_ABSOLUTE 0
#define GBFEM_TOL_RELATIVE 1
#define GBFEM_TOL_RESIDUAL_REDUCTION 2
#define GBFEM_TOL_RELATIVE_RESIDUAL 3

typedef struct {
  int method;          /* GBFEM_SOLVER_* (fem.solver.method) */
  double tolerance;    /* fem.solver.tolerance */
  int error_measure;   /* GBFEM_TOL_* (fem.solver.errormeasure) */
  int max_iterations;  /* fem.solver.maxiterations */
  int restart;         /* fem.solver.gmres.restart; FCG: directions kept */
  int verbose;         /* print per-iteration residuals to stdout */
  int graph_chunk;     /* CG only: > 0 runs the loop device-resident, chunks of this many
                          iterations captured in a CUDA graph; 0 = host loop.  Same iterates. */
} gbfem_solver_params;

typedef struct {
  int converged;
  int iterations;        /* iterations; negative if not converged (as the reference) */
  double residual;       /* final residual norm in the solver's measure */
  double time_ms;
  int operator_applies;
  int preconditioner_applies;
  int status;            /* GBFEM_OK, GBFEM_ERR_NONFINITE on NaN/Inf */
  int fallbacks;         /* flexible solvers: switches to the fallback preconditioner */
  int outer_iterations;  /* gbfem_solve_mixed: refinement steps / outer Krylov iterations */
  int stagnated;         /* gbfem_solve_mixed: stopped because the true FP64 residual no longer
                            decreased (its rounding floor lies above the tolerance) */
} gbfem_solver_info;

/* Fills the reference's defaults: cg, tolerance 1e-8, absolute, max
 * iterations INT_MAX, restart 20 (solver/parameter.hh:91-201). */
int gbfem_solver_params_default(gbfem_solver_params* prm);
/* u = op^{-1}(f) with optional preconditioner pc (NULL = none).  All vectors
 * in the operator's precision; dot products are summed into FP64 (see gbfem_dot). */
int gbfem_solve(gbfem_operator op, gbfem_preconditioner pc, const gbfem_solver_params* prm, const void* f,
                void* u, gbfem_solver_info* info);

/* Mixed precision: an FP64 outer iteration (residual f - A u, update and
 * convergence test in FP64 with op64) around an FP32 inner Krylov solve with
 * op32 and pc32.  No counterpart in the reference.
 * outer_method 0: iterative refinement, u += ||r|| A32^{-1}(r/||r||).  It
 *   converges while cond(A) times the FP32 rounding of the apply stays well
 *   below 1.
 * outer_method GBFEM_SOLVER_FGMRES or GBFEM_SOLVER_FCG: that flexible FP64
 *   Krylov method (restart outer_restart) with the FP32 inner solve as its
 *   preconditioner, which also converges where refinement stalls.  max_outer
 *   then bounds the outer Krylov iterations.
 * Both stop early, with info->stagnated = 1, when the true relative residual
 * ||f - A u|| / ||f|| fails to drop by 10 % over two refinement steps (or one
 * flexible restart): the FP64 apply's rounding floor is then above the
 * tolerance. */
typedef struct {
  double tolerance;          /* outer relative residual ||f - A u|| / ||f|| */
  int max_outer;             /* refinement steps / outer Krylov iterations */
  gbfem_solver_params inner; /* FP32 inner solve; its tolerance is relative */
  int outer_method;          /* 0 = refinement, GBFEM_SOLVER_FGMRES, GBFEM_SOLVER_FCG */
  int outer_restart;         /* directions kept by the flexible outer method (0 = 20) */
} gbfem_ir_params;
int gbfem_solve_mixed(gbfem_operator op64, gbfem_operator op32, gbfem_preconditioner pc32,
                      const gbfem_ir_params* prm, const void* f, void* u, gbfem_solver_info* info);

/* ---- nonlinear DG operator, Jacobian, Newton ------------------------------
 * S(u) = A u + R(u): the DG operator above plus the volume reaction
 * R(u)_l = int_K r(u_h) phi_l, r(u) = linear u + cubic u^3 + exponential e^u,
 * by the operator's Gauss rule (q points per direction).  ≙ GalerkinOperator
 * over a nonlinear UFL integrand (schemes/galerkin.hh:332-360,1383-1504).
 * gbfem_operator_apply evaluates S; diagonal, block diagonal and assembly are
 * those of the Jacobian. */
typedef struct {
  double linear, cubic, exponential;
} gbfem_reaction;
int gbfem_dg_nonlinear_operator_create(const gbfem_dg_desc* desc, const gbfem_reaction* reaction,
                                       gbfem_operator* op);
/* The same operator with a user-defined pointwise reaction r(u, x, y, z),
 * compiled at run time: cubin_path is an sm_103a cubin holding the kernel
 * gbfem_user_reaction_<f64|f32>_n<p+1>_q<q> for this operator's precision,
 * order and quadrature (the Python package's integrands module generates and
 * compiles it from an expression; r' comes from dual numbers).  ≙ a
 * GalerkinOperator over UFL-generated integrands (python/dune/models/
 * integrands/ufl.py). */
int gbfem_dg_nonlinear_operator_create_jit(const gbfem_dg_desc* desc, const char* cubin_path, gbfem_operator* op);
/* A general DG form compiled at run time: S(u) = sum_K int_K s.v + F:grad v
 * + sum_F int_F (own side) s.v + F:grad v + boundary terms, for `components`
 * (1..4) solution components, with the user's pointwise interior / skeleton /
 * boundary functions of (x, u, grad u) (both sides' traces on a face).
 * cubin_path holds the kernels gbfem_form_<f64|f32>_n<p+1>_q<q>_m<M>_val and
 * _lin (the dual-number linearisation), which the Python package's
 * integrands module generates and compiles.  desc supplies the grid, order,
 * quadrature, precision and penalty (sigma = penalty / h_F is handed to the
 * face functions); its diffusion, mass, velocity and weak_dirichlet fields
 * are not used, kappa and kappa_cell must be NULL.  Dof layout
 * dof = cell * M (p+1)^3 + i * M + m (i the scalar Legendre index, m the
 * component), the reference's vector-valued DG layout
 * (space/basisfunctionset/vectorial.hh:139-165).  The operator is nonlinear:
 * gbfem_operator_jacobian gives S'(u) exactly (forward-mode dual numbers
 * through the same kernel) with apply, diagonal, block diagonal and assembly;
 * Newton, the Krylov solvers, the preconditioners and the explicit
 * Runge-Kutta solver take it like the other DG operators.  ≙ GalerkinOperator
 * over UFL-generated integrands (schemes/galerkin.hh:332-537, 1383-1504,
 * 1548-1643; python/dune/models/integrands/ufl.py:197-348).  A Jacobian must
 * not outlive its form. */
int gbfem_form_operator_create(const gbfem_dg_desc* desc, int components, const char* cubin_path,
                               gbfem_operator* op);
/* Solution components of an operator (1 except for general forms). */
int gbfem_operator_components(gbfem_operator op, int* components);
/* ≙ Operator::nonlinear() (operator/common/operator.hh:64). */
int gbfem_operator_nonlinear(gbfem_operator op, int* nonlinear);
/* A Jacobian operator for op (storage for the linearisation; initially at u = 0
 * for a nonlinear op, the op itself for a linear one).  Destroy it with
 * gbfem_operator_destroy. */
int gbfem_operator_jacobian_create(gbfem_operator op, gbfem_operator* jac);
/* Linearises op at the device vector u into jac: jac = A + R'(u), a linear
 * operator with apply, diagonal, block diagonal and assembly.
 * ≙ DifferentiableOperator::jacobian(u, jOp) (operator/common/
 * differentiableoperator.hh:54; schemes/galerkin.hh:1548-1643, 362-410). */
int gbfem_operator_jacobian(gbfem_operator op, const void* u, gbfem_operator jac, void* stream);

/* Newton's method for S(w) = rhs: NewtonInverseOperator::operator()
 * (solver/newtoninverseoperator.hh:688-790) statement by statement: residual
 * r = S(w) - rhs, Jacobian at w, linear solve J dw = r (Krylov `linear`
 * with the chosen preconditioner of J), w -= dw, new residual, optional
 * line search (:588-630), Eisenstat-Walker forcing of the linear tolerance
 * (:44-81, :559-564), stop when |r| < tolerance or on a failure (:570-586). */
#define GBFEM_PC_NONE 0
#define GBFEM_PC_DIAGONAL 1
#define GBFEM_PC_BLOCK_JACOBI 2
#define GBFEM_LINESEARCH_NONE 0
#define GBFEM_LINESEARCH_SIMPLE 1
#define GBFEM_FORCING_NONE 0
#define GBFEM_FORCING_EISENSTAT_WALKER 1
typedef struct {
  double tolerance;             /* |S(w) - rhs|_2 (dof Euclidean norm) < tolerance; default 1e-6 */
  int max_iterations;           /* default INT_MAX */
  int max_linear_iterations;    /* total over all linear solves; default linear.max_iterations */
  int max_line_search_iterations; /* default INT_MAX */
  int line_search;              /* GBFEM_LINESEARCH_* */
  int forcing;                  /* GBFEM_FORCING_* */
  double eta_max, gamma;        /* Eisenstat-Walker parameters (0.99, 0.1) */
  int simplified;               /* 1: keep the first Jacobian (simplified Newton) */
  int preconditioner;           /* GBFEM_PC_* of each Jacobian */
  int verbose;
  gbfem_solver_params linear;   /* the linear solver (its tolerance is replaced under forcing) */
  int assembled;                /* 1: assemble each Jacobian into the block-sparse matrix
                                   (gbfem_operator_assemble) and solve and precondition with it, as the
                                   reference's Newton does with its sparse-matrix Jacobian; 0 (default):
                                   matrix-free */
} gbfem_newton_params;
/* NewtonFailure (solver/newtoninverseoperator.hh:389-400) */
#define GBFEM_NEWTON_SUCCESS 0
#define GBFEM_NEWTON_INVALID_RESIDUAL 1
#define GBFEM_NEWTON_LINE_SEARCH_FAILED 4
#define GBFEM_NEWTON_TOO_MANY_ITERATIONS 5
#define GBFEM_NEWTON_TOO_MANY_LINEAR_ITERATIONS 6
#define GBFEM_NEWTON_LINEAR_SOLVER_FAILED 7
typedef struct {
  int converged;
  int iterations;          /* Newton iterations */
  int linear_iterations;   /* total; negative if a linear solve failed */
  double residual;         /* final |S(w) - rhs| */
  int failure;             /* GBFEM_NEWTON_* */
  double time_ms;
} gbfem_newton_info;
int gbfem_newton_params_default(gbfem_newton_params* prm);
/* w: initial guess in, solution out (device, op's precision). */
int gbfem_newton_solve(gbfem_operator op, const gbfem_newton_params* prm, const void* rhs, void* w,
                       gbfem_newton_info* info);

/* ---- projection of closed-form functions (coefficient fields, data) ----- */
#define GBFEM_FN_EXP_FOURIER 0 /* exp(sum_k a_k cos(2 pi w_k.x + phi_k)): log-Gaussian random field */
#define GBFEM_FN_GAUSSIAN 1    /* exp(-|x-c|^2/width^2); params = cx, cy, cz, width */
#define GBFEM_FN_CONSTANT 2    /* params[0] */
/* Seeded random Fourier modes of a Gaussian field with squared-exponential
 * correlation: modes[5m..5m+4] = (w_x, w_y, w_z, phi, a), w ~ N(0, (1/(2 pi
 * corr_length))^2 I), phi ~ U[0, 2 pi), a = stddev sqrt(2/nmodes).  Host
 * array.  No counterpart in the reference (benchmark input generator). */
int gbfem_fourier_modes(uint64_t seed, int nmodes, double corr_length, double stddev, double* modes);
/* L2 projection onto the DG Q_order space (same dof layout as the DG
 * operator), q-point Gauss per direction (0 = order+2); scale_by_volume = 1
 * gives the load vector int_K f phi_l instead.  ≙ interpolating / projecting a
 * grid function into a DiscreteFunction (space.interpolate, function/
 * localfunction and operator/projection/l2projection.hh). */
int gbfem_dg_project(const gbfem_grid_desc* grid, int order, int quad_points, int kind, const double* params,
                     const double* modes_host, int nmodes, int scale_by_volume, int precision, void* out,
                     void* stream);

/* ---- local dof orderings --------------------------------------------------
 * The library's local order is the non-hierarchical i0 (p+1)^2 + i1 (p+1) + i2
 * (i0 the x-degree).  The hierarchical LegendreShapeFunctionSet sorts by
 * maximal degree, then lexicographically by (i0, i1, i2)
 * (space/shapefunctionset/legendre.hh:236-249, 294-299; the Python default
 * dglegendre(hierarchical=True)).  perm[h] = the non-hierarchical index of
 * the h-th hierarchical shape function ((order+1)^dim entries). */
int gbfem_legendre_hierarchical_permutation(int order, int dim, int* perm);
/* The cell means of a DG field (the coefficient of the constant basis
 * function, the basis being orthonormal): out[c] = in[c (order+1)^3]. */
int gbfem_dg_cell_means(int precision, int64_t ncells, int order, const void* in, void* out, void* stream);
/* Whole 3-D DG dof vectors between the orderings (device arrays, in != out):
 * to_hierarchical = 1: out[c][h] = in[c][perm[h]]; 0: the inverse. */
int gbfem_dg_permute(int precision, int64_t ncells, int order, int to_hierarchical, const void* in, void* out,
                     void* stream);

/* ---- explicit SSP-RK3 of the method-of-lines DG operator --------------------
 * u' = -M^{-1} A(u), M^{-1} = 1/|K| for the orthonormal basis on affine cells.
 * ≙ ExplicitRungeKuttaSolver with tvd3ButcherTable (solver/rungekutta/
 * explicit.hh:160-215, butchertable.cc:43-52) over MOLGalerkinOperator
 * (schemes/molgalerkin.hh:100-196).
 * ----------------------------------------------------------------------- */
typedef struct gbfem_rk_solver_s* gbfem_rk_solver;
int gbfem_rk3_create(gbfem_operator op, gbfem_rk_solver* rk);
/* One step of size dt, in place on the device vector u (op's precision). */
int gbfem_rk3_step(gbfem_rk_solver rk, void* u, double dt, void* stream);
int gbfem_rk3_destroy(gbfem_rk_solver rk);
/* Time-step information for the explicit method, the operator's counterpart
 * of SpaceOperatorInterface::timeStepEstimate (operator/common/
 * spaceoperatorif.hh:52-124) fed to TimeProvider::provideTimeStepEstimate /
 * provideTimeStepUpperBound (solver/timeprovider.hh:142-155):
 *   dt_estimate    = h_min / (|b| (2p+1)), the advective CFL-1 step (DBL_MAX
 *                    without advection); the time provider scales it by its CFL factor;
 *   dt_upper_bound = 2 / rho(M^{-1} A) from power_iterations steps of the power
 *                    method on the device from a seeded random vector (DBL_MAX
 *                    for 0 iterations): SSP-RK3 is stable on [-2.51, 0]. */
int gbfem_dg_time_step_estimate(gbfem_operator op, int power_iterations, uint64_t seed, double* dt_estimate,
                                double* dt_upper_bound);

/* ---- learned preconditioner ------------------------------------------------
 * A 4-level convolutional network (32 channels, 3x3x3 convolutions, BF16
 * weights/activations, FP32 accumulation) on the cells x cells x cells grid of
 * a DG Q_order space: input the residual's per-cell coefficients (scaled by
 * 1/rms) and log of the cell mean of kappa, output per-cell coefficients.
 * Trained on the GPU by its own forward/backward kernels.  Used as
 * z = BJ(r) + S rms(r) NN(r/rms(r)) inside flexible CG/GMRES, with block
 * Jacobi as the fallback.  No counterpart in the reference (an extension of
 * the path); it plugs in where the reference takes a user preconditioner
 * (solver/preconditionfunctionwrapper.hh:18-47, schemes/femscheme.hh:202-209).
 * ----------------------------------------------------------------------- */
typedef struct gbfem_cnn_s* gbfem_cnn;
/* cells: per direction (cubic grid), a multiple of 8; seeded He initialisation. */
int gbfem_cnn_create(int order, int cells, uint64_t seed, gbfem_cnn* cnn);
int gbfem_cnn_destroy(gbfem_cnn cnn);
/* Sets the log-kappa input channel from DG kappa coefficients (device; NULL = 1). */
int gbfem_cnn_set_kappa(gbfem_cnn cnn, int precision, const void* kappa, void* stream);
/* Coarse mode (1): the network reads only the cell means of r (coefficient 0)
 * and log kappa, and writes only the cell means of z: a learned coarse-grid
 * correction for the two-level form of the learned preconditioner. */
int gbfem_cnn_set_coarse(gbfem_cnn cnn, int coarse);
/* The engine of the 3x3x3 convolutions (forward and backward-data):
 * GBFEM_CNN_CONV_TENSOR_CORE (default) runs them as implicit GEMMs on the
 * tcgen05 tensor cores (TMA tensor loads, BF16 operands, FP32 accumulators
 * in tensor memory) on grid levels with a power-of-two size >= 8, and
 * mma.sync on the others; GBFEM_CNN_CONV_MMA_SYNC on warp-level mma.sync
 * everywhere. */
#define GBFEM_CNN_CONV_TENSOR_CORE 0
#define GBFEM_CNN_CONV_MMA_SYNC 1
int gbfem_cnn_set_conv_engine(gbfem_cnn cnn, int engine);
/* 0, or 1 once a tensor-core convolution gave up on a bounded wait (its
 * output is then incomplete).  Synchronises with the device. */
int gbfem_cnn_status(gbfem_cnn cnn, int* status);
/* Self-test: the float <-> double conversions the elementwise kernels do in
 * integer arithmetic against the hardware's, on n random bit patterns
 * (including values near the binary32 range limits and rounding ties);
 * mismatches is 0 when they agree everywhere. */
int gbfem_selftest_conversions(uint64_t n, uint64_t seed, uint64_t* mismatches);
int gbfem_cnn_set_output_scale(gbfem_cnn cnn, double scale);
int gbfem_cnn_get_output_scale(gbfem_cnn cnn, double* scale);
/* z = S rms(r) NN(r/rms(r)) (accumulate = 1: z += ...). */
int gbfem_cnn_forward(gbfem_cnn cnn, int precision, const void* r, void* z, int accumulate, void* stream);
/* Loss = mean_l (NN(r/rms)_l - target_l/(S rms))^2 and all weight gradients
 * (no update); loss may be NULL (then no synchronisation). */
int gbfem_cnn_loss_grad(gbfem_cnn cnn, int precision, const void* r, const void* target, double* loss,
                        void* stream);
/* loss_grad followed by one Adam step (lr, beta = 0.9/0.999, eps 1e-8). */
int gbfem_cnn_train_step(gbfem_cnn cnn, int precision, const void* r, const void* target, double lr,
                         double* loss, void* stream);
/* One Adam step for a loss L whose gradient with respect to the network's
 * dof-space output z = S rms(r) NN(r/rms(r)) the caller supplies (grad_z, a
 * dof vector), e.g. the A-norm loss (z-e)^T A (z-e) / e^T A e with
 * grad_z = 2 A (z-e) / e^T A e. */
int gbfem_cnn_train_step_grad(gbfem_cnn cnn, int precision, const void* r, const void* grad_z, double lr,
                              void* stream);
int gbfem_cnn_num_params(gbfem_cnn cnn, int64_t* n);
/* Host FP32 copies of weights / gradients, layer by layer, [taps][cout][cin]. */
int gbfem_cnn_get_params(gbfem_cnn cnn, float* host);
int gbfem_cnn_set_params(gbfem_cnn cnn, const float* host);
int gbfem_cnn_get_grads(gbfem_cnn cnn, float* host);
/* Weight file (checkpoint/resume); load rejects files of another shape or
 * with non-finite weights. */
int gbfem_cnn_save(gbfem_cnn cnn, const char* path);
int gbfem_cnn_load(gbfem_cnn cnn, const char* path);
/* op == NULL: additive form z = bj(r) + NN(r).
 * op != NULL: two-level form z = NN(r); z += bj(r - op(z)) (the network as
 * the coarse correction, one block-Jacobi smoothing step; one extra apply).
 * bj is the fallback of flexible solvers.  cnn, bj and op are not owned. */
int gbfem_preconditioner_learned_create(gbfem_cnn cnn, gbfem_preconditioner bj, gbfem_operator op,
                                        gbfem_preconditioner* pc);

/* ---- BLAS-1 on dof vectors (function/common/discretefunction.hh:781-901,
 *      function/common/scalarproducts.hh:101-127).  Reductions are
 *      deterministic: fixed-order two-pass, independent of launch shape. -- */
/* x . y into *result (FP64).  FP64 vectors: FP64 products and sums.  FP32
 * vectors: every product exact (FMA two-product), each thread's share summed
 * in float-float (about 48 significant bits) and the shares in FP64 -- all
 * on the FP32 pipe but for one FP64 add per thread; products keep the FP32
 * exponent range. */
int gbfem_dot(int precision, int64_t n, const void* x, const void* y, double* result, void* stream);
int gbfem_axpy(int precision, int64_t n, double alpha, const void* x, void* y, void* stream);
int gbfem_scal(int precision, int64_t n, double alpha, void* x, void* stream);
int gbfem_copy(int precision, int64_t n, const void* x, void* y, void* stream);
/* y = (precision_y) x : precision conversion between FP64 and FP32 vectors. */
int gbfem_convert(int64_t n, int precision_x, const void* x, int precision_y, void* y, void* stream);

/* Allocation-free dot product.  No counterpart in the reference: it exists
 * for callers that cannot let the library allocate device memory (a host
 * whose memory pool owns all of HBM, or a latency-critical loop that cannot
 * take cudaMalloc's implicit synchronisation).  The deterministic two-pass
 * reduction of gbfem_dot, but its partial sums live
 * in a fixed file-scope device array (65536 partials + a result slot, about
 * 512 KB, held by every GPU that loads the library until exit), so it calls
 * no cudaMalloc/cudaFree.  For n <= 8,388,608 (1024 chunks of 8192) it uses
 * gbfem_dot's partition and returns bitwise the same value; for larger n its
 * chunks stay <= 8192 elements while gbfem_dot's grow, so the two agree to
 * rounding only.  n may be at most 536,870,912 (65536 chunks of 8192); larger
 * n returns GBFEM_ERR_INVALID; n <= 0 writes 0.0.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) with that
 * device current and caches it; make that first call before any stream
 * capture, and do not call it again after a cudaDeviceReset of that device.
 * All calls share the one array: calls that overlap on the GPU (other
 * streams, other host threads) race and must be serialised by the caller.
 * Synchronises `stream` and writes the result to the host double *result. */
int gbfem_dot_noalloc(int precision, int64_t n, const void* x, const void* y, double* result, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GBFEM_H */
