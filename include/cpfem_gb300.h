/*
 * cpfem_gb300 -- C ABI of the GB300 crystal-plasticity FE hot path.
 *
 * Plain pointers and sizes only.  Every entry point returns an int status
 * (CPFEM_OK on success) and, for device work, takes the cudaStream_t it runs on as a
 * void*.  Device pointers are caller-owned; no entry point allocates device memory.
 * On failure cpfem_last_error() returns a message for the calling thread.
 *
 * State arrays are structure-of-arrays, component-major: component c of Gauss point
 * gp sits at ptr[c * num_gp + gp], with gp = cell * 8 + quad.  A 3x3 tensor T has
 * components c = 3*i + j (row-major), a 4th-order dP/dF has c = 9*(3i+J) + (3k+L).
 *
 * Each entry point names the reference code it replaces (paths relative to the
 * reference project root).
 */
#ifndef CPFEM_GB300_H
#define CPFEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CPFEM_ABI_VERSION 1
#define CPFEM_MAX_SLIP 24

enum cpfem_status {
  CPFEM_OK = 0,
  CPFEM_ERR_ARG = 1,     /* bad argument (null pointer, size out of range, ...) */
  CPFEM_ERR_CUDA = 2,    /* a CUDA runtime call failed */
  CPFEM_ERR_SIZE = 3,    /* a size exceeds a documented limit */
  CPFEM_ERR_SOLVE = 4    /* an iterative solve failed (see the info outputs) */
};

/* Per-Gauss-point failure bits, OR-ed into cpfem_gp_args_t.status[0]. */
#define CPFEM_GP_MAXITER   1   /* local Newton hit max_iter (the reference has no cap) */
#define CPFEM_GP_NONFINITE 2   /* non-finite residual or stress */

/*
 * Material constants shared by every Gauss point of a launch.
 * Replaces CrystalPlasticity.custom_init constants
 * (singlecrystal_copper/models_copper.py:52-130) and the hard-coded local-solver
 * settings (models_copper.py:212, :232; crystal_plasticity_OR_design/models_sens_rot.py:211,230).
 * Slip directions/normals are given in the lattice frame and must be normalised.
 */
typedef struct {
  int32_t num_slip;        /* 1..CPFEM_MAX_SLIP (12 FCC/BCC12, 24 BCC24) */
  int32_t qmode;           /* 0: q = r everywhere; 1: q = r with ones on 3-blocks 3*floor(i/3) */
  int32_t max_sub_step;    /* cut-half line-search cap (5, 8 or 10 in the reference) */
  int32_t max_iter;        /* local Newton iteration cap (safety, not in the reference) */
  double local_tol;        /* stop when ||r(S)||_2 <= local_tol (1e-8 or 1e-6) */
  double ao;               /* reference slip rate gamma_dot_0 (1e-3) */
  double C11, C12, C44;    /* cubic elastic constants, lattice frame (MPa) */
  double slip_d[CPFEM_MAX_SLIP][3];
  double slip_n[CPFEM_MAX_SLIP][3];
} cpfem_material_t;

/*
 * Arguments of one constitutive pass over num_gp Gauss points.
 * Kinematics come either from nodal u (u != NULL; needs cells and shape_grads) or from
 * u_grad given per GP (u == NULL).  Rotations and parameters are looked up through
 * per-GP index arrays into small tables (per grain / per instance / per GP).
 * param_table rows are (gss_a, h, t_sat, xm, r), as the internal variables of
 * crystal_plasticity_OR_design/models_sens_rot.py:139.
 * Every output pointer may be NULL.  With weight_jxw != 0, pk1/tangent/stress are
 * multiplied by the GP's JxW.
 */
typedef struct {
  int64_t num_gp;
  int32_t num_cells;
  int32_t weight_jxw;
  double dt;
  const double* u;            /* [3*num_nodes] or NULL */
  const int32_t* cells;       /* [num_cells*8] */
  const double* shape_grads;  /* [num_cells*8*8*3] (cell, quad, node, dim) */
  const double* jxw;          /* [num_cells*8] */
  const double* u_grad;       /* [9*num_gp] when u == NULL */
  const double* fpi;          /* [9*num_gp]  Fp^-1 at the start of the step */
  const double* g;            /* [num_slip*num_gp] slip resistance */
  const double* slip;         /* [num_slip*num_gp] accumulated slip */
  const double* rot_table;    /* [9*n_rot] orthonormal rotations */
  const int32_t* rot_idx;     /* [num_gp] */
  const double* param_table;  /* [5*n_param] */
  const int32_t* param_idx;   /* [num_gp] or NULL (row 0 for every GP) */
  double* pk1;                /* [9*num_gp]  first Piola-Kirchhoff stress P */
  double* tangent;            /* [81*num_gp] dP/dF */
  double* stress;             /* [9*num_gp]  Cauchy stress */
  double* fpi_new;            /* [9*num_gp] */
  double* g_new;              /* [num_slip*num_gp] */
  double* slip_new;           /* [num_slip*num_gp] */
  double* s_out;              /* [9*num_gp] converged second Piola-Kirchhoff S (global frame) */
  int32_t* iters;             /* [num_gp] local Newton iterations */
  int32_t* status;            /* [1] OR of CPFEM_GP_* bits (caller zeroes it) */
} cpfem_gp_args_t;

/* Library identity and error text. */
int cpfem_abi_version(void);
const char* cpfem_last_error(void);

/*
 * Node-block sparsity of a HEX8 mesh (host memory, host work).
 * Replaces the scipy COO->CSR conversion of crystal_plasticity_OR_design/solver.py:279-282
 * (duplicates summed, column indices sorted).  The pattern is stored per node: node a's
 * sorted neighbour list is node_cols[node_rowptr[a] .. node_rowptr[a+1]).  The scalar CSR
 * value of row 3a+i, column 3b+k sits at 9*node_rowptr[a] + i*3*deg(a) + 3*pos(b) + k,
 * which is exactly the position scipy gives it.  elem_pos[e*64 + 8*a + b] = pos of
 * cells[e,b] in the list of cells[e,a].
 */
int cpfem_pattern_count(int32_t num_cells, const int32_t* cells, int32_t num_nodes,
                        int64_t* num_blocks);
int cpfem_pattern_build(int32_t num_cells, const int32_t* cells, int32_t num_nodes,
                        int32_t* node_rowptr, int32_t* node_cols, uint8_t* elem_pos,
                        int32_t* node_tpos);
/* node_tpos (may be NULL): for the block of node a at list position j (neighbour b),
 * the position of a in b's list -- what the transposed SpMV of the adjoint needs. */
/* Scalar CSR arrays (indptr [3n+1], indices [9*num_blocks]) of the pattern, host. */
int cpfem_pattern_expand_csr(int32_t num_nodes, const int32_t* node_rowptr,
                             const int32_t* node_cols, int32_t* indptr, int32_t* indices);

/*
 * Constitutive pass: local Newton on S, stress, consistent tangent, trial state.
 * Replaces the per-GP tensor_map / update_int_vars_map of
 * singlecrystal_copper/models_copper.py:139-271 (newton_solver :204-249, f_jvp :251-259)
 * as evaluated under jax.vmap by JAX-FEM's newton_update, update_int_vars_gp (:273-282)
 * and compute_avg_stress (:297-319).
 */
int cpfem_gp_eval(const cpfem_material_t* mat, const cpfem_gp_args_t* args, void* stream);

/*
 * Element residual and tangent scatter: R_ai += sum_q P_iJ dN_a/dX_J JxW and
 * K_(ai)(bk) += sum_q dN_a/dX_J dP_iJ/dF_kL dN_b/dX_L JxW into the node-block CSR values.
 * pk1_w / tangent_w are the JxW-weighted outputs of cpfem_gp_eval.  Replaces JAX-FEM's
 * newton_update (called at crystal_plasticity_OR_design/solver.py:392): the
 * 'laplace'-kernel residual, its jax.jacfwd element tangent and the COO V array.
 * residual and values are accumulated into; zero them first.
 */
int cpfem_elem_assemble(int32_t num_cells, const int32_t* cells, const double* shape_grads,
                        const int32_t* node_rowptr, const uint8_t* elem_pos,
                        const double* pk1_w, const double* tangent_w,
                        double* residual, double* values, void* stream);

/*
 * Row elimination: residual[d] = u[d] - val for every Dirichlet dof d, and (values != NULL)
 * the matrix row of d becomes the unit row.  Replaces apply_bc_vec
 * (crystal_plasticity_OR_design/solver.py:119-133) and PETSc zeroRows (:290-293).
 * bc_dofs must be unique; where the reference lists a dof twice the later entry wins
 * (solver.py:127-129), and the host wrapper keeps that entry when it builds the list.
 */
int cpfem_apply_dirichlet(int32_t num_bc, const int32_t* bc_dofs, const double* bc_vals,
                          const double* u, double* residual, int32_t num_nodes,
                          const int32_t* node_rowptr, const int32_t* node_cols,
                          double* values, void* stream);

/*
 * Initial Krylov guess of linear_incremental_solver (solver.py:221-227):
 * x0 = 0, x0[d] = val - u[d] on Dirichlet dofs.
 */
int cpfem_bc_initial_guess(int64_t ndof, int32_t num_bc, const int32_t* bc_dofs,
                           const double* bc_vals, const double* u, double* x0, void* stream);

/* JxW-weighted per-cell average of a per-GP 3x3 field (models_copper.py:315). */
int cpfem_cell_average(int32_t num_cells, const double* jxw, const double* field_w,
                       double* out, void* stream);

/* y = y + alpha * x (the Newton update dofs + inc, solver.py:234). */
int cpfem_axpy(int64_t n, double alpha, const double* x, double* y, void* stream);

/* Device dot product x.y into *result (device), deterministic order. */
size_t cpfem_dot_workspace_bytes(int64_t n);
int cpfem_dot(int64_t n, const double* x, const double* y, double* result,
              void* workspace, void* stream);

/*
 * y = A x with A in the node-block CSR layout (scalar CSR values as scipy orders them).
 */
int cpfem_spmv(int32_t num_nodes, const int32_t* node_rowptr, const int32_t* node_cols,
               const double* values, const double* x, double* y, void* stream);
/* y = A^T x (gather form, needs node_tpos from cpfem_pattern_build). */
int cpfem_spmv_t(int32_t num_nodes, const int32_t* node_rowptr, const int32_t* node_cols,
                 const int32_t* node_tpos, const double* values, const double* x, double* y,
                 void* stream);

/*
 * BiCGSTAB with Jacobi (precond=1), 3x3 block-Jacobi (precond=2) or no (0)
 * preconditioner.  Replaces jax_solve (crystal_plasticity_OR_design/solver.py:19-48):
 * same recurrences as jax.scipy.sparse.linalg.bicgstab, stop when
 * ||r||^2 <= max(tol^2 ||b||^2, atol^2).  transpose != 0 solves A^T x = b
 * (the adjoint solve of implicit_vjp, solver.py:844).
 * x holds x0 on entry and the solution on exit.  info[0] = iterations (or the
 * breakdown code -10/-11), info[1] = 1 if converged.  workspace: see
 * cpfem_bicgstab_workspace_bytes.  The call synchronises the stream to read the
 * convergence flag every check_every iterations.
 */
size_t cpfem_bicgstab_workspace_bytes(int32_t num_nodes);
int cpfem_bicgstab(int32_t num_nodes, const int32_t* node_rowptr, const int32_t* node_cols,
                   const int32_t* node_tpos, const double* values, const double* b, double* x,
                   int32_t precond,
                   int32_t transpose, double tol, double atol, int32_t maxiter,
                   int32_t check_every, void* workspace, int32_t* info, void* stream);

/*
 * FP64 FMA throughput probe (measurement only, not on the solve path): launches `blocks`
 * blocks of 256 threads, each running 8 independent FMA chains of `iters` steps; *flops
 * receives the FP64 flop count of the launch (an FMA counts 2).  Time it with events on
 * `stream`.  No reference counterpart: it supplies the roofline denominator of the
 * constitutive kernel, which the measured peaks do not include.
 */
int cpfem_probe_dfma(int64_t iters, int32_t blocks, double* out, double* flops, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* CPFEM_GB300_H */
