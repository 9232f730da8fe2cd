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

#define CPFEM_ABI_VERSION 3
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
#define CPFEM_GP_BOUNDS    4   /* an index read from the inputs was out of range (skipped) */

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
  const double* elastic_table; /* [3*n_param] (C11, C12, C44) per parameter row, or NULL for
                                  the material's constants (per-phase stiffness,
                                  polycrystal_DPsteel/models_DPsteel_inhomo.py:184-186) */
  double* pk1;                /* [9*num_gp]  first Piola-Kirchhoff stress P */
  double* tangent;            /* [81*num_gp] dP/dF */
  double* stress;             /* [9*num_gp]  Cauchy stress */
  double* fpi_new;            /* [9*num_gp] */
  double* g_new;              /* [num_slip*num_gp] */
  double* slip_new;           /* [num_slip*num_gp] */
  double* s_out;              /* [9*num_gp] converged second Piola-Kirchhoff S (global frame) */
  int32_t* iters;             /* [num_gp] local Newton iterations */
  int32_t* status;            /* [1] OR of CPFEM_GP_* bits (caller zeroes it) */
  const int32_t* cell_list;   /* [num_listed] or NULL: with nodal u, evaluate only the 8 GPs
                                 of each listed cell; every output of other GPs is left
                                 untouched (a ragged batch skips its converged instances) */
  int32_t num_listed;
  int32_t local_flags;        /* local Newton options, OR-ed bits:
                                 1 (with s_warm, s_dsdf, s_f): start at the linear prediction
                                   s_warm + ds/dF : (F - s_f) instead of at s_warm;
                                 2: Newton directions from an FP32 Jacobian / LU while the
                                   Jacobian's scale max_a d(dgamma_a)/d(tau_a) C11 <= 1e4
                                   (else FP64); the residual, its stop test and the tangent
                                   stay FP64, so the converged state is the same root;
                                 4: the consistent tangent (dP/dF, and ds/dF for the
                                   prediction) in FP32 under the same scale test (else
                                   FP64): it is only the global Newton's Jacobian, so the
                                   converged solution is unchanged.
                                 0 with s_warm = NULL: the reference's iterates. */
  const int32_t* order;       /* [num_gp] permutation or NULL (no cell list): thread t
                                 evaluates GP order[t].  Ordering GPs by their previous
                                 local-Newton iteration count keeps a warp's lanes busy for
                                 the same number of iterations; results are unchanged. */
  double* s_warm;             /* [6*num_gp] or NULL: lattice-frame S (11,22,33,23,13,12) of the
                                 GP's last converged local solve, read and written.  The
                                 local Newton starts there instead of at S = 0 (the
                                 reference's start), falling back to S = 0 when that start has
                                 not converged after 8 iterations; the result is the root of
                                 the same residual to the same tolerance.  Zeros = S = 0. */
  double* s_dsdf;             /* [54*num_gp] or NULL (with s_warm and s_f): ds/dF of the last
                                 tangent pass, lattice-frame s by F component, entry
                                 (6*kl + k)*num_gp + gp; written by tangent passes */
  double* s_f;                /* [9*num_gp] or NULL (with s_warm and s_dsdf): F at which s_warm
                                 converged, written with it.  The prediction is worth it once
                                 ds/dF is that of a plastic state near the new one (not, for
                                 instance, right after a state commit, when the relaxed
                                 state's near-elastic ds/dF overshoots the flow stress). */
  float* tangent32;           /* [81*num_gp] or NULL: with local_flags bit 4 and tangent == NULL,
                                 dP/dF stored in FP32 (points whose tangent was formed in FP64
                                 are rounded), for cpfem_elem_assemble_ex with k_precision 2;
                                 half the tangent's memory and no conversion in the scatter */
} cpfem_gp_args_t;

/*
 * Arguments of the per-Gauss-point backward pass of one load step (cpfem_gp_vjp).
 * The converged local state is recomputed from the checkpoint (u, Fp^-1, g of the step's
 * start).  Output cotangents: cell_sig_bar [num_cells*9] on the JxW-averaged cell
 * Cauchy stress, fpi_bar [9*G] and g_bar [num_slip*G] on the committed state, and in
 * mode 2 the equilibrium adjoint mu [3*num_nodes] (Dirichlet dofs zeroed), which enters
 * as the P cotangent -JxW grad(mu).  Mode 1 returns the F cotangent f_bar [9*G] (to be
 * gathered into the right-hand side of the transposed solve); mode 2 returns the
 * cotangents of the step's inputs: fpi_bar_old, g_bar_old, theta_bar [5*G] (gss_a, h,
 * t_sat, xm, r) and rot_bar [3*G] (spatial rotation increment, R -> (I + [w]x) R).
 */
typedef struct {
  int64_t num_gp;
  int32_t num_cells;
  int32_t mode;
  double dt;
  int32_t num_nodes;          /* sizes of u/mu, the rotation and parameter tables: every */
  int32_t num_rot;            /* gathered index is checked against them, and an index out */
  int32_t num_param;          /* of range sets CPFEM_GP_BOUNDS instead of being read */
  int32_t pad;
  const double* u;
  const int32_t* cells;
  const double* shape_grads;
  const double* jxw;
  const double* fpi;
  const double* g;
  const double* rot_table;
  const int32_t* rot_idx;
  const double* param_table;
  const int32_t* param_idx;
  const double* elastic_table;
  const double* cell_sig_bar;
  const double* fpi_bar;
  const double* g_bar;
  const double* mu;
  double* f_bar;
  double* fpi_bar_old;
  double* g_bar_old;
  double* theta_bar;
  double* rot_bar;
  int32_t* status;
  const double* s_start;      /* [6*num_gp] or NULL: lattice-frame S the recomputation of the
                                 converged state starts from (the forward's converged S of
                                 this step makes it take no iterations); NULL starts at S = 0 */
} cpfem_vjp_args_t;

/* Library identity and error text. */
int cpfem_abi_version(void);
const char* cpfem_last_error(void);

/*
 * Node-block sparsity of a HEX8 mesh (host memory, host work).
 * Replaces the scipy COO->CSR conversion of crystal_plasticity_OR_design/solver.py:279-282
 * (duplicates summed, column indices sorted).  Node a's sorted neighbour list is
 * node_cols[node_rowptr[a] .. node_rowptr[a+1]); the scalar CSR of the reference has row
 * 3a+i, column 3b+k.  elem_pos[e*64 + 8*a + b] = position of cells[e,b] in the list of
 * cells[e,a].  node_tpos (may be NULL): for list entry j of node a (neighbour b), the
 * position of a in b's list.
 */
int cpfem_pattern_count(int32_t num_cells, const int32_t* cells, int32_t num_nodes,
                        int64_t* num_blocks);
int cpfem_pattern_build(int32_t num_cells, const int32_t* cells, int32_t num_nodes,
                        int32_t* node_rowptr, int32_t* node_cols, uint8_t* elem_pos,
                        int32_t* node_tpos);
/* Scalar CSR arrays (indptr [3n+1], indices [9*num_blocks]) of the pattern, host. */
int cpfem_pattern_expand_csr(int32_t num_nodes, const int32_t* node_rowptr,
                             const int32_t* node_cols, int32_t* indptr, int32_t* indices);

/*
 * Sliced-ELL device layout of the matrix values (groups of 32 consecutive nodes, one
 * thread per node, coalesced across the warp).  Group g holds group_width[g] neighbour
 * slots; slot j of node a (lane a%32 of group a/32) has neighbour cols[group_off[g] + 32j
 * + lane] and the 3x3 block value (row i, column k) at
 *   values[9*group_off[g] + 32*(9j + 3i + k) + lane].
 * Padding slots point at the node itself with zero values.  tpos is the slot of this node
 * in the neighbour's list (the transposed product of the adjoint solve); diag_slot[a] is
 * the slot of a itself.  The values array holds 9*group_off[num_groups] doubles.
 */
typedef struct {
  int32_t num_nodes;
  int32_t num_groups;
  const int64_t* group_off;   /* [num_groups+1] */
  const int32_t* group_width; /* [num_groups]   */
  const int32_t* cols;        /* [group_off[num_groups]] */
  const int32_t* tpos;        /* [group_off[num_groups]] */
  const int32_t* diag_slot;   /* [num_nodes] */
} cpfem_sell_t;

/* Host builders: total slots (= group_off[num_groups]), the layout, and the map from the
 * reference's scalar CSR value order to the sliced-ELL index (map [9*num_blocks]). */
int cpfem_sell_count(int32_t num_nodes, const int32_t* node_rowptr, int64_t* total_slots);
int cpfem_sell_build(int32_t num_nodes, const int32_t* node_rowptr, const int32_t* node_cols,
                     const int32_t* node_tpos, int64_t* group_off, int32_t* group_width,
                     int32_t* cols, int32_t* tpos, int32_t* diag_slot);
int cpfem_sell_csr_map(int32_t num_nodes, const int32_t* node_rowptr, const int64_t* group_off,
                       int64_t* map);

/*
 * Constitutive pass: local Newton on S, stress, consistent tangent, trial state.
 * Replaces the per-GP tensor_map / update_int_vars_map of
 * singlecrystal_copper/models_copper.py:139-271 (newton_solver :204-249, f_jvp :251-259)
 * as evaluated under jax.vmap by JAX-FEM's newton_update, update_int_vars_gp (:273-282)
 * and compute_avg_stress (:297-319).
 */
int cpfem_gp_eval(const cpfem_material_t* mat, const cpfem_gp_args_t* args, void* stream);

/*
 * Backward of the converged local Newton at every GP for one load step: the
 * implicit-function VJP (x_bar = (dy/dx)^T y_bar - (dr/dx)^T J^-T (dy/ds)^T y_bar) of the
 * reference's newton_solver custom_jvp (singlecrystal_copper/models_copper.py:251-259)
 * as jax.grad transposes it inside ad_wrapper/implicit_vjp
 * (crystal_plasticity_OR_design/solver.py:801-874).
 */
int cpfem_gp_vjp(const cpfem_material_t* mat, const cpfem_vjp_args_t* args, void* stream);

/*
 * Element residual and tangent scatter: R_ai += sum_q P_iJ dN_a/dX_J JxW and
 * K_(ai)(bk) += sum_q dN_a/dX_J dP_iJ/dF_kL dN_b/dX_L JxW into the node-block CSR values.
 * pk1_w / tangent_w are the JxW-weighted outputs of cpfem_gp_eval; values use the
 * sliced-ELL layout of cpfem_sell_t.  Replaces JAX-FEM's
 * newton_update (called at crystal_plasticity_OR_design/solver.py:392): the
 * 'laplace'-kernel residual, its jax.jacfwd element tangent and the COO V array.
 * residual and values are accumulated into; zero them first.
 */
int cpfem_elem_assemble(int32_t num_cells, const int32_t* cells, const double* shape_grads,
                        const cpfem_sell_t* sell, const uint8_t* elem_pos,
                        const int32_t* cell_list, int32_t num_listed,
                        const double* pk1_w, const double* tangent_w,
                        double* residual, double* values, void* stream);
/* With cell_list == NULL every cell is scattered with FP64 atomics (summation order not
 * fixed).  With a list of cells that share no node (one colour of cpfem_color_cells) the
 * listed cells add without atomics; calling the colours in order gives a bitwise
 * reproducible assembly. */
/* The same with a choice of precision for the tangent part: k_precision 0, the FP64 tangent
 * and FP64 element stiffness (cpfem_elem_assemble); 1, the FP64 tangent (const double*)
 * with the element stiffness formed in FP32; 2, the FP32 tangent of cpfem_gp_args_t's
 * tangent32 (const float*) with the element stiffness formed in FP32.  The FP32 stiffness
 * is added to the FP64 values: it is for a tangent that only serves as the global Newton's
 * Jacobian, so the FP64 residual and its stop rule decide the converged solution.  The
 * residual is FP64 in every case. */
int cpfem_elem_assemble_ex(int32_t num_cells, const int32_t* cells, const double* shape_grads,
                           const cpfem_sell_t* sell, const uint8_t* elem_pos,
                           const int32_t* cell_list, int32_t num_listed,
                           const double* pk1_w, const void* tangent_w,
                           double* residual, double* values, int32_t k_precision, void* stream);

/* Greedy cell colouring (host): cells of one colour share no node.  color [num_cells]. */
int cpfem_color_cells(int32_t num_cells, const int32_t* cells, int32_t num_nodes, int32_t* color,
                      int32_t* num_colors);

/*
 * Row elimination: residual[d] = u[d] - val for every Dirichlet dof d, and (values != NULL)
 * the matrix row of d becomes the unit row.  Replaces apply_bc_vec
 * (crystal_plasticity_OR_design/solver.py:119-133) and PETSc zeroRows (:290-293).
 * bc_dofs must be unique; where the reference lists a dof twice the later entry wins
 * (solver.py:127-129), and the host wrapper keeps that entry when it builds the list.
 */
int cpfem_apply_dirichlet(int32_t num_bc, const int32_t* bc_dofs, const double* bc_vals,
                          const double* u, double* residual, const cpfem_sell_t* sell,
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

/* Per-segment dot products out[i] = x[off[i]:off[i+1]] . y[off[i]:off[i+1]] (device),
 * e.g. the per-instance residual norms of a ragged batch.  No reference counterpart. */
int cpfem_segmented_dot(int32_t num_segments, const int64_t* offsets, const double* x,
                        const double* y, double* out, void* stream);

/* Device dot product x.y into *result (device), deterministic order. */
size_t cpfem_dot_workspace_bytes(int64_t n);
int cpfem_dot(int64_t n, const double* x, const double* y, double* result,
              void* workspace, void* stream);

/* y = A x (transpose = 0) or y = A^T x (transpose != 0), values in the sliced-ELL layout. */
int cpfem_spmv(const cpfem_sell_t* sell, const double* values, const double* x, double* y,
               int32_t transpose, void* stream);

/*
 * BiCGSTAB with Jacobi (precond=1), 3x3 block-Jacobi (precond=2) or no (0)
 * preconditioner.  Replaces jax_solve (crystal_plasticity_OR_design/solver.py:19-48):
 * the recurrences of jax.scipy.sparse.linalg.bicgstab, stop when
 * ||r||^2 <= max(tol^2 ||b||^2, atol^2), early exit on ||s||, breakdown codes -10/-11.
 * transpose != 0 solves A^T x = b (the adjoint solve of implicit_vjp, solver.py:844).
 * The whole solve is one persistent cooperative launch: every grid-wide wait is bounded
 * and reports CPFEM_ERR_SOLVE instead of hanging.  x holds x0 on entry and the solution
 * on exit; info[0] = iterations (or breakdown code), info[1] = 1 if converged.
 * workspace: cpfem_bicgstab_workspace_bytes(num_nodes) bytes, 256-byte aligned.
 * The call synchronises the stream to read info.
 */
size_t cpfem_bicgstab_workspace_bytes(int32_t num_nodes);
int cpfem_bicgstab(const cpfem_sell_t* sell, const double* values, const double* b, double* x,
                   int32_t precond, int32_t transpose, double tol, double atol, int32_t maxiter,
                   void* workspace, int32_t* info, void* stream);

/*
 * Options of cpfem_bicgstab_ex.  max_restarts = 0 keeps jax's semantics exactly (a
 * breakdown, rho = 0 or alpha/omega = 0, ends the solve with code -10/-11 and the current
 * x).  max_restarts > 0 instead restarts at a breakdown that is not yet converged, from the
 * current x with the true residual as the new shadow vector (rhat = p = r = b - A x), at
 * most that many times; info[0] then counts every iteration.  Near-singular systems (a
 * free rigid rotation under BiCGSTAB, which the reference avoids by switching to UMFPACK,
 * calibration/case4.py) stagnate into exact rho = 0 in FP64; restarting lets the solve
 * reach its tolerance instead of returning an unconverged increment.
 */
/*
 * Geometric multigrid hierarchy of a structured box of nodes (x fastest, the numbering of
 * box meshes and of the reference's Neper voxel meshes), the BiCGSTAB preconditioner
 * precond = 3.  No reference counterpart: the reference preconditions with Jacobi
 * (jax_solve, crystal_plasticity_OR_design/solver.py:32-33) or PETSc's ILU/Jacobi
 * (solver.py:63-88).  One V-cycle of damped 3x3 block-Jacobi smoothing on every level,
 * trilinear prolongation P (zero on Dirichlet dofs of level 0), restriction P^T and
 * Galerkin coarse operators P^T A P rebuilt from the current tangent by cpfem_mg_setup
 * (P is a tensor product, so the product runs as three 1-D coarsening passes).
 * The preconditioner only changes the Krylov iterates: the solve still stops on the
 * same true-residual tolerance.  Level l+1 has (dims[l][d]-1)/2+1 nodes per direction
 * (every dims[l][d]-1 even).  The caller owns every array.
 */
#define CPFEM_MG_MAX_LEVELS 8
typedef struct {
  int32_t num_levels;      /* 2..CPFEM_MG_MAX_LEVELS; level 0 is the system being solved */
  int32_t pre_sweeps;      /* smoothing sweeps before restriction (>= 1; the first from zero) */
  int32_t post_sweeps;     /* smoothing sweeps after prolongation (>= 0) */
  int32_t coarse_sweeps;   /* sweeps on the coarsest level (>= 1) */
  double omega;            /* damping of the block-Jacobi smoother */
  int32_t dims[CPFEM_MG_MAX_LEVELS][3];       /* nodes per direction, x fastest */
  cpfem_sell_t sell[CPFEM_MG_MAX_LEVELS];     /* layout per level (level 0: the system's) */
  double* values[CPFEM_MG_MAX_LEVELS];        /* levels >= 1: coarse operators (cpfem_mg_setup) */
  double* minv[CPFEM_MG_MAX_LEVELS];          /* [9*nodes] inverted 3x3 diagonal blocks (setup) */
  const int8_t* slot[CPFEM_MG_MAX_LEVELS];    /* every level: [27*nodes] slot of each neighbour
                                                 offset (dz+1)*9+(dy+1)*3+(dx+1), -1 if absent */
  double* x[CPFEM_MG_MAX_LEVELS];             /* [3*nodes] work vectors of every level */
  double* t[CPFEM_MG_MAX_LEVELS];
  double* r[CPFEM_MG_MAX_LEVELS];
  double* b[CPFEM_MG_MAX_LEVELS];             /* levels >= 1 */
  const int8_t* free_dof;                     /* [3*nodes of level 0]: 0 on Dirichlet dofs */
  double* scratch[2];                         /* Galerkin product in three 1-D passes: stencils of
                                                 the x-coarsened and xy-coarsened operators, each
                                                 [243*scratch_nodes] */
  int64_t scratch_nodes;                      /* >= max over l of dims_c[0]*dims[l][1]*dims[l][2] */
  int32_t precision;       /* 0: the V-cycle in FP64 on the arrays above; 1: in FP32 on the
                              arrays below (set up from the FP64 operators).  The Krylov
                              iteration stays FP64 either way: with the preconditioner on
                              the right, q = A phat and t = A shat are FP64 products of the
                              actual phat / shat, so r stays the residual of the FP64 system
                              and the stop rule is unchanged; only the iterates differ. */
  int32_t local_nodes;     /* levels >= 2 with at most this many nodes run inside one block
                              (0: 256) */
  float* values32[CPFEM_MG_MAX_LEVELS];       /* precision 1: the operators of levels >= 1 in
                                                 FP32 (setup); level 0 reads the system's FP64
                                                 values, rounded in registers (may be NULL) */
  float* minv32[CPFEM_MG_MAX_LEVELS];         /* precision 1: [9*nodes] */
  float* x32[CPFEM_MG_MAX_LEVELS];            /* precision 1: [3*nodes] work vectors */
  float* t32[CPFEM_MG_MAX_LEVELS];
  float* r32[CPFEM_MG_MAX_LEVELS];            /* levels < num_levels-1 */
  float* b32[CPFEM_MG_MAX_LEVELS];            /* levels >= 1 */
} cpfem_mg_t;

/* Host: sizeof of this header's structs as compiled into the library (0 material, 1 gp
 * args, 2 vjp args, 3 sell, 4 mg hierarchy, 5 krylov opts, 6 solve report; 0 for any other
 * value), so a
 * binding can check its own mirror of each layout. */
size_t cpfem_struct_size(int32_t which);
/* Host: the slot table of one level from its node-block CSR pattern (rows sorted, as
 * cpfem_pattern_build makes them); CPFEM_ERR_ARG if a neighbour is not within one node
 * in every direction (not a structured box). */
int cpfem_mg_slot_table(int32_t num_nodes, const int32_t* dims, const int32_t* node_rowptr,
                        const int32_t* node_cols, int8_t* out);
/* Device: block-Jacobi inverses of level 0 from values0 (the BC-eliminated tangent), the
 * Galerkin coarse operators and their block-Jacobi inverses.  Once per new tangent. */
int cpfem_mg_setup(const cpfem_mg_t* mg, const double* values0, void* stream);

/* What one BiCGSTAB launch reports (cpfem_bicgstab_last_stats_ex returns its values; with
 * cpfem_krylov_opts_t.flags bit 1 it is copied to the caller's memory instead). */
typedef struct {
  int32_t k;              /* iterations, or jax's breakdown code (-10 rho, -11 omega/alpha), or
                             -12 (an FP32 V-cycle whose residual grew by 1e8 or went non-finite) */
  int32_t error;          /* nonzero: a grid barrier gave up waiting; the solve is invalid */
  double rs, atol2;       /* ||r||^2 of the recursion at the end, and the stop threshold
                             max(tol^2 b.b, atol^2): converged when rs <= atol2 */
  double rho, alpha, omega;   /* scalars of the last iteration */
  int32_t restarts, pad;
  double true_rs;         /* ||b - A x||^2 of the returned x (flags bit 0), else -1 */
  double bb;              /* b.b */
} cpfem_solve_report_t;

typedef struct {
  int32_t precond;        /* 0 none, 1 Jacobi (the reference), 2 3x3 block-Jacobi, 3 multigrid */
  int32_t transpose;      /* solve A^T x = b (precond 0..2) */
  int32_t maxiter;
  int32_t max_restarts;
  double tol, atol;
  const cpfem_mg_t* mg;   /* precond 3: a hierarchy set up for this matrix */
  int32_t grid_blocks;    /* blocks of the persistent launch; 0: one per 256 nodes, at most the
                             co-resident limit (larger requests are clamped to it) */
  int32_t flags;          /* bit 0: also form ||b - A x||^2 of the returned x in the same launch
                             (cpfem_bicgstab_last_stats_ex), for the caller's true-residual check;
                             bit 1: deferred report -- the call queues the copy of the launch's
                             report to `report` on the stream and returns without waiting for
                             the solve (info and the last-solve statistics are not updated);
                             the caller reads `report` after its next synchronisation of the
                             stream, and must treat report->error as a failed solve */
  cpfem_solve_report_t* report;   /* flags bit 1: host memory (pinned, for an asynchronous copy) */
} cpfem_krylov_opts_t;
int cpfem_bicgstab_ex(const cpfem_sell_t* sell, const double* values, const double* b, double* x,
                      const cpfem_krylov_opts_t* opts, void* workspace, int32_t* info, void* stream);

/*
 * Allocation-free BiCGSTAB.  No reference counterpart: the reference's jax_solve
 * (crystal_plasticity_OR_design/solver.py:19-48) lets JAX allocate.  Same solver and
 * arguments as cpfem_bicgstab, but the scratch is a fixed device array inside the library
 * (every GPU that loads it keeps CPFEM_NOALLOC_SCRATCH_BYTES until the process exits), for
 * callers that cannot allocate device memory -- host codes that own all device memory
 * through their own pool, or loops that must not allocate.  Limit: num_nodes <=
 * CPFEM_NOALLOC_MAX_NODES, else CPFEM_ERR_SIZE with a message.  The first call on a
 * device resolves the array's device address (cudaGetSymbolAddress); make that first call
 * before any stream capture.  The address is kept per device index and belongs to the
 * device's primary context (the one the CUDA runtime API uses): after cudaDeviceReset, or
 * from a context made current through the driver API, it is stale, and such callers are not
 * supported.  Every call shares the one array, so calls that overlap on the GPU (other
 * streams or threads) race; serialise them.  Calls no cudaMalloc/cudaFree.
 */
#define CPFEM_NOALLOC_MAX_NODES 65536
#define CPFEM_NOALLOC_SCRATCH_BYTES (20u * 1024u * 1024u)
int cpfem_bicgstab_noalloc(const cpfem_sell_t* sell, const double* values, const double* b,
                           double* x, int32_t precond, int32_t transpose, double tol, double atol,
                           int32_t maxiter, int32_t* info, void* stream);

/*
 * Scalars of the last cpfem_bicgstab / _ex / _noalloc call made by this host thread:
 * out[7] = (iterations or breakdown code, final ||r||^2, stop threshold
 * max(tol^2 ||b||^2, atol^2), rho, alpha and omega of the last iteration, restarts).  For logging
 * a solve the way jax's BiCGSTAB state would be inspected (solver.py:34-40 keeps only x).
 */
int cpfem_bicgstab_last_stats(double* out);
/* The same scalars followed by ||b - A x||^2 (-1 unless cpfem_krylov_opts_t.flags bit 0 was
 * set) and b.b: out[0..n) of those 9 values.  The ||Ax - b|| < 0.1 check of jax_solve
 * (crystal_plasticity_OR_design/solver.py:43-46) reads them instead of a separate product. */
int cpfem_bicgstab_last_stats_ex(double* out, int32_t n);

/*
 * Ragged batch of independent systems (block-diagonal A over instances, instance i owning
 * nodes [node_off[i], node_off[i+1])): BiCGSTAB per instance with its own scalars and
 * its own stop test.  Same recurrences and stop rule as cpfem_bicgstab.
 *   node_off [num_instances+1]  HOST array, non-decreasing, within the system;
 *   active   [num_active]       HOST array of distinct instance ids to solve;
 *   weights  [num_active]       HOST work estimate per listed instance (e.g. nodes x the
 *                               previous solve's iterations), or NULL for nodes^(4/3);
 *   info     [2*num_instances]  HOST output, (iterations or breakdown code, converged) of
 *                               every listed instance; other entries are left untouched.
 * One cooperative launch: with no more instances than co-resident blocks, each instance
 * gets a team of blocks sized by its weight (team barriers bounded like the grid barrier);
 * otherwise every block solves whole instances from a queue, heaviest first.  The call
 * synchronises the stream.  CPFEM_ERR_SOLVE if a team barrier timed out.  No reference
 * counterpart: the reference solves one RVE per jax_solve call
 * (crystal_plasticity_OR_design/solver.py:19-48).
 */
size_t cpfem_bicgstab_batched_workspace_bytes(int32_t num_nodes);
int cpfem_bicgstab_batched(const cpfem_sell_t* sell, const double* values, const double* b,
                           double* x, int32_t precond, double tol, double atol, int32_t maxiter,
                           int32_t num_instances, const int32_t* node_off, int32_t num_active,
                           const int32_t* active, const double* weights, void* workspace,
                           int32_t* info, void* stream);

/*
 * FP64 FMA throughput probe (measurement only, not on the solve path): launches `blocks`
 * blocks of 256 threads, each running 8 independent FMA chains of `iters` steps; *flops
 * receives the FP64 flop count of the launch (an FMA counts 2).  Time it with events on
 * `stream`.  No reference counterpart: it supplies the roofline denominator of the
 * constitutive kernel (the measured copy-bandwidth and bf16-GEMM peaks do not cover FP64).
 */
int cpfem_probe_dfma(int64_t iters, int32_t blocks, double* out, double* flops, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* CPFEM_GB300_H */
