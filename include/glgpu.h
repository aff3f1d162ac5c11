/*
 * glgpu.h — C ABI of the GB300 (sm_103a) implementation of femgl's Newton hot path.
 *
 * The reference keeps this path in private members of FemGL_mpi::FemGL<3>
 * (reference femgl/inc/femgl.h:130-137): assemble_system(), compute_residual(),
 * solve(const double&), newton_iteration(), driven by run().  Their state lives in
 * class members (local_solution, locally_relevant_newton_solution,
 * locally_relevant_damped_vector, system_matrix, system_rhs, residual_vector and
 * the two AffineConstraints, femgl.h:304-316).  Here that state lives in an opaque
 * context that owns all device memory and one CUDA stream; every entry point below
 * replaces one reference member (cited beside it).
 *
 * Conventions
 *   - Plain C types only; every array argument is HOST memory, copied in or out.
 *   - Every function returns a glgpu_status; nothing aborts, traps or exits.
 *     glgpu_last_error() gives a one-line message for the last failure.
 *   - One context per host thread.  A context may hold several independent
 *     instances (meshes with their own coefficients), solved together; the
 *     single-mesh calls are the 1-instance case.
 *   - Vectors are node-major: x[18*node + c] (3D) or x[2*node + c] (2D), the
 *     component packing of femgl/src/s_vector2matrix.cc:159-160 (c < 9: u(c/3,c%3);
 *     c >= 9: v((c-9)/3,(c-9)%3)).  Instances are concatenated in creation order.
 *   - Sign convention of the reference: system_rhs = -R (femgl/src/assemble.cc:257).
 */
#ifndef GLGPU_H
#define GLGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum
{
  GLGPU_OK = 0,
  GLGPU_ERR_ARG = 1,          /* invalid argument or mesh */
  GLGPU_ERR_CUDA = 2,         /* a CUDA call failed; the context should be destroyed */
  GLGPU_ERR_NOMEM = 3,        /* device allocation failed */
  GLGPU_ERR_NOT_CONVERGED = 4, /* linear or nonlinear solve stopped before its tolerance */
  GLGPU_ERR_NAN = 5,          /* NaN or Inf in a residual or a norm */
  GLGPU_ERR_TIMEOUT = 6,      /* a bounded device-side wait gave up */
  GLGPU_ERR_STATE = 7         /* call out of order (e.g. solve before assemble) */
} glgpu_status;

typedef enum
{
  GLGPU_FP64 = 0,  /* assembly, Krylov solve and residual in FP64 (the reference's arithmetic) */
  GLGPU_MIXED = 1  /* FP32 Jacobian + FP32 GMRES; FP64 residual, line search and free energy */
} glgpu_precision;

typedef enum
{
  GLGPU_PC_NONE = 0,
  GLGPU_PC_BLOCK_JACOBI = 1,   /* inverse of each node's diagonal block */
  GLGPU_PC_CHEBYSHEV = 2,      /* Chebyshev polynomial in (block-Jacobi)^-1 J */
  GLGPU_PC_MULTIGRID = 3       /* geometric V-cycle (box meshes, uniform or once-refined; others fall back
                                  to block-Jacobi), flexible GMRES outside */
} glgpu_precond;

/*
 * Mesh of one instance, in the form the reference's setup_system() produces it
 * (femgl/src/setup_uniform_B-phase.cc:125-198): nodes, Q1 cells, the zero-Dirichlet
 * component mask of every node and the hanging-node constraints.
 */
typedef struct
{
  int dim;                       /* 3: femgl tensor GL (18 components); 2: complexGL (2 components) */
  int n_nodes;
  int n_cells;
  const double *xyz;             /* [n_nodes][dim] coordinates */
  const int32_t *cells;          /* [n_cells][2^dim] deal.II vertex order v = ix + 2 iy (+ 4 iz); axis-aligned boxes */
  const uint32_t *dirichlet_mask;/* [n_nodes]: bit c set <=> component c is a zero-Dirichlet dof (may be NULL) */
  const int32_t *hang_ptr;       /* [n_nodes+1] CSR of hanging constraints, or NULL for none */
  const int32_t *hang_parent;    /* parents of hanging nodes */
  const double *hang_weight;     /* their weights (1/2 edge, 1/4 face) */
} glgpu_mesh;

/*
 * Coefficients and solver controls of one instance.
 * Physics (femgl/src/assemble.cc:229-252; femgl/inc/femgl.h:320-322):
 *   J_ij += [K1 k1 + (K2+K3) k23 + alpha a + 2 sum_t beta_t b_t] JxW.
 * For dim == 2 (complexGL archive, complexGL.cc:479-548): K1 is the gradient
 * weight K (the residual uses K/2 |grad psi|^2 ... see glgpu_free_energy),
 * alpha and beta[0] are the bulk coefficients, the rest is unused.
 */
typedef struct
{
  double K1, K2, K3;
  double alpha;
  double beta[5];
  int precision;        /* glgpu_precision */
  int precond;          /* glgpu_precond */
  int cheb_degree;      /* Chebyshev degree (precond == GLGPU_PC_CHEBYSHEV), e.g. 3 */
  int gmres_restart;    /* Krylov basis size before restart, e.g. 50 */
  int gmres_max_iter;   /* "maximum linear iteration number" (declare.cc), e.g. 10000 */
  double ls_step;       /* "primary step length of dampped newton iteration", 0.83 */
  int ls_max_trials;    /* trials of the backtracking line search, 100 (iteration.cc:170) */
  int damped;           /* "Using dampped Newton iteration" (1) or full Newton (0) */
  int mg_pre, mg_post;  /* multigrid: l1 block-Jacobi sweeps before / after the coarse correction (1, 1) */
  double mg_omega;      /* multigrid: damping of the l1 block-Jacobi smoother (default 1) */
  int mf_cells;         /* cells per CTA of the matrix-free FP32 operator: 4, 8 (default) or 16 */
  double prec_reuse;    /* mixed multigrid: keep the previous Newton step's preconditioner (and skip
                           re-assembling the block matrix, rebuilt on demand) while the last step
                           |a delta| / |x| < prec_reuse; 0 (default) rebuilds every step */
  double bt;            /* "AdGR diffuse length" (declare.cc:123, femgl.cc:150): bt < 1e10 adds the
                           Robin term (K1/bt) int |A_t|^2 dS of the pair-breaking faces
                           (assemble.cc:286-348, residual.cc:235-278), A_t = A with the face's
                           normal column zeroed; default 1e10 (no Robin term); must be > 0 */
  double mg_coarse_shift; /* multigrid: the coarsest level is solved with the dense inverse of
                           A + mg_coarse_shift * mean|diag A| * 1 (default 1e-4).  The shift bounds
                           the amplification of the near-null modes (global phase and spin
                           rotations are exact symmetries of the functional); must be > 0 */
  int mg_small_fuse;    /* multigrid, how the small coarse levels run.  0 (default): one launch per
                           sweep, residual and transfer.  1: the levels of at most 20,000 nodes (all
                           instances together), down to the dense coarsest solve, as one cooperative
                           launch per V-cycle whose CTAs walk the levels phase by phase with
                           grid-wide barriers (bounded waits: GLGPU_ERR_TIMEOUT if one gives up).
                           2: the levels of at most 160 nodes per instance and the dense solve as one
                           launch of one thread-block cluster per instance (hardware cluster barriers
                           between phases); contexts with too many instances for clusters of at least
                           4 CTAs keep separate launches */
} glgpu_params;

typedef struct glgpu_ctx glgpu_ctx;

/* Fills p with the reference's defaults (declare.cc) and K1 = K2 = K3 = 0.42072. */
void glgpu_default_params(glgpu_params *p);

/* Library version string. */
const char *glgpu_version(void);

/* Last error message of this thread (empty string when none). */
const char *glgpu_last_error(void);

/*
 * Creates a context for n_inst instances (mesh[k], prm[k]); builds the block-CSR
 * pattern and the assembly plan once per mesh (the reference does this in
 * setup_system(), femgl/src/setup_uniform_B-phase.cc:188-198) and allocates all
 * device memory.  The solution starts at zero.  The host side (plans, multigrid
 * transfer and Galerkin tables) runs on OpenMP threads, all host cores unless
 * OMP_NUM_THREADS says otherwise; its tables do not depend on the thread count.
 */
glgpu_status glgpu_create(const glgpu_mesh *mesh, const glgpu_params *prm, int n_inst, glgpu_ctx **out);
glgpu_status glgpu_destroy(glgpu_ctx *ctx);

/* Sizes: total nodes, total block nonzeros, block size (18 or 2), instances. */
glgpu_status glgpu_sizes(const glgpu_ctx *ctx, int64_t *n_nodes, int64_t *nnzb, int *block, int *n_inst);

/*
 * local_solution (femgl.h:313).  set_solution copies x in and applies the
 * solution constraints (constraints_solution.distribute, setup_uniform_B-phase.cc:263).
 */
glgpu_status glgpu_set_solution(glgpu_ctx *ctx, const double *x);
glgpu_status glgpu_get_solution(const glgpu_ctx *ctx, double *x);

/* Page-locked host memory for the arrays passed to set_solution / get_solution (and the
 * other host-array entry points): copies from and to it run as direct DMA instead of
 * being staged through a CUDA-internal bounce buffer.  Free with glgpu_host_free. */
glgpu_status glgpu_host_alloc(size_t bytes, void **p);
glgpu_status glgpu_host_free(void *p);

/*
 * FemGL<3>::assemble_system (femgl/src/assemble.cc:109-372): Jacobian (block CSR,
 * condensed) and system_rhs = -R at the current solution.  In GLGPU_MIXED mode
 * the Jacobian is FP32 and system_rhs comes from the FP64 residual kernel.
 * rhs_norm (may be NULL) receives ||system_rhs|| per instance.
 */
glgpu_status glgpu_assemble_system(glgpu_ctx *ctx, double *rhs_norm);

/*
 * FemGL<3>::compute_residual (femgl/src/residual.cc:110-297) evaluated at the
 * current solution; norm receives ||R|| per instance (residual_vector.l2_norm()).
 */
glgpu_status glgpu_compute_residual(glgpu_ctx *ctx, double *norm);

/*
 * FemGL<3>::solve(tol) (femgl/src/solve.cc:109-187): newton update delta with
 * ||J delta - rhs|| <= tol ||rhs|| (per instance), then distributed through the
 * constraints (solve.cc:181).  GMRES(restart) with the preconditioner of prm
 * replaces FGMRES + Trilinos ML AMG.  its (may be NULL) gets the iteration count
 * per instance.  Returns GLGPU_ERR_NOT_CONVERGED when gmres_max_iter is reached
 * (delta is still the last iterate).
 */
glgpu_status glgpu_solve(glgpu_ctx *ctx, double tol, int *its);

/*
 * FemGL<3>::newton_iteration (femgl/src/iteration.cc:110-215): backtracking
 * x + ls_step^i delta, i < ls_max_trials, accepting the first trial whose residual
 * norm is below ||system_rhs||; when none is, the last trial is kept.  res (may be
 * NULL) receives the residual norm at the accepted point, trials the number of
 * trials evaluated (per instance).
 */
glgpu_status glgpu_newton_iteration(glgpu_ctx *ctx, double *res, int *trials);

/*
 * The free energy F = integral of K1|grad A|^2 + (K2+K3) sum_mu |div A_mu|^2
 * + alpha tr(AA^+) + sum_t beta_t I_t at the current solution, per instance, evaluated
 * with the FP64 kernel in every precision mode (it also leaves the FP64 residual at the
 * solution in residual_vector).  The reference's residual is (1/2) dF/dx; the reference
 * itself never evaluates F.
 */
glgpu_status glgpu_free_energy(glgpu_ctx *ctx, double *F);

/*
 * FemGL<3>::run Newton loop of one refinement cycle (femgl/src/run.cc:207-252):
 * up to max_newton+1 times assemble, solve(linear_tol), newton_iteration, stop an
 * instance when its residual <= converge_acc.  Per instance outputs (any may be
 * NULL): newton_its, total GMRES iterations, final residual norm.
 * The stop test is always taken on an FP64 residual (run.cc:234): in GLGPU_MIXED mode the
 * line search evaluates |R| in double-float arithmetic, and when that value passes, the
 * FP64 residual at the accepted state decides; if it misses, Newton takes another step.
 * final_res is then that FP64 norm.
 */
glgpu_status glgpu_run(glgpu_ctx *ctx, int max_newton, double linear_tol, double converge_acc, int *newton_its,
                       int *gmres_its, double *final_res);

/*
 * The last glgpu_run step's residual norms per instance (either pointer may be NULL): the
 * line search's value (double-float in GLGPU_MIXED mode) and the FP64 value that took the
 * stop test.  They are equal in GLGPU_FP64 mode.  No reference counterpart: the reference
 * evaluates every residual in FP64.
 */
glgpu_status glgpu_stop_norms(const glgpu_ctx *ctx, double *line_search_norm, double *fp64_norm);

/* Downloads the pattern (rowptr [n_nodes+1], cols [nnzb]) and the Jacobian values
 * as FP64 [nnzb][B][B] (any pointer may be NULL), plus system_rhs [n_nodes*B]. */
glgpu_status glgpu_get_system(const glgpu_ctx *ctx, int32_t *rowptr, int32_t *cols, double *vals, double *rhs);

/* Downloads residual_vector (+R, condensed) [n_nodes*B] of the last residual evaluation. */
glgpu_status glgpu_get_residual(const glgpu_ctx *ctx, double *R);

/* Downloads the last newton update delta [n_nodes*B]. */
glgpu_status glgpu_get_update(const glgpu_ctx *ctx, double *delta);

/* y = J x with the assembled Jacobian (in its stored precision), host vectors. */
glgpu_status glgpu_spmv(glgpu_ctx *ctx, const double *x, double *y);

/*
 * Timing on the context's stream (CUDA events).  phase_ms receives accumulated
 * milliseconds of {assembly, compute_residual, solve, newton_iteration} since
 * the last reset, mirroring the reference's TimerOutput sections
 * (assemble.cc:111, residual.cc:112, solve.cc:111, iteration.cc:112).
 */
glgpu_status glgpu_timers(glgpu_ctx *ctx, double *phase_ms, int reset);

/*
 * Per-kernel-class device time, measured with events around each launch of the
 * kinds whose bit is set in enable (bit k = kind k; -1 = all; 0 = off; small
 * overhead per timed launch): kernel_ms[k] and launches[k] (launches are always
 * counted) for k = {spmv, cell assembly, row gather, residual, precond, vector ops}.
 */
glgpu_status glgpu_kernel_timing(glgpu_ctx *ctx, int enable, double *kernel_ms, int64_t *launches, int reset);

/* Number of kernels this context has launched since creation. */
int64_t glgpu_launch_count(const glgpu_ctx *ctx);

/* Device memory this context holds (its own allocations and its multigrid levels'), in
 * bytes; and the device's free and total memory (cudaMemGetInfo).  A sweep larger than the
 * device uses them to pack instances into batched contexts that fit. */
int64_t glgpu_device_bytes(const glgpu_ctx *ctx);
glgpu_status glgpu_mem_info(size_t *free_bytes, size_t *total_bytes);

/* Coarse levels of the multigrid hierarchy (0 when the preconditioner is not multigrid
 * or an instance is neither a uniform box grid nor a once-refined one).  Levels are nested
 * tensor grids (every other node line per coarsened axis; the first coarse level of a
 * once-refined box is its unrefined grid), coarse Jacobians are Galerkin products P^T J P. */
int glgpu_mg_levels(const glgpu_ctx *ctx);

/* Linear solves whose multigrid cycles stalled (true residual not halved by a restart
 * cycle) or diverged and that finished with block-Jacobi GMRES. */
int64_t glgpu_mg_fallbacks(const glgpu_ctx *ctx);

/* Handoff (default off): an instance whose multigrid solve stalls again after its fresh
 * multigrid pass does not finish with block-Jacobi GMRES in this context; glgpu_run stops its
 * Newton iteration at the state it reached (no update from the unfinished solve), counts it
 * as not converged (GLGPU_ERR_NOT_CONVERGED) and flags it, so that the caller can finish it in
 * a context of its own (a batch then does not wait for one hard instance on launches sized
 * for the whole batch). */
glgpu_status glgpu_set_mg_handoff(glgpu_ctx *ctx, int on);
/* flags[k] = 1 when instance k was handed off in the last glgpu_run, else 0 (n_inst bytes). */
glgpu_status glgpu_mg_handed_off(const glgpu_ctx *ctx, uint8_t *flags);

/* GMRES orthogonalization: classical Gram-Schmidt with one projection (off, the default: two
 * passes over the basis per iteration) or with one reorthogonalization (on: three passes).
 * The true residual is checked after every restart cycle either way; on the 32^3 workload both
 * take the same iterations and the single projection is 3 % faster per solve. */
glgpu_status glgpu_set_reorthogonalization(glgpu_ctx *ctx, int on);

/* Sizes of coarse level `level` (1 = first coarse level .. glgpu_mg_levels): its node
 * count, block count, and the entries of the prolongation from it to level - 1. */
glgpu_status glgpu_mg_level_info(const glgpu_ctx *ctx, int level, int64_t *n_nodes, int64_t *nnzb, int64_t *p_nnz);

/* Pattern and FP64 values of the Jacobian of coarse level `level` as of the last
 * assembly (same layout as glgpu_get_system). */
glgpu_status glgpu_mg_level_system(const glgpu_ctx *ctx, int level, int32_t *rowptr, int32_t *cols, double *vals);

/* Prolongation from coarse level `level` to level - 1 as node-level CSR over the finer
 * level's nodes: ptr [fine nodes + 1], idx (coarse node ids), w (weights).  It acts on
 * every component of a node; restriction is its transpose. */
glgpu_status glgpu_mg_prolongation(const glgpu_ctx *ctx, int level, int32_t *ptr, int32_t *idx, double *w);

/* The coarsest level's dense FP32 inverse of instance `inst` as of the last preconditioner
 * setup: *nd = its unknowns; inv (nd * nd, row-major, may be NULL to query nd) receives
 * (A + shift * mean|diag A| * I)^-1 with A that level's Jacobian and shift the
 * mg_coarse_shift parameter, or the identity when the factorisation met a zero pivot.
 * Synchronises the context's stream. */
glgpu_status glgpu_mg_coarse_inverse(glgpu_ctx *ctx, int inst, int *nd, float *inv);

/*
 * Launch mode of the solve's kernels, process-wide (default 1): with 1 they are launched
 * with programmatic dependent launch, so each kernel's CTAs are scheduled while its
 * predecessor finishes and wait on the device (griddepcontrol.wait) before touching
 * memory; 0 gives plain stream order.  Results are identical; contexts created (and
 * V-cycle graphs captured) afterwards use the new mode.  No reference counterpart.
 */
glgpu_status glgpu_set_launch_mode(int programmatic);

/* Blocks until all work of the context's stream is done. */
glgpu_status glgpu_sync(glgpu_ctx *ctx);

/* Device time (ms) between two calls on the context's stream: start, then stop. */
glgpu_status glgpu_event_start(glgpu_ctx *ctx);
glgpu_status glgpu_event_stop(glgpu_ctx *ctx, double *ms);

/* ---------------------------------------------------------------------------
 * Host-side helpers (no device work).
 * --------------------------------------------------------------------------- */

/*
 * Matep (reference matep/src/matep.cc:140-206,213-250) at pressure p [bar] and
 * t = T/Tc with strong-coupling corrections on (scc != 0) or off.
 * out[13] = {alpha, beta1..beta5, gap_A, gap_B, Tc_mK, f_A, f_B, beta_A, beta_B}.
 * p outside [0, 34) is rejected (the reference interpolation is undefined there).
 */
glgpu_status glgpu_matep(double p, double t, int scc, double *out);

/*
 * Structured box mesh in the reference's make_grid form
 * (femgl/src/makegrid_cube-z-normal_AdGR.cc:157-195): [lo, hi] with n[3] cells,
 * cells whose centre is within refine_band of a z face refined once (hanging nodes
 * constrained as DoFTools::make_hanging_node_constraints does for Q1), and the
 * zero-Dirichlet masks of the pair-breaking boundary (orbital column z of u and v
 * on z faces, femgl.h:300-301).  dirichlet_xy[0/1] selects the x / y faces' condition:
 *   0 natural (homogeneous Neumann), 1 pair-breaking (zero orbital column x / y),
 *   2 periodic: every node of the upper face is constrained to its image on the lower
 *     face (makegrid_retangle-z-AdGR_xy-periodic.cc:150-200 with
 *     DoFTools::make_periodicity_constraints, setup_weak-coupling-PDW-configuration.cc:192-202),
 *     chains (edges of two periodic axes, hanging nodes on a periodic face) resolved to
 *     unconstrained parents as AffineConstraints::close does.
 * First call with NULL arrays to get the sizes, then with arrays of those sizes.
 */
glgpu_status glgpu_mesh_box(const double *lo, const double *hi, const int *n, double refine_band,
                            const int *dirichlet_xy, int *n_nodes, int *n_cells, int *n_hang_entries, double *xyz,
                            int32_t *cells, uint32_t *mask, int32_t *hang_ptr, int32_t *hang_parent,
                            double *hang_weight);

/*
 * The same box with the cells chosen by flags[n[0] n[1] n[2]] (cells of the unrefined grid,
 * x fastest, the order glgpu_mesh_box gives them) refined once, e.g. the refinement flags of
 * glgpu_refine_flags on an unrefined box (refine.cc:155-170: execute_coarsening_and_refinement,
 * one level; coarsening flags are ignored).  Hanging constraints, masks and periodic faces as
 * in glgpu_mesh_box; periodic faces need the same refinement on both sides.
 */
glgpu_status glgpu_mesh_box_refine(const double *lo, const double *hi, const int *n, const int8_t *flags,
                                   const int *dirichlet_xy, int *n_nodes, int *n_cells, int *n_hang_entries,
                                   double *xyz, int32_t *cells, uint32_t *mask, int32_t *hang_ptr,
                                   int32_t *hang_parent, double *hang_weight);

/*
 * Solution transfer onto a refined box (SolutionTransfer::interpolate, refine.cc:160-170):
 * x[p] = the trilinear interpolant of x_box (values at the (n+1)^3 nodes of the unrefined
 * n-grid, node-major 18-vectors) at the points xyz[p].
 */
glgpu_status glgpu_box_interpolate(const double *lo, const double *hi, const int *n, const double *x_box, int n_points,
                                   const double *xyz, double *x);

/*
 * B-phase initial guess of setup_uniform_B-phase.cc:238-259: u11 = u22 = u33 =
 * gap_B(p,t) * 0.577350269f, everything else 0, for n_nodes nodes.  When
 * noise_sigma > 0 adds noise_sigma * N(0,1) per dof from a counter-based
 * generator keyed by seed (the reference draws from an unseeded std::random_device;
 * the seeded noise is this implementation's).
 */
glgpu_status glgpu_bphase_guess(double p, double t, int scc, int n_nodes, double noise_sigma, uint64_t seed,
                                double *x);

/*
 * Weak-coupling pair-density-wave initial state of
 * setup_weak-coupling-PDW-configuration.cc:286-320 (femgl/inc/pdw_config.h:111-298) at
 * the n_nodes points xyz[n][3]: the B phase gap_B(p,t)/sqrt(3) on the diagonal of u plus
 * the modulation of amplitude gap_B * u ("amplitude u parameter") across a slab of
 * thickness 2 half_D ("half z length of retangle") with in-plane wave number
 * pi / (2 sqrt(3) half_D).  glgpu_set_solution then applies the constraints
 * (constraints_solution.distribute in the reference).
 */
glgpu_status glgpu_pdw_guess(double p, double t, int scc, double u, double half_D, int n_nodes, const double *xyz,
                             double *x);

/*
 * Kelly error estimator on the GPU (replaces KellyErrorEstimator::estimate, refine.cc:147-152,
 * QGauss<2>(2) faces, no Neumann boundaries, all components) at the current solution:
 *   eta_K = sqrt( diam_K / 24 * sum over interior faces F of K of int_F |[du/dn]|^2 dS ),
 * boundary faces contributing nothing, periodic faces interior, a coarse-fine face split
 * into the fine faces.  eta [n_cells of all instances] (host, FP32; may be NULL to keep it
 * on the device for glgpu_refine_flags).  3D contexts with at most one level of refinement
 * difference across a face.
 */
glgpu_status glgpu_estimate_error(glgpu_ctx *ctx, float *eta);

/*
 * refine_and_coarsen_fixed_number (refine.cc:154-157) on the last estimate, per instance of
 * n_K cells: the floor(top_fraction n_K) cells of largest eta get flag 1 (every cell with
 * eta >= that rank's value), the floor(bottom_fraction n_K) of smallest eta flag -1, others 0.
 * The rank values are found on the GPU by an exact radix select.  flags [n_cells] (host).
 */
glgpu_status glgpu_refine_flags(glgpu_ctx *ctx, double top_fraction, double bottom_fraction, int8_t *flags);

/*
 * Host-only inspection of the once-per-mesh plan (no device needed):
 * info[6] = {n_nodes, nnzb, longest block row, cell contributions, hanging targets,
 * reduction segments}; the block pattern as CSR (rowptr [n_nodes+1], cols [nnzb]),
 * the condensed sparsity of DoFTools::make_sparsity_pattern(..., constraints, false)
 * at node granularity (femgl/src/setup_uniform_B-phase.cc:191-197).
 */
glgpu_status glgpu_plan_info(const glgpu_mesh *mesh, int n_inst, int64_t *info);
glgpu_status glgpu_plan_pattern(const glgpu_mesh *mesh, int n_inst, int32_t *rowptr, int32_t *cols);
/* faces[nc] (cells of all instances in order): bit f = 2 axis + side set when face f of the
 * cell is a Robin (AdGR) face, i.e. a boundary face with boundary id 2/3/4 in the reference
 * (assemble.cc:286-292), recognised by the zero-Dirichlet normal column of its nodes.
 * The term is assembled only where bt < 1e10. */
glgpu_status glgpu_plan_robin(const glgpu_mesh *mesh, int n_inst, uint8_t *faces);
/* Interior face pairs of the error estimator: pair k joins face fa[k] (2 axis + side) of cell
 * a[k] with face fb[k] of cell b[k]; sub[k] = 1 when a's face is a quarter of b's (coarse-fine),
 * 0 when they coincide (periodic pairs included).  First call with NULL arrays for n_pairs. */
glgpu_status glgpu_plan_kelly(const glgpu_mesh *mesh, int n_inst, int64_t *n_pairs, int32_t *a, int8_t *fa,
                              int32_t *b, int8_t *fb, int8_t *sub);
/* Multigrid prolongation from the first coarse level to the instance meshes, as the
 * multigrid preconditioner builds it: node-level CSR over the fine nodes, ptr [n_nodes + 1],
 * idx (coarse node ids), w; constrained fine nodes have empty rows, constrained coarse nodes
 * are replaced by their parents.  coarse_xyz [n_coarse][3] are the coarse nodes'
 * coordinates.  First call with NULL arrays for n_coarse and nnz; n_coarse = 0 when
 * multigrid does not apply to the meshes. */
glgpu_status glgpu_plan_prolongation(const glgpu_mesh *mesh, int n_inst, int64_t *n_coarse, int64_t *nnz,
                                     int32_t *ptr, int32_t *idx, double *w, double *coarse_xyz);

/* ---------------------------------------------------------------------------
 * Learned initial guess (no counterpart in the reference, which starts Newton from a
 * uniform B phase, setup_uniform_B-phase.cc:238-259).  An MLP
 *   (x, y, z, t = T/Tc, p [bar], D [xi0]) -> 256 -> 256 -> 256 -> 256 -> 18
 * with SiLU hidden activations, BF16 weights/activations and FP32 accumulation on the
 * tcgen05 tensor cores, FP32 master weights trained with Adam on converged states.
 * Inputs are normalised as (input - shift) * scale.  Arrays are HOST memory:
 * inputs [P][6], targets/outputs [P][18], parameters in layer order (W [out][in], b [out]).
 * --------------------------------------------------------------------------- */
typedef struct glgpu_surrogate glgpu_surrogate;

glgpu_status glgpu_surrogate_create(uint64_t seed, glgpu_surrogate **out);
glgpu_status glgpu_surrogate_destroy(glgpu_surrogate *s);
glgpu_status glgpu_surrogate_set_normalization(glgpu_surrogate *s, const float *shift, const float *scale);
glgpu_status glgpu_surrogate_param_count(int64_t *n);
glgpu_status glgpu_surrogate_get_params(glgpu_surrogate *s, float *params);
glgpu_status glgpu_surrogate_set_params(glgpu_surrogate *s, const float *params);
/* outputs[P][18] = network(inputs[P][6]) */
glgpu_status glgpu_surrogate_predict(glgpu_surrogate *s, const float *inputs, int P, float *outputs);
/* loss = (1/2P) sum |y - target|^2 and its gradient (parameter order) for one batch, no update */
glgpu_status glgpu_surrogate_gradient(glgpu_surrogate *s, const float *inputs, const float *targets, int P,
                                      float *loss, float *grad);
/* `steps` Adam steps on minibatches of `batch` rows (seeded shuffle); loss_out = mean loss
 * of the last steps */
glgpu_status glgpu_surrogate_train(glgpu_surrogate *s, const float *inputs, const float *targets, int n_rows,
                                   int steps, int batch, float lr, uint64_t seed, float *loss_out);
int64_t glgpu_surrogate_launch_count(const glgpu_surrogate *s);

/*
 * Deterministic FP64 dot product result[0] = sum_i x[i] * y[i] of two DEVICE vectors
 * of length n, written to a DEVICE double, enqueued on `stream` (a cudaStream_t;
 * NULL = the legacy default stream).  No counterpart in the reference: it exists for
 * callers that cannot allocate device memory where they need a norm (inside stream
 * capture, in allocation-free loops, or when the host framework owns all device
 * memory).  It allocates nothing: its partial sums live in a fixed per-device array
 * of 16,384 doubles, so n <= 16,777,216 (larger n returns GLGPU_ERR_ARG).  The first
 * call on a device looks up that array's address; make it before any stream capture.
 * The array is shared by all calls and keeps the last call's partials; calls that
 * overlap on the GPU race on it and must be serialised by the caller.
 */
glgpu_status glgpu_dot_noalloc(const double *x, const double *y, int64_t n, double *result, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GLGPU_H */
