/* GB300 Newton hot path for Q2/P1 Navier-Stokes (+ energy): the C ABI of
 * libgbnewton.so.
 *
 * This is the drop-in boundary for the reference's Newton path.  A Goma
 * build links the library and calls these entry points where it calls the
 * functions named beside each declaration.  Plain pointers and sizes only;
 * every entry point returns 0 (GOMA_SUCCESS, include/mm_eh.h:34) or -1
 * (GOMA_ERROR) and leaves a message for gb_last_error().  Nothing calls
 * exit() or aborts.
 *
 * Host/device convention: functions without a _device suffix take HOST
 * arrays and copy them in and out; _device variants take device pointers
 * (allocated by the caller or obtained from gb_device_buffers) and a CUDA
 * stream (NULL = the library's stream) and never synchronise the host.
 */
#ifndef GB_NEWTON_H
#define GB_NEWTON_H

#include "gb_problem.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gb_ctx gb_ctx;

/* Builds the DOF map, the CSR/MSR sparsity, the element colouring and the
 * device copies of one problem; the state the reference builds in
 * setup_problem (src/rf_setup_problem.c:194) and alloc_MSR_sparse_arrays
 * (src/mm_fill_util.c:2865, called from src/rf_solve.c:769). */
int gb_create(const gb_problem_desc *desc, gb_ctx **out);
void gb_destroy(gb_ctx *ctx);
/* Message of the last failed call on this thread ("" if none). */
const char *gb_last_error(void);

/* Sizes: unknowns N (NumUnknowns), MSR length ija[N] (the reference's
 * "Number of matrix nonzeroes" + 1), CSR nonzeros (diagonal in row). */
int gb_num_unknowns(const gb_ctx *ctx);
long long gb_msr_length(const gb_ctx *ctx);
long long gb_csr_nnz(const gb_ctx *ctx);
int gb_num_colors(const gb_ctx *ctx);

/* The reference's MSR pattern, bit for bit: ija[0..N] row pointers into
 * the off-diagonal part (which starts at N+1), then the off-diagonal
 * columns in ascending order (src/mm_fill_util.c:3229
 * find_MSR_problem_graph).  ija holds gb_msr_length() ints. */
int gb_msr_pattern(const gb_ctx *ctx, int *ija);
/* Host-only form of the same query, without a GPU or a context: fills ija
 * (may be NULL) and its length, as alloc_MSR_sparse_arrays does
 * (src/mm_fill_util.c:2865). */
int gb_msr_pattern_host(const gb_problem_desc *desc, int *ija, long long *msr_length);
/* Host only: the multicoloured node order of the GB_ILU_MULTICOLOUR
 * preconditioner (gb_set_ilu_ordering) and the matrix in it.  perm[n]: new
 * number of node n (num_nodes); num_colours: its ILU dependency levels;
 * umap[i']: old unknown of new unknown i' (N); rowptr/colidx: the permuted
 * CSR pattern (N + 1, nnz); vmap[k']: old CSR position of new entry k'
 * (nnz).  Any output may be NULL. */
int gb_ilu_permutation_host(const gb_problem_desc *desc, int *perm, int *num_colours, int *umap,
                            long long *rowptr, int *colidx, long long *vmap);
/* Host only: the order in which the sync-free ILU(0) sweeps add each row's
 * off-node entries (oldest dependency level first) for the given node
 * ordering (GB_ILU_*), in the CSR layout of that ordering (the permuted one
 * of gb_ilu_permutation_host for GB_ILU_MULTICOLOUR): entry p of a row's
 * off-node lower or upper segment is read from the segment's start +
 * rel[p] (nnz values); lev / levu (num_nodes, may be NULL) get every
 * node's forward / backward dependency level.  For inspecting the sweeps;
 * no counterpart in the reference. */
int gb_sweep_order_host(const gb_problem_desc *desc, int ordering, unsigned short *rel,
                        int *lev, int *levu);
/* CSR pattern used on the device: rowptr (N+1, int64), colidx (nnz). */
int gb_csr_pattern(const gb_ctx *ctx, long long *rowptr, int *colidx);
/* One row of the CSR matrix: its 64-bit start offset in the CSR arrays, its
 * columns (from the layout) and its values (copied from d_vals, this
 * context's CSR values on the device; the library stream is synchronised).
 * Returns the row's length (cols and vals may be NULL to ask for it), or -1
 * when it exceeds capacity.  For inspecting rows of matrices too large to
 * copy out whole; no counterpart in the reference. */
long long gb_csr_row(gb_ctx *ctx, const double *d_vals, int row, long long *start, int *cols,
                     double *vals, long long capacity);
/* First unknown of every node (num_nodes + 1 ints), as
 * Nodes[i]->First_Unknown (src/mm_unknown_map.c:758). */
int gb_first_unknown(const gb_ctx *ctx, int *fu);
/* Writes the Dirichlet values (later cards win) and the pressure datum into
 * the host vector x, as find_and_set_Dirichlet does (src/mm_bc.c:132). */
int gb_dirichlet_init(const gb_ctx *ctx, double *x);

/* Drop-in for matrix_fill_full (src/mm_fill.c:158): residual R and, when
 * a_msr is not NULL, the analytic Jacobian in the reference's MSR layout
 * (a_msr holds gb_msr_length() doubles; entry N is unused and written 0).
 * Host arrays; R and a_msr are overwritten (the reference's caller zeroes
 * them before the call, src/mm_sol_nonlinear.c:1114-1120, so the result is
 * the same).  Returns -1 when an element has a non-positive Jacobian
 * determinant, as matrix_fill_full does (src/mm_fill.c:217-312).  A
 * page-locked a_msr (cudaHostAlloc / cudaHostRegister), 16-byte aligned, is
 * written by a copy kernel at the host link's rate; a pageable one goes
 * through a staged copy. */
int gb_matrix_fill_full(gb_ctx *ctx, const double *x, double *resid_vector, double *a_msr);

/* Device form: d_x (N), d_R (N) and d_vals (CSR values, gb_csr_nnz()) are
 * device pointers; d_vals NULL assembles the residual only
 * (af->Assemble_Jacobian = FALSE).  Enqueued on stream; the determinant
 * status is checked at the next gb_status() call. */
int gb_matrix_fill_full_device(gb_ctx *ctx, const double *d_x, double *d_R, double *d_vals,
                               void *stream);
/* Transient form of matrix_fill_full (its x, xdot, delta_t and theta
 * arguments, src/mm_fill.c:158-176): the residual gets the mass terms of the
 * time derivative xdot (momentum -rho v_dot phi dA, energy -rho Cp T_dot phi
 * dA, species -Y_dot phi dA; src/mm_fill_momentum.c:471-500,
 * src/mm_fill_energy.c:315-381, src/mm_fill_species.c:525-551) and the
 * Jacobian their sensitivity (1 + 2 theta) / delta_t (:1586-1590).  Host
 * arrays as gb_matrix_fill_full; delta_t > 0, 0 <= theta <= 1. */
int gb_matrix_fill_full_transient(gb_ctx *ctx, const double *x, const double *xdot,
                                  double delta_t, double theta, double *resid_vector,
                                  double *a_msr);
/* Device form (as gb_matrix_fill_full_device), d_xdot N doubles on the
 * device. */
int gb_matrix_fill_full_transient_device(gb_ctx *ctx, const double *d_x, const double *d_xdot,
                                         double delta_t, double theta, double *d_R,
                                         double *d_vals, void *stream);
/* Synchronises the library stream and reports the determinant status of
 * all assemblies since the previous call: returns -1 (with the first bad
 * element in the message) or 0. */
int gb_status(gb_ctx *ctx);

/* Library-owned device buffers: x (N), R (N), CSR values (nnz), and the
 * CSR pattern (rowptr N+1 int64, colidx nnz int32). */
int gb_device_buffers(gb_ctx *ctx, double **d_x, double **d_R, double **d_vals,
                      const long long **d_rowptr, const int **d_colidx);
/* The library's CUDA stream (a cudaStream_t). */
void *gb_stream(gb_ctx *ctx);

/* Element-kernel path of later assemblies: 0 = automatic (4 where it
 * applies, else 1), 1 = scalar FP64, 2 = 3-D Jacobian contractions on the
 * FP64 tensor pipe (DMMA) with per-fragment coefficients, 3 = the whole 3-D
 * residual + Jacobian as DMMA products over shared-memory operand tables,
 * 4 = the 3-D residual + Jacobian by sum factorisation over the
 * tensor-product basis (the fewest FP64 operations).  Paths 3 and 4 take
 * Newtonian viscosity; Carreau and 2-D elements use path 1.  A residual-only
 * assembly uses the same kernel as the full one under paths 0, 1, 3 and 4,
 * so its R is bitwise the full assembly's; under path 2 it uses path 1.  All
 * give the same matrix to rounding. */
int gb_set_assembly_path(gb_ctx *ctx, int path);

/* Node order of the ILU(0) preconditioner of later solves.
 * GB_ILU_NATURAL: the reference's node-major order (AztecOO's ILU(0) on one
 * subdomain); its triangular solves have one dependency level per node
 * "wavefront" (833 levels on the 32^3 HEX27 cube).  GB_ILU_MULTICOLOUR: the
 * nodes without pressure unknowns in greedy colours of the node graph, then
 * the element centroids (the pressure nodes) in theirs -- 28 levels on HEX27
 * meshes, 10 on QUAD9 -- so factorisation and sweeps run level by level with
 * a whole level in parallel; it preconditions the same system with a
 * different (not the reference's) incomplete factorisation.  The converged
 * Newton solution does not depend on the choice. */
#define GB_ILU_NATURAL 0
#define GB_ILU_MULTICOLOUR 1
int gb_set_ilu_ordering(gb_ctx *ctx, int ordering);

/* Per-element density (num_elems values, > 0) for later assemblies, in
 * place of the material's: lets one context hold several independent
 * problems that differ in Reynolds number (rho = Re with mu = U = L = 1).
 * rho = NULL returns to the material's density.  With per-element
 * densities, 3-D elements use path 4 (or 1 when path 1 is set). */
int gb_set_element_density(gb_ctx *ctx, const double *rho);

/* ILU(0) triangular solves of later linear solves: 0 = sync-free sweeps
 * (one launch per factor; each node polls the solution values it depends
 * on, bounded, then publishes its own; a CTA per node, or a warp per node
 * on meshes with short rows), 1 = level-scheduled sweeps (one launch per
 * dependency level, a CTA per node) replayed as a CUDA graph, 2 = automatic
 * (the default: the graph when the schedule has at most 64 levels, as in
 * the multicoloured order; the sync-free sweeps otherwise).  All give the
 * same result to rounding.  No counterpart in the reference (AztecOO's ILU
 * solves are sequential). */
int gb_set_triangular_solve(gb_ctx *ctx, int mode);

/* Host-side fault injection for the sync-free sweeps' bounded waits; no
 * counterpart in the reference.  spin_limit sets the polls a wait makes
 * before it gives up (<= 0: the default, 2^22, about 0.3 s).  With
 * reverse_lower != 0 the lower sweep hands its nodes out in reverse order
 * (every dependency after the node that needs it) on a grid of one CTA,
 * so its first wait can only end by running out: the sweep then finishes
 * with the error word set, later waits of the solve stop within 1024 polls,
 * and the linear solve returns -1 ("a dependency wait gave up") with the
 * context still usable.  (0, 0) restores the normal sweeps.  Applies to
 * the sync-free sweeps only (gb_set_triangular_solve mode 0, or 2 with a
 * deep schedule). */
int gb_set_sweep_fault(gb_ctx *ctx, long long spin_limit, int reverse_lower);

/* Replaces the material of a context (same mesh, DOF map and pattern), as
 * update_parameterC does during continuation (src/ac_conti.c:755,
 * src/ac_update_parameter.c). */
int gb_set_material(gb_ctx *ctx, const gb_material *mat);

/* Instrumentation: with enable = 1, every following assembly records CUDA
 * events around its element-kernel launches (on the launch stream, then
 * synchronises); a call returns the accumulated kernel time and launch
 * count since the previous call and sets the new state. */
int gb_kernel_timing(gb_ctx *ctx, int enable, double *kernel_ms, long long *launches);

/* Converts device CSR values (same ctx) to the MSR layout in host memory
 * (gb_msr_length() doubles). */
int gb_csr_to_msr_host(gb_ctx *ctx, const double *d_vals, double *a_msr);

/* ---------------------------------------------------------- Newton solve */

#define GB_LINEAR_FP64 0
#define GB_LINEAR_FP32_REFINED 1
/* FP64 flexible GMRES (the Krylov basis, Gram-Schmidt and the matrix in
 * FP64) whose ILU(0) preconditioner is factorised and applied in FP32: the
 * triangular sweeps, the cost of an iteration, run at the FP32 rate while
 * the Krylov process keeps FP64 accuracy; the flexible form (the
 * preconditioned vectors kept) makes the FP32 rounding of the sweeps
 * harmless to convergence.  Several independent problems in one matrix
 * run the batched form (one flexible GMRES per problem). */
#define GB_LINEAR_FP32_PRECONDITIONER 2

/* ILU(0) factorisation reuse, the reference's "Matrix Factorization Reuse"
 * card (src/mm_sol_nonlinear.c:1688-1709, src/sl_util.c:721-734):
 * CALC factors at every Newton step ("calc", the default; "recalc" does the
 * same numeric work here, the pattern being fixed); PER_SOLVE factors at
 * the first Newton step of each gb_solve_nonlinear_problem call and reuses
 * those factors for its later steps; REUSE keeps the last factors of this
 * context across calls ("reuse", AztecOO's AZ_reuse) and factors only when
 * there are none for the precision in use.  The matrix of every linear
 * solve is always the current one; only the preconditioner lags. */
#define GB_FACTOR_CALC 0
#define GB_FACTOR_PER_SOLVE 1
#define GB_FACTOR_REUSE 2

/* Solver cards of the input deck (src/mm_input.c rd_solver_specs). */
typedef struct gb_newton_opts {
  int max_newton;          /* "Number of Newton Iterations" */
  double residual_tol;     /* "Normalized Residual Tolerance" (Epsilon[0]) */
  double damping;          /* "Newton correction factor" */
  int krylov_dim;          /* "Size of Krylov subspace" (AztecOO default 30; at most
                              1023, and 31 for several independent problems in one
                              context) */
  int max_linear_its;      /* "Maximum Linear Solve Iterations" */
  double linear_tol;       /* "Linear Solver Tolerance" (relative residual) */
  int linear_precision;    /* GB_LINEAR_FP64, _FP32_REFINED or _FP32_PRECONDITIONER */
  double inner_tol;        /* refined mode: the tightest relative tolerance of one
                              FP32 inner GMRES solve (an inner solve stops sooner
                              when the outer tolerance allows it) */
  int max_refinements;     /* FP64 refinement steps (refined mode) */
  int verbose;             /* 1: one line per Newton step on stdout */
  /* Inexact Newton: 0 solves every linear system to linear_tol; 1 chooses
   * each step's tolerance by Eisenstat and Walker's second rule,
   * eta_k = 0.9 (|R_k| / |R_k-1|)^2 (safeguarded by 0.9 eta_k-1^2 when that
   * exceeds 0.1), kept within [linear_tol, forcing_max].  The converged
   * solution is decided by residual_tol either way. */
  int forcing;
  double forcing_max;
  int factorization_reuse; /* GB_FACTOR_CALC, _PER_SOLVE or _REUSE */
} gb_newton_opts;

typedef struct gb_newton_stats {
  int newton_its;          /* Newton steps taken (assemblies - 1 on convergence) */
  int linear_its;          /* Krylov iterations, all steps */
  int refinements;         /* FP64 refinement steps, all steps */
  double residual_l2[64];  /* scaled-residual L2 norm per Newton step */
  double residual_loo;     /* final scaled-residual L-infinity norm */
  double assemble_ms, scale_ms, factor_ms, solve_ms, total_ms;
  int factorizations;      /* ILU(0) factorisations done, all steps */
  /* the other two norms the reference prints per Newton step
   * (src/mm_sol_nonlinear.c:1451-1453: L_oo, L_1, L_2 of the scaled
   * residual) */
  double residual_l1[64];
  double residual_loo_steps[64];
} gb_newton_stats;

/* sizeof of the ABI structs, for bindings that mirror them: 0
 * gb_newton_opts, 1 gb_newton_stats, 2 gb_problem_desc, 3 gb_material;
 * 0 for any other value.  Needs no device. */
long long gb_abi_struct_size(int which);

void gb_newton_opts_default(gb_newton_opts *o);

/* Drop-in for solve_nonlinear_problem (src/mm_sol_nonlinear.c:596), steady
 * case: Newton from x (host, N doubles, Dirichlet values already set as
 * find_and_set_Dirichlet leaves them) until the row-sum-scaled residual
 * has L2 and L-infinity norms below residual_tol after at least one update
 * (:1482-1486).  Each step: matrix_fill_full, row_sum_scaling_scale
 * (src/sl_matrix_util.c:441), ILU(0)-GMRES (the AztecOO case, :1805),
 * x -= damping * dx (:2553).  x is overwritten with the last iterate;
 * *converged is 1 or 0.  Returns -1 on a non-positive Jacobian
 * determinant, a non-finite residual, or a CUDA error. */
int gb_solve_nonlinear_problem(gb_ctx *ctx, double *x, const gb_newton_opts *opts,
                               int *converged, gb_newton_stats *stats);
/* One time step of solve_nonlinear_problem (src/mm_sol_nonlinear.c:596,
 * transient arguments delta_t, theta, xdot): Newton from the predicted x
 * and xdot (host, N doubles each, both overwritten), every assembly with
 * the transient terms of gb_matrix_fill_full_transient, every update
 * x -= damping dx with xdot -= damping (1 + 2 theta) / delta_t dx
 * (:2553-2562). */
int gb_solve_nonlinear_problem_transient(gb_ctx *ctx, double *x, double *xdot, double delta_t,
                                         double theta, const gb_newton_opts *opts,
                                         int *converged, gb_newton_stats *stats);
/* Drop-in for the transient branch of solve_problem (src/rf_solve.c:
 * 1138-2601) with a constant time step (a negative "delta_t" card,
 * :1153-1158): from the initial state x (host, Dirichlet values set) with
 * zero time derivatives, num_steps steps of delta_t -- backward Euler for
 * the first three (:1375-1386), then the time-step parameter theta (0.5:
 * Crank-Nicolson with the second-order predictor) -- each predicted by
 * predict_solution (:2767) and solved by Newton to opts' tolerance.  x gets
 * the last solution; x_steps (num_steps x N doubles, may be NULL) every
 * step's; stats (may be NULL) the sums of the Newton and Krylov counts and
 * times, with residual_l2[k] / residual_loo_steps[k] the converged step k's
 * L2 / L-infinity norms; *steps_done (may be NULL) the steps completed.
 * Returns -1 when a step does not converge (no step-size reduction) or on
 * an error. */
int gb_solve_transient(gb_ctx *ctx, double *x, int num_steps, double delta_t, double theta,
                       const gb_newton_opts *opts, double *x_steps, gb_newton_stats *stats,
                       int *steps_done);
/* Same with x in device memory (N doubles); the iterate stays there. */
int gb_solve_nonlinear_problem_device(gb_ctx *ctx, double *d_x, const gb_newton_opts *opts,
                                      int *converged, gb_newton_stats *stats);

/* row_sum_scaling_scale (src/sl_matrix_util.c:441) on device CSR values
 * and residual of this context: scale[i] = sign(a_ii) sum_j |a_ij|, A and R
 * divided by it.  d_scale (N doubles) may be NULL. */
int gb_row_sum_scale_device(gb_ctx *ctx, double *d_vals, double *d_R, double *d_scale);

/* The Krylov solve of one Newton step (the Linear_Solver switch,
 * src/mm_sol_nonlinear.c:1624): factor ILU(0) of the scaled matrix
 * d_vals (device CSR values) and solve A dx = rhs by GMRES.  Device arrays.
 * With opts->factorization_reuse = GB_FACTOR_REUSE the last factors are kept
 * when there are any (a second right-hand side with the same matrix). */
int gb_linear_solve_device(gb_ctx *ctx, const double *d_vals, const double *d_rhs, double *d_dx,
                           const gb_newton_opts *opts, int *iterations, double *relres);
/* Host form taking the reference's MSR values (gb_msr_length() doubles,
 * already row-scaled as the reference does before AZ_solve) and host
 * vectors; the drop-in for aztecoo_solve_epetra
 * (src/sl_aztecoo_interface.cpp:56). */
int gb_linear_solve(gb_ctx *ctx, const double *a_msr, const double *rhs, double *dx,
                    const gb_newton_opts *opts, int *iterations, double *relres);

/* The ILU(0) preconditioner of gb_linear_solve for a row-scaled MSR matrix
 * (length ija[N]), in the library's CSR order (gb_csr_pattern): strictly
 * lower entries hold L (unit diagonal implied), the rest U.  fp32 = 1 gives
 * the factors of the FP32-refined mode (computed in FP32, widened).  For
 * checking the preconditioner against a CPU ILU(0); no counterpart in the
 * reference (AztecOO keeps its factors internal). */
int gb_ilu0_factors(gb_ctx *ctx, const double *a_msr, int fp32, double *lu_csr);

/* ---------------------------------------------- learned continuation guess */

/* A fully connected FP32 network, hidden layers tanh, trained on the GPU by
 * the library's own forward / backward / Adam kernels.  It predicts the next
 * Newton initial guess of a parameter continuation from (node coordinates,
 * parameter); the reference has no counterpart -- its predictor
 * (src/ac_conti.c:759-784, ALC_ZEROTH / ALC_FIRST) stays the fallback. */
typedef struct gb_mlp gb_mlp;
int gb_mlp_create(int n_in, int width, int hidden_layers, int n_out, unsigned long long seed,
                  gb_mlp **out);
void gb_mlp_destroy(gb_mlp *m);
int gb_mlp_num_params(const gb_mlp *m);
/* flat parameter / gradient buffers: per layer W[out][in] then b[out] */
int gb_mlp_get_params(const gb_mlp *m, float *host);
int gb_mlp_set_params(gb_mlp *m, const float *host);
int gb_mlp_get_grads(const gb_mlp *m, float *host);
/* The network's device entry points below (forward, loss and gradients,
 * training) run on the network's own stream and return once their work is
 * done.  That stream does not wait for the caller's streams: the device
 * arrays passed in must be complete on the device before the call (for
 * example, synchronise the stream that wrote them). */
/* y[B][n_out] = net(x[B][n_in]); device arrays */
int gb_mlp_forward_device(gb_mlp *m, const float *d_x, int B, float *d_y);
/* loss = sum mask (net(x) - t)^2 / sum mask, gradients kept inside (read
 * with gb_mlp_get_grads); device arrays, *loss on the host */
int gb_mlp_loss_grad_device(gb_mlp *m, const float *d_x, const float *d_t, const float *d_mask,
                            int B, float *loss);
int gb_mlp_adam_step(gb_mlp *m, float lr, float beta1, float beta2, float eps);
/* Same forward pass without allocating device memory.  This entry point has
 * no counterpart in the reference.  It is for callers that cannot call
 * cudaMalloc when they ask for a prediction: a continuation driver whose
 * device memory is all held by another allocator (a framework's caching
 * allocator that has reserved the GPU), or a solver loop that must not take
 * cudaMalloc's implicit device-wide synchronisation between Newton steps.
 * The caller still passes x and y; the hidden activations go to a fixed
 * array compiled into the library: two buffers of GB_MLP_NOALLOC_MAX_ACT
 * floats, so B times the hidden width may not exceed GB_MLP_NOALLOC_MAX_ACT
 * (larger batches are rejected with an error; split them).  Every GPU that
 * loads the library holds that 8 MB until the process exits.
 *
 * The pass is queued on `stream` (a cudaStream_t; NULL is CUDA's default
 * stream) and the call returns without waiting for it: x is read, and y
 * written, in that stream's order, so work the caller queued on `stream`
 * before the call is seen and work queued after it sees y.  The pass also
 * waits for the network's own queued work (training, parameter updates),
 * and the network's later work waits for the pass.  The network's device
 * must be current; another device is refused with an error.  The first call
 * on a device looks the array's device address up (once per device); make
 * that first call before any stream capture.  The address is kept for the
 * life of the process: after cudaDeviceReset this entry point may no longer
 * be called.  All calls share the array, so calls that overlap on the GPU
 * (other threads, other streams) race; it keeps the last call's
 * activations, and nothing in it needs to start at zero because every
 * activation is written before it is read. */
#define GB_MLP_NOALLOC_MAX_ACT (1 << 20)
int gb_mlp_forward_noalloc(gb_mlp *m, const float *d_x, int B, float *d_y, void *stream);
/* steps Adam steps on minibatches of `batch` points drawn from n_points
 * (fixed integer-hash sampling from seed) */
int gb_mlp_train_device(gb_mlp *m, const float *d_x, const float *d_t, const float *d_mask,
                        int n_points, int steps, int batch, float lr, unsigned long long seed,
                        float *final_loss);

/* Measures this GPU's FP64 throughput (TFLOP/s) with two short kernels:
 * mma.sync m8n8k4 f64 (tensor pipe) and scalar FMA.  The FP64 roofline
 * denominators of the element kernels. */
int gb_probe_fp64_peaks(double *dmma_tflops, double *fma_tflops);
/* FP64 mma.sync m8n8k4 throughput (TFLOP/s) with operands that change every
 * iteration, as in a real contraction. */
int gb_probe_dmma_varying(double *tflops);

#ifdef __cplusplus
}
#endif
#endif
