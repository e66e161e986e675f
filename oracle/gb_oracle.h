/* CPU oracle for the Q2/P1 Newton hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's algorithm for the path that the
 * GB300 library replaces: DOF map and MSR sparsity (src/mm_unknown_map.c,
 * src/exo_conn.c:204, src/mm_fill_util.c:3229), element residual and
 * analytic Jacobian (src/mm_fill.c:317 matrix_fill with assemble_momentum
 * src/mm_fill_momentum.c:100, assemble_continuity
 * src/mm_fill_continuity.c:119, assemble_energy src/mm_fill_energy.c:109,
 * assemble_mass_transport src/mm_fill_species.c:194),
 * hard-set Dirichlet rows (src/bc_dirich.c:44), the MSR scatter
 * (src/mm_fill.c:5175), row-sum scaling (src/sl_matrix_util.c:506) and the
 * Newton loop (src/mm_sol_nonlinear.c:1108).  It is pinned against golden
 * vectors produced by the reference itself (tests/golden/).  Only tests,
 * the smoke check and the CPU-baseline leg of the benchmark may use it; the
 * product path never calls it.
 */
#ifndef GB_ORACLE_H
#define GB_ORACLE_H

#include "../include/gb_problem.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_problem orc_problem;

/* Builds the DOF map, Dirichlet marks and MSR pattern.  A problem whose MSR
 * would exceed the reference's 32-bit indexing gets no pattern: only the
 * element-level calls and residual-only fills (a == NULL) work on it. */
orc_problem *orc_create(const gb_problem_desc *desc);
void orc_destroy(orc_problem *p);
int orc_num_unknowns(const orc_problem *p);
/* MSR length = ija[N] = N + 1 + number of off-diagonal entries */
long orc_msr_len(const orc_problem *p);
void orc_msr_pattern(const orc_problem *p, int *ija);
/* First_Unknown per node, num_nodes + 1 entries */
void orc_first_unknown(const orc_problem *p, int *fu);
/* 1 for every unknown carrying a Dirichlet condition or the pressure datum */
void orc_dirichlet_mask(const orc_problem *p, int *mask);
/* Writes the Dirichlet values (later cards win) and the datum into x. */
void orc_dirichlet_init(const orc_problem *p, double *x);
/* Adds the contributions of elements [e0, e1) to R (length N) and, when a
 * is not NULL, to the MSR values a (length msr_len).  Returns 0, or -1 when
 * an element has a non-positive Jacobian determinant. */
int orc_matrix_fill(const orc_problem *p, const double *x, double *R, double *a, int e0, int e1);
/* The same over the n elements listed in elems. */
int orc_matrix_fill_list(const orc_problem *p, const double *x, double *R, double *a,
                         const int *elems, int n);
/* Greedy colouring of the elements (no two elements of a colour share a
 * node, so their contributions touch disjoint rows); returns the number of
 * colours, or -1. */
int orc_element_colors(const orc_problem *p, int *color);
/* Element-level residual and Jacobian (before the Dirichlet rows are
 * applied when apply_bc == 0), in the oracle's local DOF order:
 * velocity component a of local node k at a*nn + k, temperature at
 * dim*nn + k, species w at (dim+energy+w)*nn + k, pressure mode l at
 * (dim+energy+species)*nn + l. */
int orc_element(const orc_problem *p, int e, const double *x, double *Re, double *Je,
                int apply_bc);
int orc_local_size(const orc_problem *p);
void orc_element_dofs(const orc_problem *p, int e, int *gdof);
/* scale[i] = sign(a_ii) * sum_j |a_ij|; a and R are divided by it. */
void orc_row_sum_scale(const orc_problem *p, double *a, double *R, double *scale);
/* ILU(0) (IKJ order, pivots below tau in magnitude set to +-tau) of the
 * MSR matrix a into lu (same layout).  Returns 0, -1 on allocation failure. */
int orc_ilu0(const orc_problem *p, const double *a, double tau, double *lu);
/* Full Newton from x with a banded direct solve.  Returns the number of
 * iterations (>= 0) on convergence, -1 on failure.  norms (optional) gets
 * the scaled-residual L2 norm of every iteration (max_it entries). */
int orc_newton(const orc_problem *p, double *x, int max_it, double tol, double *norms);
/* Transient terms of later fills: the time derivative xdot (N values, NULL
 * for steady) and the mass coefficient (1 + 2 theta) / delta_t. */
void orc_set_transient(orc_problem *p, const double *xdot, double mass_c);
/* orc_newton for one time step: xdot follows every update
 * (xdot -= mass_c dx); the transient terms are cleared on return. */
int orc_newton_transient(orc_problem *p, double *x, double *xdot, double mass_c, int max_it,
                         double tol, double *norms);
/* Restarted right-preconditioned GMRES(m) with the ILU(0) factors lu (from
 * orc_ilu0) on the MSR system a x = b, from x = 0, until the residual is
 * below tol * |b| or maxit iterations.  Returns 0 when converged, 1 when
 * not, -1 on allocation failure; *its and *relres (optional) report. */
int orc_gmres_ilu0(const orc_problem *p, const double *a, const double *lu, const double *b,
                   double *x, int m, int maxit, double tol, int *its, double *relres);
/* Newton as orc_newton with ILU(0)-GMRES(m) (pivot floor tau, linear
 * tolerance lin_tol, at most lin_maxit iterations per solve) instead of the
 * direct solve.  Returns the Newton iterations on convergence, -1 on
 * failure; *linear_its (optional) gets the total Krylov iterations. */
int orc_newton_gmres(const orc_problem *p, double *x, int max_it, double tol, double lin_tol,
                     int m, int lin_maxit, double tau, int *linear_its, double *norms);

#ifdef __cplusplus
}
#endif
#endif
