/* Dump hooks for the reference-as-oracle build (test infrastructure).
 *
 * The recipe links with -Wl,--wrap=matrix_fill_full, so every call the
 * reference's Newton loop (src/mm_sol_nonlinear.c:1279) makes to
 * matrix_fill_full (src/mm_fill.c:158) passes through here.  Environment:
 *   GB_REF_X_IN   raw little-endian float64 file; when set, x[] is replaced
 *                 by its contents before the first assembly (a seeded state,
 *                 or the initial guess of a Newton solve)
 *   GB_REF_DUMP   path prefix; the first assembly writes <prefix>.ija
 *                 (int32, MSR bindx), <prefix>.a (float64, MSR values),
 *                 <prefix>.R and <prefix>.x (float64, length N)
 *   GB_REF_XDOT_IN  raw float64 file; when set, xdot[] is replaced by it
 *                 before the first assembly (a seeded time derivative)
 *   GB_REF_EXIT   when set, exit(0) right after that first dump
 * A transient first assembly also writes <prefix>.xdot (float64, N) and
 * <prefix>.dt (float64: delta_t, theta). 
 * With -Wl,--wrap=numerical_jacobian the reference's Jacobian checker
 * (src/mm_numjac.c:716, run when the deck sets Debug = -1/-2/-3) also gets
 * the GB_REF_X_IN state before it copies x, so its perturbed states are
 * taken around that state.
 * Everything else runs the unmodified reference code. */
#include <stdio.h>
#include <stdlib.h>

#include "std.h"
#include "exo_struct.h"
#include "dpi.h"
#include "mm_as_structs.h"
#include "sl_util_structs.h"

int __real_matrix_fill_full(struct GomaLinearSolverData *ams, double x[], double resid_vector[],
                            double x_old[], double x_older[], double xdot[], double xdot_old[],
                            double x_update[], double *ptr_delta_t, double *ptr_theta,
                            struct elem_side_bc_struct *first_elem_side_BC_array[],
                            double *ptr_time_value, Exo_DB *exo, Dpi *dpi,
                            int *ptr_num_total_nodes, dbl *ptr_h_elem_avg, dbl *ptr_U_norm,
                            dbl *estifm);

static int g_calls = 0;

/* x[] <- the GB_REF_X_IN file (N doubles) */
static void read_x_in(const char *xin, double *x, int N) {
  FILE *f = fopen(xin, "rb");
  if (!f || fread(x, sizeof(double), (size_t)N, f) != (size_t)N) {
    fprintf(stderr, "harness: cannot read %d doubles from %s\n", N, xin);
    exit(3);
  }
  fclose(f);
}

void __real_numerical_jacobian(struct GomaLinearSolverData *ams, double x[],
                               double resid_vector[], double delta_t, double theta,
                               double x_old[], double x_older[], double xdot[],
                               double xdot_old[], double x_update[], int num_total_nodes,
                               struct elem_side_bc_struct *first_elem_side_BC_array[],
                               int Debug_Flag, double time_value, Exo_DB *exo, Dpi *dpi,
                               double *h_elem_avg, double *U_norm);

void __wrap_numerical_jacobian(struct GomaLinearSolverData *ams, double x[],
                               double resid_vector[], double delta_t, double theta,
                               double x_old[], double x_older[], double xdot[],
                               double xdot_old[], double x_update[], int num_total_nodes,
                               struct elem_side_bc_struct *first_elem_side_BC_array[],
                               int Debug_Flag, double time_value, Exo_DB *exo, Dpi *dpi,
                               double *h_elem_avg, double *U_norm) {
  const char *xin = getenv("GB_REF_X_IN");
  if (xin) read_x_in(xin, x, ams->npu);
  __real_numerical_jacobian(ams, x, resid_vector, delta_t, theta, x_old, x_older, xdot, xdot_old,
                            x_update, num_total_nodes, first_elem_side_BC_array, Debug_Flag,
                            time_value, exo, dpi, h_elem_avg, U_norm);
}

static void dump(const char *prefix, const char *ext, const void *p, size_t sz, size_t n) {
  char path[4096];
  snprintf(path, sizeof path, "%s.%s", prefix, ext);
  FILE *f = fopen(path, "wb");
  if (!f || fwrite(p, sz, n, f) != n) {
    fprintf(stderr, "harness: cannot write %s\n", path);
    exit(3);
  }
  fclose(f);
}

int __wrap_matrix_fill_full(struct GomaLinearSolverData *ams, double x[], double resid_vector[],
                            double x_old[], double x_older[], double xdot[], double xdot_old[],
                            double x_update[], double *ptr_delta_t, double *ptr_theta,
                            struct elem_side_bc_struct *first_elem_side_BC_array[],
                            double *ptr_time_value, Exo_DB *exo, Dpi *dpi,
                            int *ptr_num_total_nodes, dbl *ptr_h_elem_avg, dbl *ptr_U_norm,
                            dbl *estifm) {
  const int N = ams->npu;
  const char *xin = getenv("GB_REF_X_IN");
  if (xin && g_calls == 0) read_x_in(xin, x, N);
  const char *xdin = getenv("GB_REF_XDOT_IN");
  if (xdin && g_calls == 0 && xdot) read_x_in(xdin, xdot, N);
  int err = __real_matrix_fill_full(ams, x, resid_vector, x_old, x_older, xdot, xdot_old,
                                    x_update, ptr_delta_t, ptr_theta, first_elem_side_BC_array,
                                    ptr_time_value, exo, dpi, ptr_num_total_nodes,
                                    ptr_h_elem_avg, ptr_U_norm, estifm);
  const char *prefix = getenv("GB_REF_DUMP");
  if (prefix && g_calls == 0) {
    const int len = ams->bindx[N]; /* MSR length: N diagonal + 1 + off-diagonals */
    dump(prefix, "ija", ams->bindx, sizeof(int), (size_t)len);
    dump(prefix, "a", ams->val, sizeof(double), (size_t)len);
    dump(prefix, "R", resid_vector, sizeof(double), (size_t)N);
    dump(prefix, "x", x, sizeof(double), (size_t)N);
    if (xdot && ptr_delta_t && ptr_theta) {
      const double dt[2] = {*ptr_delta_t, *ptr_theta};
      dump(prefix, "xdot", xdot, sizeof(double), (size_t)N);
      dump(prefix, "dt", dt, sizeof(double), 2);
    }
    fprintf(stderr, "harness: dumped N=%d msr_len=%d err=%d\n", N, len, err);
    if (getenv("GB_REF_EXIT")) exit(0);
  }
  g_calls++;
  return err;
}
