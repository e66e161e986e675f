// Transient path: the assembly with time-derivative terms, the Newton solve
// of one time step and the fixed-step time loop of include/gb_newton.h.
//
// Restates the transient branch of solve_problem (src/rf_solve.c:1138-2601)
// for a constant time step: the histories start at the initial state with
// zero time derivatives (:1218-1230); the first three steps are backward
// Euler (theta = 0, :1375-1386) and later ones use the caller's theta; each
// step predicts x and xdot (predict_solution, :2767-2834), solves the step
// by Newton with xdot following every update (src/mm_sol_nonlinear.c:2560),
// and shifts the histories (:2359-2366).  The element kernels add the mass
// terms of xdot and their (1 + 2 theta) / delta_t sensitivity.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>

#include "../../include/gb_newton.h"
#include "gb_context.h"

namespace gb {

// predict_solution: the trapezoid rule's second-order extrapolation
// (order2), else the first-order one; xdot consistent with the prediction
__global__ void predict_kernel(int N, int order2, double c1, double c2, double c3,
                               double mass_c, double two_theta,
                               const double *__restrict__ x_old,
                               const double *__restrict__ x_older,
                               const double *__restrict__ x_oldest,
                               const double *__restrict__ xd_old,
                               const double *__restrict__ xd_older, double *__restrict__ x,
                               double *__restrict__ xd) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const double xo = x_old[i];
    const double xp = order2 ? c3 * xo + c2 * x_older[i] + c1 * x_oldest[i]
                             : xo + c1 * xd_old[i] - c2 * xd_older[i];
    x[i] = xp;
    xd[i] = mass_c * (xp - xo) - two_theta * xd_old[i];
  }
}

static int check_step(double delta_t, double theta) {
  if (!(delta_t > 0.0) || !std::isfinite(delta_t)) return fail("delta_t must be positive");
  if (!(theta >= 0.0 && theta <= 1.0)) return fail("theta must lie in [0, 1]");
  return 0;
}

static double mass_coefficient(double delta_t, double theta) {
  return (1.0 + 2.0 * theta) / delta_t;
}

}  // namespace gb

using gb::Context;

extern "C" {

int gb_matrix_fill_full_transient_device(gb_ctx *ctx, const double *d_x, const double *d_xdot,
                                         double delta_t, double theta, double *d_R,
                                         double *d_vals, void *stream) {
  if (!ctx || !d_x || !d_xdot || !d_R) return gb::fail("NULL argument");
  if (gb::check_step(delta_t, theta)) return -1;
  Context &c = ctx->c;
  c.d_xdot = d_xdot;
  c.mass_c = gb::mass_coefficient(delta_t, theta);
  const int rc = c.assemble(d_x, d_R, d_vals, (cudaStream_t)stream);
  c.d_xdot = nullptr;
  c.mass_c = 0.0;
  return rc;
}

int gb_matrix_fill_full_transient(gb_ctx *ctx, const double *x, const double *xdot,
                                  double delta_t, double theta, double *resid_vector,
                                  double *a_msr) {
  if (!ctx || !x || !xdot || !resid_vector) return gb::fail("NULL argument");
  if (gb::check_step(delta_t, theta)) return -1;
  Context &c = ctx->c;
  const size_t nb = sizeof(double) * c.L.N;
  double *d_xd = nullptr;
  cudaError_t e = cudaMalloc(&d_xd, nb);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c.d_x, x, nb, cudaMemcpyHostToDevice, c.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_xd, xdot, nb, cudaMemcpyHostToDevice, c.stream);
  int rc = 0;
  if (e != cudaSuccess) {
    rc = gb::cuda_fail(e, "transient fill upload");
  } else {
    rc = gb_matrix_fill_full_transient_device(ctx, c.d_x, d_xd, delta_t, theta, c.d_R,
                                              a_msr ? c.d_vals : nullptr, c.stream);
    if (rc == 0) {
      e = cudaMemcpyAsync(resid_vector, c.d_R, nb, cudaMemcpyDeviceToHost, c.stream);
      if (e != cudaSuccess) rc = gb::cuda_fail(e, "R copy");
    }
    if (rc == 0 && a_msr) rc = c.to_msr_host(c.d_vals, a_msr);
    if (rc == 0) rc = c.check_status();
  }
  cudaStreamSynchronize(c.stream);
  cudaFree(d_xd);
  return rc;
}

int gb_solve_nonlinear_problem_transient(gb_ctx *ctx, double *x, double *xdot, double delta_t,
                                         double theta, const gb_newton_opts *opts,
                                         int *converged, gb_newton_stats *stats) {
  if (!ctx || !x || !xdot || !converged) return gb::fail("NULL argument");
  if (gb::check_step(delta_t, theta)) return -1;
  Context &c = ctx->c;
  gb_newton_opts o;
  if (opts)
    o = *opts;
  else
    gb_newton_opts_default(&o);
  const size_t nb = sizeof(double) * c.L.N;
  double *d_xd = nullptr;
  cudaError_t e = cudaMalloc(&d_xd, nb);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c.d_x, x, nb, cudaMemcpyHostToDevice, c.stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_xd, xdot, nb, cudaMemcpyHostToDevice, c.stream);
  int rc = 0;
  if (e != cudaSuccess) {
    rc = gb::cuda_fail(e, "transient step upload");
  } else {
    rc = gb::newton(&c, c.d_x, o, converged, stats, d_xd,
                    gb::mass_coefficient(delta_t, theta));
    e = cudaMemcpyAsync(x, c.d_x, nb, cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(xdot, d_xd, nb, cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess && rc == 0) rc = gb::cuda_fail(e, "transient step copy back");
  }
  cudaFree(d_xd);
  return rc;
}

int gb_solve_transient(gb_ctx *ctx, double *x, int num_steps, double delta_t, double theta,
                       const gb_newton_opts *opts, double *x_steps, gb_newton_stats *stats,
                       int *steps_done) {
  if (!ctx || !x) return gb::fail("NULL argument");
  if (num_steps < 1) return gb::fail("num_steps must be at least 1");
  if (gb::check_step(delta_t, theta)) return -1;
  Context &c = ctx->c;
  gb_newton_opts o;
  if (opts)
    o = *opts;
  else
    gb_newton_opts_default(&o);
  if (steps_done) *steps_done = 0;
  gb_newton_stats total;
  memset(&total, 0, sizeof(total));
  const int N = c.L.N;
  const size_t nb = sizeof(double) * N;
  // histories: x_old, x_older, x_oldest, xdot, xdot_old, xdot_older
  double *h[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  cudaError_t e = cudaSuccess;
  for (auto &p : h)
    if (e == cudaSuccess) e = cudaMalloc(&p, nb);
  int rc = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(c.d_x, x, nb, cudaMemcpyHostToDevice, c.stream);
  for (int k = 0; k < 3 && e == cudaSuccess; k++)
    e = cudaMemcpyAsync(h[k], c.d_x, nb, cudaMemcpyDeviceToDevice, c.stream);
  for (int k = 3; k < 6 && e == cudaSuccess; k++) e = cudaMemsetAsync(h[k], 0, nb, c.stream);
  if (e != cudaSuccess) rc = gb::cuda_fail(e, "transient histories");
  double *x_old = h[0], *x_older = h[1], *x_oldest = h[2];
  double *xd = h[3], *xd_old = h[4], *xd_older = h[5];
  for (int nt = 0; rc == 0 && nt < num_steps; nt++) {
    // backward Euler for the first three steps, then the caller's scheme
    const double th = nt < 3 ? 0.0 : theta;
    const double dt = delta_t;
    const bool order2 = th == 0.5;
    // predict_solution's coefficients with equal steps (dt_old = dt_older = dt)
    double c1, c2, c3 = 0.0;
    if (order2) {  // x = 3 x_old - 3 x_older + x_oldest
      c1 = 1.0;
      c2 = -3.0;
      c3 = 3.0;
    } else {  // x = x_old + dt (1 + theta) xdot_old - theta dt xdot_older
      c1 = dt * (1.0 + th);
      c2 = th * dt;
    }
    const double mc = gb::mass_coefficient(dt, th);
    gb::predict_kernel<<<304, 256, 0, c.stream>>>(N, order2 ? 1 : 0, c1, c2, c3, mc, 2.0 * th,
                                                  x_old, x_older, x_oldest, xd_old, xd_older,
                                                  c.d_x, xd);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
      rc = gb::cuda_fail(e, "predictor");
      break;
    }
    int conv = 0;
    gb_newton_stats st;
    rc = gb::newton(&c, c.d_x, o, &conv, &st, xd, mc);
    if (rc) break;
    total.newton_its += st.newton_its;
    total.linear_its += st.linear_its;
    total.refinements += st.refinements;
    total.assemble_ms += st.assemble_ms;
    total.scale_ms += st.scale_ms;
    total.factor_ms += st.factor_ms;
    total.solve_ms += st.solve_ms;
    total.total_ms += st.total_ms;
    total.factorizations += st.factorizations;
    if (nt < 64) {
      total.residual_l2[nt] = st.residual_l2[st.newton_its < 64 ? st.newton_its : 63];
      total.residual_loo_steps[nt] = st.residual_loo;
    }
    total.residual_loo = st.residual_loo;
    if (!conv) {
      char msg[96];
      snprintf(msg, sizeof msg, "time step %d did not converge", nt);
      rc = gb::fail(msg);
      break;
    }
    if (x_steps) {
      e = cudaMemcpyAsync(x_steps + (size_t)nt * N, c.d_x, nb, cudaMemcpyDeviceToHost, c.stream);
      if (e != cudaSuccess) {
        rc = gb::cuda_fail(e, "step copy");
        break;
      }
    }
    // shift the histories: oldest <- older <- old <- x, older <- old <- xdot
    double *t = x_oldest;
    x_oldest = x_older;
    x_older = x_old;
    x_old = t;
    e = cudaMemcpyAsync(x_old, c.d_x, nb, cudaMemcpyDeviceToDevice, c.stream);
    if (e != cudaSuccess) {
      rc = gb::cuda_fail(e, "history shift");
      break;
    }
    t = xd_older;
    xd_older = xd_old;
    xd_old = xd;
    xd = t;
    if (steps_done) *steps_done = nt + 1;
  }
  if (rc == 0) {
    e = cudaMemcpyAsync(x, c.d_x, nb, cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) rc = gb::cuda_fail(e, "x copy back");
  } else {
    cudaStreamSynchronize(c.stream);
  }
  for (auto p : h) cudaFree(p);
  if (stats) *stats = total;
  return rc;
}

}  // extern "C"
