// Newton driver and the linear-solve entry points of include/gb_newton.h.
//
// Restates the steady branch of solve_nonlinear_problem
// (src/mm_sol_nonlinear.c:596): per step, assemble (matrix_fill_full,
// :1279), row-sum scale (:1317), residual norms (:1451-1453), convergence
// test on the scaled residual after the first step (:1482-1486), Krylov
// solve (:1805), full-step update x -= damping * dx (:2553-2557).  The whole
// step runs on the device; the host reads back three norms per step.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "../../include/gb_newton.h"
#include "gb_context.h"

namespace gb {

__global__ void update_kernel(int N, double damp, const double *__restrict__ dx,
                              double *__restrict__ x) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    x[i] = fma(-damp, dx[i], x[i]);
}

// the transient update: x -= damp dx and xdot -= damp (1 + 2 theta) / dt dx
// (src/mm_sol_nonlinear.c:2553-2562)
__global__ void update_transient_kernel(int N, double damp, double mass_c,
                                        const double *__restrict__ dx, double *__restrict__ x,
                                        double *__restrict__ xdot) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const double d = damp * dx[i];
    x[i] -= d;
    xdot[i] = fma(-mass_c, d, xdot[i]);
  }
}

// inverse of csr_to_msr: MSR values -> CSR values of this layout
__global__ void msr_to_csr_kernel(int N, const int64_t *__restrict__ rowptr,
                                  const int *__restrict__ colidx, const double *__restrict__ msr,
                                  double *__restrict__ vals) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (i >= N) return;
  for (int64_t k = rowptr[i] + lane; k < rowptr[i + 1]; k += 32) {
    const int c = colidx[k];
    vals[k] = c == i ? msr[i] : msr[(int64_t)N + 1 + k - i - (c > i ? 1 : 0)];
  }
}

static LinearOpts linear_opts(const gb_newton_opts &o) {
  LinearOpts l;
  l.krylov = o.krylov_dim > 0 ? (o.krylov_dim < 1023 ? o.krylov_dim : 1023) : 30;
  l.maxit = o.max_linear_its > 0 ? o.max_linear_its : 500;
  l.tol = o.linear_tol > 0 ? o.linear_tol : 1e-6;
  l.fp32_inner = o.linear_precision == GB_LINEAR_FP32_REFINED;
  l.fp32_prec = o.linear_precision == GB_LINEAR_FP32_PRECONDITIONER;
  l.inner_tol = o.inner_tol > 0 ? o.inner_tol : 1e-3;
  l.max_refinements = o.max_refinements > 0 ? o.max_refinements : 20;
  return l;
}

static int ensure_solver(Context *C, int krylov) {
  if (C->solver && C->solver->max_krylov >= krylov) return 0;
  C->solver.reset(new Solver);
  return C->solver->init(C, krylov);
}

static float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

// Newton from d_x.  With d_xdot (a transient step) the assemblies carry the
// time-derivative terms of d_xdot with sensitivity mass_c = (1 + 2 theta) /
// delta_t, and every update moves d_xdot with d_x.
int newton(Context *C, double *d_x, const gb_newton_opts &o, int *converged,
           gb_newton_stats *st, double *d_xdot, double mass_c) {
  LinearOpts lo = linear_opts(o);
  if (ensure_solver(C, lo.krylov)) return -1;
  struct TransientScope {  // the context's transient terms for this solve only
    Context *C;
    TransientScope(Context *c, const double *xd, double mc) : C(c) {
      C->d_xdot = xd;
      C->mass_c = xd ? mc : 0.0;
    }
    ~TransientScope() {
      C->d_xdot = nullptr;
      C->mass_c = 0.0;
    }
  } transient_scope(C, d_xdot, mass_c);
  const double tol_min = lo.tol;
  const double eta_max = o.forcing_max > 0 ? std::max(o.forcing_max, tol_min) : 1e-2;
  double eta = eta_max, prev_norm = -1.0;
  Solver &S = *C->solver;
  cudaStream_t s = C->stream;
  const int N = C->L.N;
  double *d_dx = nullptr;
  if (cudaMalloc(&d_dx, sizeof(double) * N) != cudaSuccess) return fail("dx allocation");
  cudaEvent_t ev[6];
  for (auto &e : ev) cudaEventCreate(&e);
  *converged = 0;
  gb_newton_stats local;
  gb_newton_stats &S_ = st ? *st : local;
  memset(&S_, 0, sizeof(S_));
  cudaEventRecord(ev[0], s);
  int rc = 0;
  const int maxit = o.max_newton > 0 ? o.max_newton : 20;
  const int reuse = o.factorization_reuse;
  if (reuse < GB_FACTOR_CALC || reuse > GB_FACTOR_REUSE) {
    cudaFree(d_dx);
    for (auto &e : ev) cudaEventDestroy(e);
    return fail("unknown factorization_reuse");
  }
  bool factored = false;  // in this call
  for (int it = 0; it < maxit; it++) {
    cudaEventRecord(ev[1], s);
    if (C->assemble(d_x, C->d_R, C->d_vals, s)) {
      rc = -1;
      break;
    }
    cudaEventRecord(ev[2], s);
    if (C->check_status()) {
      rc = -1;
      break;
    }
    S_.assemble_ms += elapsed(ev[1], ev[2]);
    if (row_sum_scale(C, C->d_vals, C->d_R, s)) {
      rc = -1;
      break;
    }
    double n3[3];
    if (device_norms(C, C->d_R, N, n3, s)) {
      rc = -1;
      break;
    }
    cudaEventRecord(ev[3], s);
    cudaEventSynchronize(ev[3]);
    S_.scale_ms += elapsed(ev[2], ev[3]);
    if (it < 64) {
      S_.residual_l2[it] = n3[0];
      S_.residual_l1[it] = n3[1];
      S_.residual_loo_steps[it] = n3[2];
    }
    S_.residual_loo = n3[2];
    if (o.verbose) printf("  newton [%d] |R|_2 %.3e |R|_inf %.3e\n", it, n3[0], n3[2]);
    if (!std::isfinite(n3[0]) || !std::isfinite(n3[1]) || !std::isfinite(n3[2])) {
      rc = fail("non-finite residual norm");
      break;
    }
    if (it > 0 && n3[0] < o.residual_tol && n3[2] < o.residual_tol) {
      *converged = 1;
      S_.newton_its = it;
      break;
    }
    if (o.forcing == 1) {
      // Eisenstat-Walker choice 2 (gamma 0.9, alpha 2) with its safeguard
      if (prev_norm > 0.0) {
        const double r = n3[0] / prev_norm;
        double e = 0.9 * r * r;
        const double safe = 0.9 * eta * eta;
        if (safe > 0.1) e = std::max(e, safe);
        eta = std::min(eta_max, std::max(tol_min, e));
      }
      lo.tol = eta;
      prev_norm = n3[0];
    }
    // the preconditioner: new factors, or the last ones (factorization_reuse)
    const bool refactor = reuse == GB_FACTOR_CALC || !S.has_factors(lo.fp32_factors()) ||
                          (reuse == GB_FACTOR_PER_SOLVE && !factored);
    if (refactor ? S.factor(C->d_vals, lo.fp32_factors(), s)
                 : S.refresh(C->d_vals, lo.fp32_factors(), s)) {
      rc = -1;
      break;
    }
    if (refactor) {
      factored = true;
      S_.factorizations++;
    }
    cudaEventRecord(ev[4], s);
    LinearStats ls;
    if (linear_solve(C, C->d_R, d_dx, lo, &ls, s)) {
      rc = -1;
      break;
    }
    if (d_xdot)
      update_transient_kernel<<<304, 256, 0, s>>>(N, o.damping > 0 ? o.damping : 1.0, mass_c,
                                                  d_dx, d_x, d_xdot);
    else
      update_kernel<<<304, 256, 0, s>>>(N, o.damping > 0 ? o.damping : 1.0, d_dx, d_x);
    cudaEventRecord(ev[5], s);
    cudaEventSynchronize(ev[5]);
    S_.factor_ms += elapsed(ev[3], ev[4]);
    S_.solve_ms += elapsed(ev[4], ev[5]);
    S_.linear_its += ls.iterations;
    S_.refinements += ls.refinements;
    S_.newton_its = it + 1;
    if (o.verbose)
      printf("           linear its %d (refinements %d) relres %.2e\n", ls.iterations,
             ls.refinements, ls.relres);
  }
  cudaEventRecord(ev[1], s);
  cudaEventSynchronize(ev[1]);
  S_.total_ms = elapsed(ev[0], ev[1]);
  for (auto &e : ev) cudaEventDestroy(e);
  cudaFree(d_dx);
  cudaError_t e = cudaGetLastError();
  if (rc == 0 && e != cudaSuccess) rc = cuda_fail(e, "newton");
  return rc;
}

}  // namespace gb

using gb::Context;


extern "C" {

void gb_newton_opts_default(gb_newton_opts *o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->max_newton = 20;
  o->residual_tol = 1e-10;
  o->damping = 1.0;
  o->krylov_dim = 30;
  o->max_linear_its = 500;
  o->linear_tol = 1e-6;
  o->linear_precision = GB_LINEAR_FP64;
  o->inner_tol = 1e-3;
  o->max_refinements = 20;
  o->forcing = 0;
  o->forcing_max = 1e-2;
  o->factorization_reuse = GB_FACTOR_CALC;
}

long long gb_abi_struct_size(int which) {
  switch (which) {
    case 0: return (long long)sizeof(gb_newton_opts);
    case 1: return (long long)sizeof(gb_newton_stats);
    case 2: return (long long)sizeof(gb_problem_desc);
    case 3: return (long long)sizeof(gb_material);
    default: return 0;
  }
}

int gb_solve_nonlinear_problem_device(gb_ctx *ctx, double *d_x, const gb_newton_opts *opts,
                                      int *converged, gb_newton_stats *stats) {
  if (!ctx || !d_x || !converged) return gb::fail("NULL argument");
  gb_newton_opts o;
  if (opts)
    o = *opts;
  else
    gb_newton_opts_default(&o);
  return gb::newton(&ctx->c, d_x, o, converged, stats, nullptr, 0.0);
}

int gb_solve_nonlinear_problem(gb_ctx *ctx, double *x, const gb_newton_opts *opts, int *converged,
                               gb_newton_stats *stats) {
  if (!ctx || !x || !converged) return gb::fail("NULL argument");
  Context &c = ctx->c;
  cudaError_t e = cudaMemcpyAsync(c.d_x, x, sizeof(double) * c.L.N, cudaMemcpyHostToDevice, c.stream);
  if (e != cudaSuccess) return gb::cuda_fail(e, "x copy");
  int rc = gb_solve_nonlinear_problem_device(ctx, c.d_x, opts, converged, stats);
  e = cudaMemcpyAsync(x, c.d_x, sizeof(double) * c.L.N, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return gb::cuda_fail(e, "x copy back");
  return rc;
}

int gb_row_sum_scale_device(gb_ctx *ctx, double *d_vals, double *d_R, double *d_scale) {
  if (!ctx || !d_vals || !d_R) return gb::fail("NULL argument");
  Context &c = ctx->c;
  if (gb::ensure_solver(&c, 30)) return -1;
  if (gb::row_sum_scale(&c, d_vals, d_R, c.stream)) return -1;
  if (d_scale) {
    cudaError_t e = cudaMemcpyAsync(d_scale, c.solver->d_scale, sizeof(double) * c.L.N,
                                    cudaMemcpyDeviceToDevice, c.stream);
    if (e != cudaSuccess) return gb::cuda_fail(e, "scale copy");
  }
  return 0;
}

int gb_linear_solve_device(gb_ctx *ctx, const double *d_vals, const double *d_rhs, double *d_dx,
                           const gb_newton_opts *opts, int *iterations, double *relres) {
  if (!ctx || !d_vals || !d_rhs || !d_dx) return gb::fail("NULL argument");
  gb_newton_opts o;
  if (opts)
    o = *opts;
  else
    gb_newton_opts_default(&o);
  Context &c = ctx->c;
  const gb::LinearOpts lo = gb::linear_opts(o);
  if (gb::ensure_solver(&c, lo.krylov)) return -1;
  // GB_FACTOR_REUSE keeps the last factors when there are any (a second
  // solve with the same matrix, or a lagged preconditioner)
  const bool reuse = o.factorization_reuse == GB_FACTOR_REUSE &&
                     c.solver->has_factors(lo.fp32_factors());
  if (reuse ? c.solver->refresh(d_vals, lo.fp32_factors(), c.stream)
            : c.solver->factor(d_vals, lo.fp32_factors(), c.stream))
    return -1;
  gb::LinearStats ls;
  if (gb::linear_solve(&c, d_rhs, d_dx, lo, &ls, c.stream)) return -1;
  cudaError_t e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return gb::cuda_fail(e, "linear solve");
  if (iterations) *iterations = ls.iterations;
  if (relres) *relres = ls.relres;
  return 0;
}

int gb_linear_solve(gb_ctx *ctx, const double *a_msr, const double *rhs, double *dx,
                    const gb_newton_opts *opts, int *iterations, double *relres) {
  if (!ctx || !a_msr || !rhs || !dx) return gb::fail("NULL argument");
  Context &c = ctx->c;
  const int N = c.L.N;
  const int64_t len = gb::layout_msr_length(c.L);
  double *d_msr = nullptr, *d_vals = nullptr, *d_rhs = nullptr, *d_dx = nullptr;
  cudaError_t e = cudaMalloc(&d_msr, sizeof(double) * len);
  if (e == cudaSuccess) e = cudaMalloc(&d_vals, sizeof(double) * c.L.nnz);
  if (e == cudaSuccess) e = cudaMalloc(&d_rhs, sizeof(double) * N);
  if (e == cudaSuccess) e = cudaMalloc(&d_dx, sizeof(double) * N);
  int rc = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_msr, a_msr, sizeof(double) * len, cudaMemcpyHostToDevice, c.stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_rhs, rhs, sizeof(double) * N, cudaMemcpyHostToDevice, c.stream);
  if (e != cudaSuccess) {
    rc = gb::cuda_fail(e, "linear solve upload");
  } else {
    gb::msr_to_csr_kernel<<<(int)(((int64_t)N * 32 + 255) / 256), 256, 0, c.stream>>>(
        N, c.d_rowptr, c.d_colidx, d_msr, d_vals);
    rc = gb_linear_solve_device(ctx, d_vals, d_rhs, d_dx, opts, iterations, relres);
    if (rc == 0) {
      e = cudaMemcpy(dx, d_dx, sizeof(double) * N, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) rc = gb::cuda_fail(e, "dx copy");
    }
  }
  cudaFree(d_msr);
  cudaFree(d_vals);
  cudaFree(d_rhs);
  cudaFree(d_dx);
  return rc;
}

int gb_ilu0_factors(gb_ctx *ctx, const double *a_msr, int fp32, double *lu_csr) {
  if (!ctx || !a_msr || !lu_csr) return gb::fail("NULL argument");
  Context &c = ctx->c;
  const int N = c.L.N;
  const int64_t len = gb::layout_msr_length(c.L), nnz = c.L.nnz;
  if (gb::ensure_solver(&c, 30)) return -1;
  double *d_msr = nullptr, *d_vals = nullptr;
  cudaError_t e = cudaMalloc(&d_msr, sizeof(double) * len);
  if (e == cudaSuccess) e = cudaMalloc(&d_vals, sizeof(double) * nnz);
  int rc = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_msr, a_msr, sizeof(double) * len, cudaMemcpyHostToDevice, c.stream);
  if (e != cudaSuccess) {
    rc = gb::cuda_fail(e, "factor upload");
  } else {
    gb::msr_to_csr_kernel<<<(int)(((int64_t)N * 32 + 255) / 256), 256, 0, c.stream>>>(
        N, c.d_rowptr, c.d_colidx, d_msr, d_vals);
    rc = c.solver->factor(d_vals, fp32 != 0, c.stream);
    if (rc == 0) rc = c.solver->copy_factors(lu_csr, fp32 != 0, c.stream);
  }
  cudaFree(d_msr);
  cudaFree(d_vals);
  return rc;
}

}  // extern "C"
