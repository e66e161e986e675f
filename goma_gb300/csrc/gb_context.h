// Per-problem state behind the gb_ctx handle of include/gb_newton.h.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "../../include/gb_newton.h"
#include "gb_device.h"
#include "gb_layout.h"
#include "gb_solve.h"

#include <memory>

namespace gb {

extern thread_local std::string g_err;
int fail(const std::string &m);
int cuda_fail(cudaError_t e, const char *where);

struct Context {
  gb_problem_desc desc{};
  Layout L;
  MaterialDev mat{};
  bool carreau = false;
  // element kernel: 0 automatic (4 where it applies, else 1), 1 scalar FP64,
  // 2 DMMA with per-fragment coefficients, 3 DMMA products over operand tables
  // (3-D Newtonian), 4 sum factorisation (3-D Newtonian)
  int path = 0;
  int tc_grid = 0;     // persistent grid of the DMMA kernels
  // ILU triangular solves: 0 sync-free sweeps, 1 level-scheduled graph,
  // 2 automatic (the graph for short level schedules)
  int trsv = 2;
  // host-injected fault of the sync-free sweeps (gb_set_sweep_fault)
  long long sweep_spin_limit = 0;  // polls per wait; <= 0: the default
  int sweep_reverse_lower = 0;
  int ilu_ordering = 0;  // ILU(0) node order: 0 the reference's, 1 multicoloured
  cudaStream_t stream = nullptr;
  double *d_coords = nullptr;
  int *d_conn = nullptr;
  int *d_fu = nullptr;
  uint8_t *d_dbc = nullptr;
  double *d_dbc_val = nullptr;
  int64_t *d_rowptr = nullptr;
  int *d_colidx = nullptr;
  int *d_nbr_ptr = nullptr, *d_nbr_off = nullptr, *d_nbr_offT = nullptr, *d_nbr_node = nullptr;
  uint16_t *d_nslot = nullptr;
  double *d_tab_phi = nullptr, *d_tab_dphi = nullptr, *d_tab_w = nullptr, *d_tab_pt = nullptr;
  double *d_tab_iso = nullptr;  // 3-D: [value, d/dxi_r] x points x nodes (gemm kernel)
  SfTables *d_sf = nullptr;     // 3-D: tables of the sum-factorised kernel
  int *d_color_elems = nullptr;
  double *d_x = nullptr, *d_R = nullptr, *d_vals = nullptr;
  int *d_status = nullptr;
  double *d_elem_rho = nullptr;  // per-element density (gb_set_element_density); NULL: none
  // transient terms of later assemblies: device time derivative (N) and
  // (1 + 2 theta) / delta_t; NULL / 0 when steady
  const double *d_xdot = nullptr;
  double mass_c = 0.0;
  double *d_msr = nullptr;
  // integrated boundary conditions, one entry per side
  int num_sides = 0;
  int *d_side_elem = nullptr, *d_side_side = nullptr, *d_side_type = nullptr;
  double *d_side_val = nullptr;
  std::unique_ptr<Solver> solver;
  // optional kernel timing of the element kernels (events on the launch stream)
  bool timing = false;
  cudaEvent_t ev_k0 = nullptr, ev_k1 = nullptr;
  double kernel_ms = 0.0;
  long kernel_launches = 0;

  ~Context();
  int init(const gb_problem_desc *d);
  int set_material(const gb_material &m);
  AsmArgs args(const double *x, double *R, double *vals) const;
  // zero R (and vals), then launch one kernel per colour on st
  int assemble(const double *x, double *R, double *vals, cudaStream_t st);
  int reset_status();
  int check_status();
  // the element kernel an assembly with (vals != NULL) or without a Jacobian uses
  int kernel_path(bool jacobian) const;
  int to_msr_host(const double *vals, double *a_msr);
};

// Newton (gb_newton.cu); d_xdot != NULL: one transient step
int newton(Context *C, double *d_x, const gb_newton_opts &o, int *converged,
           gb_newton_stats *st, double *d_xdot, double mass_c);

}  // namespace gb

// the opaque handle of the C ABI
struct gb_ctx {
  gb::Context c;
};
