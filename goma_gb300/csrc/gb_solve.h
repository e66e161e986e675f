// Krylov solve on the device: row-sum scaling, norms, CSR SpMV, ILU(0)
// (node-level schedule), GMRES(m) in FP64 or FP32-inside-FP64-refinement.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "gb_layout.h"

namespace gb {

struct Context;

// Host-built schedule of the ILU(0) factorisation and triangular solves:
// nodes grouped by level; all unknowns of one node are handled by one warp
// in order, so a level only waits for the levels before it.
struct IluSchedule {
  std::vector<int> lo_nodes, lo_ptr;  // forward (L) levels
  std::vector<int> up_nodes, up_ptr;  // backward (U) levels
  std::vector<int> lev, levu;         // every node's forward / backward level
};
void build_ilu_schedule(const Layout &L, IluSchedule &S);

// Device view of the layout the ILU(0) factors live in: the context's own
// arrays in the reference's node order, permuted copies in the multicoloured
// order.
struct PrecLayout {
  const int *fu = nullptr;
  const int64_t *rowptr = nullptr;
  const int *colidx = nullptr;
  const int64_t *diag = nullptr;
  const int *nbr_ptr = nullptr, *nbr_node = nullptr, *nbr_off = nullptr, *nbr_offT = nullptr;
  const int *nbr_self = nullptr;  // each node's position in its own neighbour list
};

struct Solver {
  Context *C = nullptr;
  // ILU(0) node order: 0 the reference's, 1 multicoloured (few dependency
  // levels; the preconditioner of P A P^T, applied as P^T (LU)^-1 P)
  int ordering = 0;
  int num_levels = 0;
  PrecLayout P;
  int *d_umap = nullptr;        // permuted unknown -> unknown
  int64_t *d_vmap = nullptr;    // permuted CSR entry -> CSR entry
  double *d_Ap = nullptr;       // permuted scaled matrix
  double *d_tp = nullptr;       // permuted preconditioner vector
  float *d_tp32 = nullptr;
  std::vector<void *> owned;    // permuted layout arrays
  // Independent problems held in one matrix (diagonal blocks over contiguous
  // node ranges, found from the node graph): GMRES runs per block
  // (segmented reductions, one Hessenberg per block).  nseg == 1: one system.
  int nseg = 1, ntiles = 0;
  std::vector<int64_t> seg_ptr;   // unknown range of block s: [seg_ptr[s], seg_ptr[s+1])
  int *d_tile_seg = nullptr, *d_tile_ptr = nullptr;
  int64_t *d_tile_beg = nullptr, *d_tile_end = nullptr;
  double *d_segpart = nullptr;    // [ntiles][32] per-tile partial dot products
  double *d_segout = nullptr;     // [3][nseg][32] reduced dots (two passes) and norms
  double *d_segcoef = nullptr;    // [nseg][32] host-set coefficients
  int *d_segactive = nullptr;     // [nseg] blocks still iterating in this cycle
  double *h_segout = nullptr;     // pinned mirror of d_segout
  int N = 0;
  int64_t nnz = 0;
  // ILU(0) factors (same pattern as A): FP64 and FP32 copies
  double *d_lu = nullptr;
  float *d_lu32 = nullptr;
  float *d_a32 = nullptr;       // FP32 copy of the scaled matrix
  // dense inverses of every node's diagonal blocks of the factors (L's then
  // U's, nr^2 values each, from d_inv_ptr[node]): FP64 and FP32
  double *d_binv = nullptr;
  float *d_binv32 = nullptr;
  int64_t *d_inv_ptr = nullptr;
  int64_t inv_len = 0;
  // the sync-free sweeps' tables (see trsv_sync_free_kernel): factors and
  // column indices in sweep order, per-row off-node segments, tickets
  double *d_lus = nullptr;
  float *d_lus32 = nullptr;
  int *d_sweep_cols = nullptr;
  longlong2 *d_segL = nullptr, *d_segU = nullptr;
  longlong2 *d_tick_lo = nullptr, *d_tick_up = nullptr, *d_tick_lo_rev = nullptr;
  int64_t *d_diag = nullptr;    // position of the diagonal in every row
  int *d_fu = nullptr;          // first unknown per node (shared with C)
  int *d_lo_nodes = nullptr, *d_up_nodes = nullptr;
  std::vector<int> lo_ptr, up_ptr;
  uint16_t *d_sweep_rel = nullptr; // level-sorted entry order of the sweeps (build_sweep_order)
  const double *d_A = nullptr;  // scaled FP64 matrix the factors were built from
  double pivot_tau = 1e-4;      // ILU(0) pivot floor on the row-scaled matrix
  int maxnb = 0, lmax = 0;      // largest node neighbourhood / block-row length
  double *d_scale = nullptr;
  double *d_work = nullptr;     // reduction scratch
  double *h_work = nullptr;     // pinned host mirror
  int max_krylov = 0;
  double *d_V = nullptr;        // (m+1) x N Krylov basis (FP64)
  float *d_V32 = nullptr;       // (m+1) x N Krylov basis (FP32)
  double *d_t = nullptr, *d_w = nullptr, *d_r = nullptr, *d_xs = nullptr;
  float *d_t32 = nullptr, *d_w32 = nullptr;
  double *d_Z = nullptr;        // m x N preconditioned vectors (flexible GMRES)
  cudaGraphExec_t prec64 = nullptr, prec32 = nullptr;  // captured ILU solves on d_t / d_t32
  unsigned *d_flags = nullptr;  // sync-free sweeps: [4] error word
  void *d_sweep_y = nullptr;    // sync-free sweeps: the L sweep's output (N values)
  int trsv_grid = 0, prep_grid = 0;
  int trsv_grid_warp = 0;
  // sync-free sweeps with one warp per node (short rows), per precision
  bool warp_sweep32 = false, warp_sweep64 = false;
  int check_trsv_error();
  // level-scheduled sweeps from a captured graph (else the sync-free ones)
  bool use_level_graph() const;
  static constexpr int kMaxGraphLevels = 64;  // automatic mode: graph up to this depth
  ~Solver();
  int init(Context *c, int krylov);
  // ILU(0) factors of the scaled matrix vals (FP64, or FP32 with the FP32
  // matrix copy); refresh() only points the solve at a new matrix (and
  // refreshes the FP32 copy), keeping the last factors as preconditioner
  int factor(const double *vals, bool fp32, cudaStream_t st);
  int refresh(const double *vals, bool fp32, cudaStream_t st);
  bool has_factors(bool fp32) const { return fp32 ? have_lu32 : have_lu64; }
  bool have_lu64 = false, have_lu32 = false;
  // the last factors (CSR order, FP64 or FP32 ones widened) to host memory
  int copy_factors(double *host, bool fp32, cudaStream_t st);
  int apply_prec64(cudaStream_t st);  // in place on d_t
  int apply_prec32(cudaStream_t st);  // in place on d_t32
};

struct LinearOpts {
  int krylov = 30;          // "Size of Krylov subspace"
  int maxit = 500;          // "Maximum Linear Solve Iterations"
  double tol = 1e-6;        // "Linear Solver Tolerance" (relative residual)
  bool fp32_inner = false;  // FP32 GMRES inside FP64 iterative refinement
  bool fp32_prec = false;   // FP64 flexible GMRES, ILU(0) factorised and applied in FP32
  double inner_tol = 1e-3;  // FP32 inner relative tolerance
  bool fp32_factors() const { return fp32_inner || fp32_prec; }
  int max_refinements = 20;
};
struct LinearStats {
  int iterations = 0;
  int refinements = 0;
  double relres = 0.0;
};

int device_norms(Context *C, const double *x, int n, double out3[3], cudaStream_t st);
int row_sum_scale(Context *C, double *vals, double *R, cudaStream_t st);
int linear_solve(Context *C, const double *R, double *dx, const LinearOpts &o, LinearStats *s,
                 cudaStream_t st);

}  // namespace gb
