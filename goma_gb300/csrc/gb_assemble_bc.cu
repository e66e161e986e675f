// Integrated (weak) boundary conditions on element sides: the surface terms
// apply_integrated_bc adds (src/mm_fill.c:2976, src/bc_integ.c), in FP64 on
// sm_103a.
//
// One warp per side.  Lanes first take the side's Gauss points (3 on a
// QUAD9 edge, 3 x 3 on a HEX27 face, find_surf_st src/el_elm_info.c:1987):
// the side's tangents from its nodes, the surface determinant sdet and the
// outward unit normal, the temperature, and the boundary function
//   QSIDE          func = q                         (src/bc_integ.c:1518)
//   QCONV          func = h (T_inf - T), dfunc/dT_j = -h phi_j
//                  (qrad_surf without radiation, src/mm_ns_bc.c:15145)
//   FLOW_PRESSURE  func_a = -P n_a                   (flow_n_dot_T_hydro,
//                  src/mm_ns_bc.c:6057)
// Then lanes take the side's nodes: R_i += sum_q w_q sdet_q phi_i(q) func(q)
// (:2207), and the QCONV Jacobian over node pairs.  Rows with a Dirichlet
// card are left to it, as put_dirichlet_in_matrix overwrites them
// (src/bc_dirich.c:44).  Sides of different elements share nodes, so the
// adds are atomic; the launch follows the element kernels on the same
// stream.
#include <cuda_runtime.h>

#include <cstdint>

#include "gb_device.h"

namespace gb {

namespace sd {

// local nodes (Goma order, 0-based) of the Exodus sides: corners, mid-edges
// (, face centre)
__constant__ int c_side2[4][3] = {{0, 1, 4}, {1, 2, 5}, {2, 3, 6}, {3, 0, 7}};
__constant__ int c_side3[6][9] = {{0, 1, 5, 4, 8, 13, 16, 12, 25},
                                  {1, 2, 6, 5, 9, 14, 17, 13, 24},
                                  {2, 3, 7, 6, 10, 15, 18, 14, 26},
                                  {0, 4, 7, 3, 12, 19, 15, 11, 23},
                                  {0, 3, 2, 1, 11, 10, 9, 8, 21},
                                  {4, 5, 6, 7, 16, 17, 18, 19, 22}};
// reference-coordinate grid offsets (0, 1, 2 for -1, 0, +1) of the local nodes
__constant__ int c_loc2[9][2] = {{0, 0}, {2, 0}, {2, 2}, {0, 2}, {1, 0},
                                 {2, 1}, {1, 2}, {0, 1}, {1, 1}};
__constant__ int c_loc3[27][3] = {
    {0, 0, 0}, {2, 0, 0}, {2, 2, 0}, {0, 2, 0}, {0, 0, 2}, {2, 0, 2}, {2, 2, 2},
    {0, 2, 2}, {1, 0, 0}, {2, 1, 0}, {1, 2, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 1},
    {2, 2, 1}, {0, 2, 1}, {1, 0, 2}, {2, 1, 2}, {1, 2, 2}, {0, 1, 2}, {1, 1, 1},
    {1, 1, 0}, {1, 1, 2}, {0, 1, 1}, {2, 1, 1}, {1, 0, 1}, {1, 2, 1}};
// the fixed reference coordinate of each side and its value
__constant__ int c_fix2[4][2] = {{1, -1}, {0, 1}, {1, 1}, {0, -1}};
__constant__ int c_fix3[6][2] = {{1, -1}, {0, 1}, {1, 1}, {0, -1}, {2, -1}, {2, 1}};

// the 1-D quadratic Lagrange factors of the nodes at -1, 0, +1
__device__ __forceinline__ double lag(int g, double s) {
  return g == 0 ? 0.5 * s * (s - 1.0) : (g == 1 ? 1.0 - s * s : 0.5 * s * (s + 1.0));
}
__device__ __forceinline__ double dlag(int g, double s) {
  return g == 0 ? s - 0.5 : (g == 1 ? -2.0 * s : s + 0.5);
}

constexpr int kWarps = 4;

template <int DIM>
struct WarpSmem {
  static constexpr int NS = DIM == 2 ? 3 : 9;
  double X[NS][DIM];
  double T[NS];
  double phi[NS][NS];  // [point][side node]
  double wsd[NS];      // Gauss weight x sdet
  double f[NS][DIM];   // func per point (energy: [q][0]; pressure: per component)
  double xc[DIM];      // element centre
};

}  // namespace sd

template <int DIM>
__global__ void __launch_bounds__(sd::kWarps * 32)
    assemble_side_kernel(AsmArgs A, SideArgs S, int energy) {
  using namespace sd;
  constexpr int NN = DIM == 2 ? 9 : 27, NS = DIM == 2 ? 3 : 9, CENT = DIM == 2 ? 8 : 20;
  __shared__ WarpSmem<DIM> smem[kWarps];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int k = blockIdx.x * kWarps + w;
  if (k >= S.num_sides) return;
  WarpSmem<DIM> &W = smem[w];
  const int e = S.elem[k], side = S.side[k], type = S.type[k];
  const double v0 = S.val[2 * k], v1 = S.val[2 * k + 1];
  const int *cn = A.conn + (int64_t)e * NN;
  auto side_loc = [&](int m) { return DIM == 2 ? c_side2[side - 1][m] : c_side3[side - 1][m]; };
  auto grid = [&](int l, int r) { return DIM == 2 ? c_loc2[l][r] : c_loc3[l][r]; };
  const int fi = DIM == 2 ? c_fix2[side - 1][0] : c_fix3[side - 1][0];
  const double fv = DIM == 2 ? c_fix2[side - 1][1] : c_fix3[side - 1][1];
  int fr[2] = {0, 0};
  {
    int nf = 0;
    for (int r = 0; r < DIM; r++)
      if (r != fi) fr[nf++] = r;
  }
  // the side's nodal coordinates and temperatures, the element centre
  if (lane < NS) {
    const int n = cn[side_loc(lane)];
#pragma unroll
    for (int j = 0; j < DIM; j++) W.X[lane][j] = A.coords[(int64_t)n * DIM + j];
    W.T[lane] = energy ? A.x[A.fu[n] + DIM] : 0.0;
  }
  if (lane < DIM) W.xc[lane] = A.coords[(int64_t)cn[CENT] * DIM + lane];
  __syncwarp();
  // per Gauss point
  if (lane < NS) {
    const int q = lane;
    double xi[3] = {0.0, 0.0, 0.0};
    const double gp[3] = {A.tab_pt[0], A.tab_pt[1], A.tab_pt[2]};
    const double gw[3] = {0.55555555555555555556, 0.88888888888888888888,
                          0.55555555555555555556};
    xi[fi] = fv;
    xi[fr[0]] = gp[q % 3];
    double wq = gw[q % 3];
    if (DIM == 3) {
      xi[fr[1]] = gp[q / 3];
      wq *= gw[q / 3];
    }
    double t[2][DIM], xq[DIM], T = 0.0;
#pragma unroll
    for (int j = 0; j < DIM; j++) {
      t[0][j] = t[1][j] = 0.0;
      xq[j] = 0.0;
    }
    for (int m = 0; m < NS; m++) {
      const int l = side_loc(m);
      double ph = 1.0, d[2] = {1.0, 1.0};
      for (int r = 0; r < DIM; r++) {
        const double lv = lag(grid(l, r), xi[r]), dv = dlag(grid(l, r), xi[r]);
        ph *= lv;
        d[0] *= r == fr[0] ? dv : lv;
        if (DIM == 3) d[1] *= r == fr[1] ? dv : lv;
      }
      W.phi[q][m] = ph;
#pragma unroll
      for (int j = 0; j < DIM; j++) {
        xq[j] = fma(ph, W.X[m][j], xq[j]);
        t[0][j] = fma(d[0], W.X[m][j], t[0][j]);
        if (DIM == 3) t[1][j] = fma(d[1], W.X[m][j], t[1][j]);
      }
      T = fma(ph, W.T[m], T);
    }
    double n[DIM], sdet;
    if (DIM == 2) {
      sdet = sqrt(t[0][0] * t[0][0] + t[0][1] * t[0][1]);
      n[0] = t[0][1] / sdet;
      n[1] = -t[0][0] / sdet;
    } else {
      const double c0 = t[0][1] * t[1][2] - t[0][2] * t[1][1];
      const double c1 = t[0][2] * t[1][0] - t[0][0] * t[1][2];
      const double c2 = t[0][0] * t[1][1] - t[0][1] * t[1][0];
      sdet = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
      n[0] = c0 / sdet;
      n[DIM > 1 ? 1 : 0] = c1 / sdet;
      n[DIM - 1] = c2 / sdet;
    }
    double o = 0.0;
#pragma unroll
    for (int j = 0; j < DIM; j++) o += n[j] * (xq[j] - W.xc[j]);
    if (o < 0.0)
#pragma unroll
      for (int j = 0; j < DIM; j++) n[j] = -n[j];
    W.wsd[q] = wq * sdet;
    if (type == GB_IBC_QSIDE) {
      W.f[q][0] = v0;
    } else if (type == GB_IBC_QCONV) {
      W.f[q][0] = v0 * (v1 - T);
    } else {
#pragma unroll
      for (int a = 0; a < DIM; a++) W.f[q][a] = -v0 * n[a];
    }
  }
  __syncwarp();
  // residual rows of the side's nodes
  if (lane < NS) {
    const int m = lane, node = cn[side_loc(m)], f0 = A.fu[node];
    if (type == GB_IBC_FLOW_PRESSURE) {
#pragma unroll
      for (int a = 0; a < DIM; a++) {
        double r = 0.0;
        for (int q = 0; q < NS; q++) r = fma(W.wsd[q] * W.phi[q][m], W.f[q][a], r);
        if (!A.dbc[f0 + a]) atomicAdd(A.R + f0 + a, r);
      }
    } else {
      double r = 0.0;
      for (int q = 0; q < NS; q++) r = fma(W.wsd[q] * W.phi[q][m], W.f[q][0], r);
      if (!A.dbc[f0 + DIM]) atomicAdd(A.R + f0 + DIM, r);
    }
  }
  // the QCONV Jacobian: J(T_i, T_j) += sum_q w sdet phi_i (-h phi_j)
  if (A.vals && type == GB_IBC_QCONV) {
    for (int p = lane; p < NS * NS; p += 32) {
      const int mi = p / NS, mj = p - mi * NS;
      const int li = side_loc(mi), lj = side_loc(mj);
      const int ni = cn[li], gr = A.fu[ni] + DIM;
      if (A.dbc[gr]) continue;
      double v = 0.0;
      for (int q = 0; q < NS; q++) v = fma(W.wsd[q] * W.phi[q][mi], -v0 * W.phi[q][mj], v);
      const int slot = A.elem_nslot[(int64_t)e * NN * NN + li * NN + lj];
      atomicAdd(A.vals + A.rowptr[gr] + A.nbr_offT[A.nbr_ptr[ni] + slot] + DIM, v);
    }
  }
}

cudaError_t launch_assemble_sides(const AsmArgs &a, const SideArgs &s, int dim, bool energy,
                                  cudaStream_t st) {
  if (s.num_sides <= 0) return cudaSuccess;
  const int grid = (s.num_sides + sd::kWarps - 1) / sd::kWarps;
  if (dim == 2)
    assemble_side_kernel<2><<<grid, sd::kWarps * 32, 0, st>>>(a, s, energy ? 1 : 0);
  else
    assemble_side_kernel<3><<<grid, sd::kWarps * 32, 0, st>>>(a, s, energy ? 1 : 0);
  return cudaGetLastError();
}

}  // namespace gb
