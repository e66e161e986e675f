// 3-D element Jacobian on the FP64 tensor pipe (DMMA, mma.sync m8n8k4 f64).
//
// Same physics and the same results (to rounding) as the scalar kernel of
// gb_assemble.cu -- assemble_momentum / assemble_continuity /
// assemble_energy of the reference (src/mm_fill_momentum.c:100,
// src/mm_fill_continuity.c:119, src/mm_fill_energy.c:109) -- with the
// velocity/temperature blocks of the element Jacobian written as sums of
// basis x basis contractions over the 27 quadrature points:
//
//   J_ab(i,j) = sum_q phi_i c_ab phi_j + sum_q d_b phi_i (-mu dA) d_a phi_j
//             + delta_ab [ sum_q phi_i CK_j + sum_p sum_q d_p phi_i (-mu dA) d_p phi_j ]
//             (+ Carreau: sum_q gm_i[a] (-cmu dA) gm_j[b])
//   J_TT       = sum_q phi_i Cp CK_j + sum_p sum_q d_p phi_i (-k dA) d_p phi_j
//   J_Tv_b     = sum_q phi_i (-rho Cp dA dT/dx_b) phi_j
//   J_vT_a     = sum_q phi_i (dA df_a/dT) phi_j
//
// with c_ab = -rho dA dv_a/dx_b and CK_j = -rho dA v . grad phi_j.  Each
// term is an (27 x 28) x (28 x 27) product of two shared-memory tables
// (phi, physical grad phi, CK, and for Carreau grad phi . gamma), with the
// per-quadrature-point coefficient folded into the A fragment.  Eight warps
// own two 32 x 32 blocks each (16 accumulator tiles of 8 x 8).  The residual
// and the pressure couplings stay on the scalar path; the scatter is the
// coloured read-modify-write of gb_assemble.cu.
#include <cuda_runtime.h>

#include <cstdint>

#include "gb_device.h"
#include "gb_element.cuh"

namespace gb {

namespace tc {

constexpr int NN = 27, NQ = 27, NP = 4, CENT = 20;
constexpr int QP_PAD = 28;  // quadrature points padded to a multiple of 4 (k-step)
constexpr int LD = 36;      // row stride of the tables: conflict-free fragment loads
constexpr int TAB = QP_PAD * LD;

// table ids
enum { T_PHI = 0, T_G0, T_G1, T_G2, T_CK, T_GM0, T_GM1, T_GM2 };
// coefficient ids (per quadrature point)
enum {
  C_AB = 0,        // 9: -rho dA gv[b][a], index a*3+b
  C_NMU = 9,       // -mu dA
  C_NK = 10,       // -k dA
  C_TV = 11,       // 3: -rho Cp dA gT[b]
  C_VT = 14,       // 3: dA dfT[a]
  C_CP = 17,       // Cp
  C_NCMU = 18,     // -cmu dA
  C_ONE = 19,      // 1
  NCOEF = 20
};
static_assert(C_VT == C_TV + 3 && C_CP == C_VT + 3, "coefficient ids overlap");

struct Smem {
  double X[NN][3], U[NN][3], Tn[NN], Pn[NP];
  int nodes[NN];
  int e;
  QP<3> qp[NQ];
  double coef[NCOEF][QP_PAD];
  double tab[8][TAB];  // PHI, G0..2, CK, GM0..2 (GM only with Carreau)
};

__device__ __forceinline__ void dmma(double (&c)[2], double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(c[0]), "+d"(c[1])
               : "d"(a), "d"(b));
}

// acc += sum over the padded quadrature points of (A * coef) x B
__device__ __forceinline__ void product(double (&acc)[16][2], const double *__restrict__ A,
                                        const double *__restrict__ cf,
                                        const double *__restrict__ B, int lane) {
  const int r = lane >> 2, c = lane & 3;
#pragma unroll
  for (int ks = 0; ks < QP_PAD / 4; ks++) {
    const int q = ks * 4 + c;
    const double s = cf[q];
    double a[4], b[4];
#pragma unroll
    for (int it = 0; it < 4; it++) a[it] = A[q * LD + it * 8 + r] * s;
#pragma unroll
    for (int jt = 0; jt < 4; jt++) b[jt] = B[q * LD + jt * 8 + r];
#pragma unroll
    for (int it = 0; it < 4; it++)
#pragma unroll
      for (int jt = 0; jt < 4; jt++) dmma(acc[it * 4 + jt], a[it], b[jt]);
  }
}

// block ids: 0..8 velocity (a*3+b), 9 TT, 10..12 T-row/v_b, 13..15 v_a-row/T
template <bool CARREAU>
__device__ __forceinline__ void run_block(double (&acc)[16][2], int blk, Smem &S, int lane) {
#pragma unroll
  for (int t = 0; t < 16; t++) acc[t][0] = acc[t][1] = 0.0;
  const double *tab = &S.tab[0][0];
  auto T = [&](int id) { return tab + id * TAB; };
  auto C = [&](int id) { return &S.coef[id][0]; };
  if (blk < 9) {
    const int a = blk / 3, b = blk - (blk / 3) * 3;
    product(acc, T(T_PHI), C(C_AB + blk), T(T_PHI), lane);
    product(acc, T(T_G0 + b), C(C_NMU), T(T_G0 + a), lane);
    if (a == b) {
      product(acc, T(T_PHI), C(C_ONE), T(T_CK), lane);
      product(acc, T(T_G0), C(C_NMU), T(T_G0), lane);
      product(acc, T(T_G1), C(C_NMU), T(T_G1), lane);
      product(acc, T(T_G2), C(C_NMU), T(T_G2), lane);
    }
    if (CARREAU) product(acc, T(T_GM0 + a), C(C_NCMU), T(T_GM0 + b), lane);
  } else if (blk == 9) {
    product(acc, T(T_PHI), C(C_CP), T(T_CK), lane);
    product(acc, T(T_G0), C(C_NK), T(T_G0), lane);
    product(acc, T(T_G1), C(C_NK), T(T_G1), lane);
    product(acc, T(T_G2), C(C_NK), T(T_G2), lane);
  } else if (blk < 13) {
    product(acc, T(T_PHI), C(C_TV + blk - 10), T(T_PHI), lane);
  } else {
    product(acc, T(T_PHI), C(C_VT + blk - 13), T(T_PHI), lane);
  }
}

// coloured read-modify-write of one 27 x 27 block
template <bool ENERGY>
__device__ __forceinline__ void scatter_block(const double (&acc)[16][2], int blk, const Smem &S,
                                              const AsmArgs &A, const uint16_t *nslot, int lane) {
  constexpr int DIM = 3;
  int rvar, cvar;
  if (blk < 9) {
    rvar = blk / 3;
    cvar = blk - rvar * 3;
  } else if (blk == 9) {
    rvar = DIM;
    cvar = DIM;
  } else if (blk < 13) {
    rvar = DIM;
    cvar = blk - 10;
  } else {
    rvar = blk - 13;
    cvar = DIM;
  }
  const bool rowT = ENERGY && rvar == DIM;
  const int r = lane >> 2, c = lane & 3;
#pragma unroll
  for (int it = 0; it < 4; it++) {
    const int i = it * 8 + r;
    if (i >= NN) continue;
    const int ni = S.nodes[i];
    const int gr = A.fu[ni] + rvar;
    if (A.dbc[gr]) continue;
    const int64_t rb = A.rowptr[gr];
    const int nb0 = A.nbr_ptr[ni];
#pragma unroll
    for (int jt = 0; jt < 4; jt++)
#pragma unroll
      for (int e2 = 0; e2 < 2; e2++) {
        const int j = jt * 8 + 2 * c + e2;
        if (j >= NN) continue;
        const int s = nslot[i * NN + j];
        const int off = rowT ? A.nbr_offT[nb0 + s] : A.nbr_off[nb0 + s];
        A.vals[rb + off + cvar] += acc[it * 4 + jt][e2];
      }
  }
}

}  // namespace tc

template <bool ENERGY, bool CARREAU>
__global__ void __launch_bounds__(256, 1)
    assemble_tc_kernel(AsmArgs A, const int *__restrict__ elems, int nelem) {
  using namespace tc;
  constexpr int DIM = 3;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem &S = *reinterpret_cast<Smem *>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const MaterialDev M = A.mat;
  const double *__restrict__ tab_phi = A.tab_phi;
  const double *__restrict__ tab_dphi = A.tab_dphi;
  const int ntab = CARREAU ? 8 : 5;
  // zero every table once (padding rows and columns stay zero), then the
  // constant phi table
  for (int t = tid; t < ntab * TAB; t += blockDim.x) (&S.tab[0][0])[t] = 0.0;
  for (int t = tid; t < NCOEF * QP_PAD; t += blockDim.x) (&S.coef[0][0])[t] = 0.0;
  __syncthreads();
  for (int t = tid; t < NQ * NN; t += blockDim.x) {
    const int q = t / NN, k = t - q * NN;
    S.tab[T_PHI][q * LD + k] = tab_phi[q * NN + k];
  }
  // warp roles: two blocks each
  int blk0, blk1;
  if (ENERGY) {
    const int roles[8][2] = {{0, 13}, {4, 14}, {8, 15}, {1, 2}, {3, 5}, {6, 7}, {9, 10}, {11, 12}};
    blk0 = roles[warp][0];
    blk1 = roles[warp][1];
  } else {
    const int roles[8][2] = {{0, -1}, {4, -1}, {8, -1}, {1, 2}, {3, 5}, {6, 7}, {-1, -1}, {-1, -1}};
    blk0 = roles[warp][0];
    blk1 = roles[warp][1];
  }

  for (int ei = blockIdx.x; ei < nelem; ei += gridDim.x) {
    const int e = elems[ei];
    __syncthreads();  // previous element's tables fully consumed
    for (int k = tid; k < NN; k += blockDim.x) {
      const int n = A.conn[(int64_t)e * NN + k];
      S.nodes[k] = n;
      const int f0 = A.fu[n];
#pragma unroll
      for (int j = 0; j < DIM; j++) {
        S.X[k][j] = A.coords[(int64_t)n * DIM + j];
        S.U[k][j] = A.x[f0 + j];
      }
      S.Tn[k] = ENERGY ? A.x[f0 + DIM] : 0.0;
      if (k == CENT)
        for (int l = 0; l < NP; l++) S.Pn[l] = A.x[f0 + A.pofs + l];
    }
    if (tid == 0) S.e = e;
    __syncthreads();
    // phase 1: quadrature points
    if (tid < NQ)
      qp_setup<DIM, ENERGY, CARREAU>(S.X, S.U, S.Tn, S.Pn, tid, tab_phi, tab_dphi, A.tab_w,
                                     A.tab_pt, M, M.density, S.qp[tid]);
    __syncthreads();
    // phase 2: tables and coefficients
    for (int t = tid; t < NQ * NN; t += blockDim.x) {
      const int q = t / NN, k = t - q * NN;
      const QP<DIM> &Q = S.qp[q];
      double g[DIM];
      double vg = 0.0;
#pragma unroll
      for (int p = 0; p < DIM; p++) {
        double s2 = 0.0;
#pragma unroll
        for (int i = 0; i < DIM; i++) s2 = fma(Q.B[p][i], tab_dphi[(q * NN + k) * DIM + i], s2);
        g[p] = s2;
        S.tab[T_G0 + p][q * LD + k] = s2;
        vg = fma(Q.v[p], s2, vg);
      }
      S.tab[T_CK][q * LD + k] = -M.density * Q.dA * vg;
      if (CARREAU) {
#pragma unroll
        for (int a = 0; a < DIM; a++) {
          double s2 = 0.0;
#pragma unroll
          for (int p = 0; p < DIM; p++) s2 = fma(g[p], Q.gam[a][p], s2);
          S.tab[T_GM0 + a][q * LD + k] = s2;
        }
      }
    }
    if (tid < NQ) {
      const int q = tid;
      const QP<DIM> &Q = S.qp[q];
      const double dA = Q.dA;
#pragma unroll
      for (int a = 0; a < DIM; a++)
#pragma unroll
        for (int b = 0; b < DIM; b++) S.coef[C_AB + a * 3 + b][q] = -M.density * dA * Q.gv[b][a];
      S.coef[C_NMU][q] = -Q.mu * dA;
      S.coef[C_NK][q] = -M.conductivity * dA;
#pragma unroll
      for (int b = 0; b < DIM; b++) {
        S.coef[C_TV + b][q] = ENERGY ? -M.density * M.heat_capacity * dA * Q.gT[b] : 0.0;
        S.coef[C_VT + b][q] = ENERGY ? dA * Q.dfT[b] : 0.0;
      }
      S.coef[C_CP][q] = M.heat_capacity;
      S.coef[C_NCMU][q] = CARREAU ? -Q.cmu * dA : 0.0;
      S.coef[C_ONE][q] = 1.0;
    }
    __syncthreads();

    // scalar part: residual rows, J_m_P (= J_c_v transposed), Dirichlet diagonals
    constexpr int NRM = DIM * NN;
    const bool own_m = tid < NRM;
    const bool own_T = ENERGY && tid >= NRM && tid < NRM + NN;
    const bool own_c = tid >= NRM + (ENERGY ? NN : 0) && tid < NRM + (ENERGY ? NN : 0) + NP;
    const int ra = tid / NN, ri = tid - (tid / NN) * NN;
    const int rT = tid - NRM;
    const int rc = tid - NRM - (ENERGY ? NN : 0);
    double Racc = 0.0, JmP[NP] = {0.0, 0.0, 0.0, 0.0};
    bool bad = false;
    for (int q = 0; q < NQ; q++) {
      const QP<DIM> &Q = S.qp[q];
      const double dA = Q.dA;
      bad |= Q.bad;
      if (own_m) {
        const double phi = S.tab[T_PHI][q * LD + ri];
        double gi[DIM];
#pragma unroll
        for (int p = 0; p < DIM; p++) gi[p] = S.tab[T_G0 + p][q * LD + ri];
        double adv = 0.0;
#pragma unroll
        for (int p = 0; p < DIM; p++) adv = fma(Q.v[p], Q.gv[p][ra], adv);
        adv = adv * M.density * (-phi * dA);
        double dif = 0.0;
#pragma unroll
        for (int p = 0; p < DIM; p++)
          dif = fma(gi[p], (p == ra ? -Q.P : 0.0) + Q.mu * Q.gam[ra][p], dif);
        dif *= -dA;
        Racc += adv + dif + Q.f[ra] * (phi * dA);
#pragma unroll
        for (int l = 0; l < NP; l++) JmP[l] = fma(gi[ra] * Q.psi[l], dA, JmP[l]);
      } else if (own_T) {
        const double phi = S.tab[T_PHI][q * LD + rT];
        double vgT = 0.0, dif = 0.0;
#pragma unroll
        for (int p = 0; p < DIM; p++) {
          vgT = fma(Q.v[p], Q.gT[p], vgT);
          dif = fma(S.tab[T_G0 + p][q * LD + rT], -M.conductivity * Q.gT[p], dif);
        }
        Racc += vgT * (-phi * M.density * M.heat_capacity * dA) + dif * dA;
      } else if (own_c) {
        double divv = 0.0;
#pragma unroll
        for (int a = 0; a < DIM; a++) divv += Q.gv[a][a];
        Racc += divv * (Q.psi[rc] * dA);
      }
    }
    if (bad && tid == 0) {
      atomicAdd(A.status, 1);
      atomicMin(A.status + 1, e);
    }

    // tensor-pipe part: mma.sync.aligned needs the whole warp converged, and
    // the residual owners above diverge inside warps
    __syncwarp();
    double acc0[16][2], acc1[16][2];
    if (blk0 >= 0) run_block<CARREAU>(acc0, blk0, S, lane);
    if (blk1 >= 0) run_block<CARREAU>(acc1, blk1, S, lane);

    // scatter (no other element of this colour touches these rows)
    const uint16_t *nslot = A.elem_nslot + (int64_t)e * NN * NN;
    if (own_m || own_T || own_c) {
      int gr, node, k, rowvar;
      if (own_m) {
        k = ri;
        node = S.nodes[ri];
        gr = A.fu[node] + ra;
        rowvar = ra;
      } else if (own_T) {
        k = rT;
        node = S.nodes[rT];
        gr = A.fu[node] + DIM;
        rowvar = DIM;
      } else {
        k = CENT;
        node = S.nodes[CENT];
        gr = A.fu[node] + A.pofs + rc;
        rowvar = A.pofs + rc;
      }
      const bool dir = A.dbc[gr] != 0;
      if (!dir) A.R[gr] += Racc;
      const int64_t rb = A.rowptr[gr];
      const int nb0 = A.nbr_ptr[node];
      const bool rowT = ENERGY && rowvar == DIM;
      if (dir) {
        const int s = nslot[k * NN + k];
        const int off = rowT ? A.nbr_offT[nb0 + s] : A.nbr_off[nb0 + s];
        A.vals[rb + off + rowvar] += 1.0;
      } else if (own_m) {
        const int s = nslot[k * NN + CENT];
        const int64_t base = rb + A.nbr_off[nb0 + s] + A.pofs;
#pragma unroll
        for (int l = 0; l < NP; l++) A.vals[base + l] += JmP[l];
      }
    }
    if (own_m) {
      const int nc = S.nodes[CENT];
      const int s = nslot[CENT * NN + ri];
      const int nb0 = A.nbr_ptr[nc];
      const int off = A.nbr_off[nb0 + s] + ra;
#pragma unroll
      for (int l = 0; l < NP; l++) {
        const int gr = A.fu[nc] + A.pofs + l;
        if (A.dbc[gr]) continue;
        A.vals[A.rowptr[gr] + off] += JmP[l];
      }
    }
    if (blk0 >= 0) scatter_block<ENERGY>(acc0, blk0, S, A, nslot, lane);
    if (blk1 >= 0) scatter_block<ENERGY>(acc1, blk1, S, A, nslot, lane);
  }
}

template <bool ENERGY, bool CARREAU>
static cudaError_t launch_tc_t(const AsmArgs &a, const int *elems, int nelem, int grid_cap,
                               cudaStream_t st) {
  const size_t sm = sizeof(tc::Smem) - (CARREAU ? 0 : 3 * sizeof(double) * tc::TAB);
  auto k = assemble_tc_kernel<ENERGY, CARREAU>;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const int grid = nelem < grid_cap ? nelem : grid_cap;
  if (grid <= 0) return cudaSuccess;
  k<<<grid, 256, sm, st>>>(a, elems, nelem);
  return cudaGetLastError();
}

cudaError_t launch_assemble_tc(const AsmArgs &a, bool energy, bool carreau, const int *elems,
                               int nelem, int grid_cap, cudaStream_t st) {
  if (energy) {
    return carreau ? launch_tc_t<true, true>(a, elems, nelem, grid_cap, st)
                   : launch_tc_t<true, false>(a, elems, nelem, grid_cap, st);
  }
  return carreau ? launch_tc_t<false, true>(a, elems, nelem, grid_cap, st)
                 : launch_tc_t<false, false>(a, elems, nelem, grid_cap, st);
}

}  // namespace gb
