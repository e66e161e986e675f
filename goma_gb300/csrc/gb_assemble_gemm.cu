// 3-D Q2/P1 element residual + analytic Jacobian (Newtonian Navier-Stokes,
// optional energy with a Boussinesq body force) written as dense products on
// the FP64 tensor pipe (DMMA, mma.sync m8n8k4 f64), with the coloured CSR
// scatter.
//
// Same physics and results (to rounding) as the scalar kernel of
// gb_assemble.cu, i.e. the reference's assemble_momentum
// (src/mm_fill_momentum.c:100, fluid_stress :2834), assemble_continuity
// (src/mm_fill_continuity.c:119), assemble_energy (src/mm_fill_energy.c:109),
// bouss_momentum_source (src/mm_std_models.c:125), the hard-set Dirichlet rows
// of put_dirichlet_in_matrix (src/bc_dirich.c:44) and the load_lec scatter
// (src/mm_fill.c:5175).
//
// On GB300 one scalar FP64 warp instruction (32 FMA) holds a partition's
// FP64 pipe about half as long as one DMMA (256 FMA), so the kernel moves
// every contraction over quadrature points or nodes onto DMMA and keeps the
// scalar FP64 work to the operand tables (O(27 x 27) per element):
//
//   isoparametric product  [phi; dphi/dxi_r](q, k) x [x y z u v w T](k)
//                          -> field values and reference gradients at the
//                          27 points (beer_belly / load_fv, 98 DMMA)
//   per point (27 lanes)   J^-1, det J, grad v, grad T and the weights below
//   operand tables         G_p = d phi / d x_p, mG_p = -mu dA G_p,
//                          CK = -rho dA v . grad phi   ([q][node], 28 x 36)
//   Jacobian blocks, with phi^T(w) = phi scaled by a per-point weight w:
//     J_ab   = phi^T(-rho dA dv_a/dx_b) phi + G_b mG_a^T
//              + delta_ab (S1 + S2),   S1 = phi CK^T,  S2 = sum_p G_p mG_p^T
//     J_TT   = Cp S1 + (k / mu) S2
//     J_Tv_b = phi^T(-rho Cp dA dT/dx_b) phi
//     J_vT_a = (df_a/dT) phi^T(dA) phi       (Boussinesq: df/dT is constant)
//     J_mP   = G_a (psi_l dA),  J_cv = J_mP^T
//   residual  R_a = phi (dA(-rho v.grad v_a + f_a)) + sum_p G_p (-dA Pi_pa),
//             R_T = phi (-rho Cp dA v.grad T) + sum_p G_p (-k dA dT/dx_p),
//             R_c = sum_q psi_l dA div v
//
// Each 27 x 27 block is 4 x 4 accumulator tiles of 8 x 8 (27 padded to 32,
// the 27 points padded to 28).  Eight warps own the blocks (two stages: the
// shared S1 / S2 are staged through shared memory between them); two CTAs
// share an SM so one's scalar set-up overlaps the other's products.  The
// scatter is the coloured read-modify-write: elements of one colour share
// no node, hence no CSR row, so there are no atomics and the result is
// deterministic.
#include <cuda_runtime.h>

#include <cstdint>

#include "gb_device.h"

namespace gb {

namespace gm {

constexpr int NN = 27, NQ = 27, NP = 4, CENT = 20;
constexpr int KP = 28;     // points (or nodes) padded to a multiple of the k-step 4
constexpr int LD = 36;     // row stride of a [q][node] table: conflict-free fragment loads
constexpr int LDS = 12;    // row stride of an 8-column table
constexpr int TABN = KP * LD;
constexpr int NISO = 112;  // rows of the isoparametric table (4 x 27 padded)

// per-point weights that scale the A operand
enum { W_AB = 0, W_TV = 9, W_DA = 12, NW = 13 };

struct Smem {
  double phi[TABN];      // phi_i(q) at [q][i] (constant)
  double G[3][TABN];     // d phi_i / d x_p (q)
  double mG[3][TABN];    // -mu dA d phi_i / d x_p
  double cK[TABN];       // -rho dA v . grad phi_i
  double w[NW][KP];
  double cR[KP * LDS];      // [q][n] residual, phi part: n = a (momentum), 3 (energy)
  double tR[3][KP * LDS];   // [p][q][n] residual, gradient part
  double psidA[KP * LDS];   // [q][l] psi_l dA
  double nod[KP * LDS];     // [k][f] x, y, z, u, v, w, T at node k
  double F[8][4][KP];       // isoparametric product: field f, (value, d/dxi_r), point
  double Bq[KP][9];         // J^-1 at each point, [p][r]
  double vq[KP][3];
  double dAq[KP];
  double S1[NN][KP], S2[NN][KP];
  double Pn[NP];
  int nodes[NN];
};

__device__ __forceinline__ void dmma(double (&c)[2], double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(c[0]), "+d"(c[1])
               : "d"(a), "d"(b));
}

__device__ __forceinline__ void zero(double (&acc)[16][2]) {
#pragma unroll
  for (int t = 0; t < 16; t++) acc[t][0] = acc[t][1] = 0.0;
}

// acc(i, j) += sum_q A[q][i] s[q] B[q][j] over the 4 x 4 tiles of a 32 x 32 block
template <bool SCALE>
__device__ __forceinline__ void prod44(double (&acc)[16][2], const double *A, const double *s,
                                       const double *B, int lane) {
  const int r = lane >> 2, c = lane & 3;
#pragma unroll
  for (int ks = 0; ks < KP / 4; ks++) {
    const int q = ks * 4 + c;
    double a[4], b[4];
#pragma unroll
    for (int it = 0; it < 4; it++) a[it] = A[q * LD + it * 8 + r];
    if (SCALE) {
      const double sc = s[q];
#pragma unroll
      for (int it = 0; it < 4; it++) a[it] *= sc;
    }
#pragma unroll
    for (int jt = 0; jt < 4; jt++) b[jt] = B[q * LD + jt * 8 + r];
#pragma unroll
    for (int it = 0; it < 4; it++)
#pragma unroll
      for (int jt = 0; jt < 4; jt++) dmma(acc[it * 4 + jt], a[it], b[jt]);
  }
}

// acc(i, n) += sum_q A[q][i] B[q][n]: 32 rows x one 8-column tile
__device__ __forceinline__ void prod41(double (&acc)[4][2], const double *A, const double *B,
                                       int lane) {
  const int r = lane >> 2, c = lane & 3;
#pragma unroll
  for (int ks = 0; ks < KP / 4; ks++) {
    const int q = ks * 4 + c;
    const double b = B[q * LDS + r];
#pragma unroll
    for (int it = 0; it < 4; it++) dmma(acc[it], A[q * LD + it * 8 + r], b);
  }
}

// coloured read-modify-write of one 27 x 27 block (row variable rv, column
// variable cv at each node), scaled by sc; Dirichlet rows are skipped
template <bool ENERGY>
__device__ __forceinline__ void scatter(const double (&acc)[16][2], int rv, int cv, double sc,
                                        const Smem &S, const AsmArgs &A, const uint16_t *nslot,
                                        int lane) {
  constexpr int DIM = 3;
  const bool rowT = ENERGY && rv == DIM;
  const int r = lane >> 2, c = lane & 3;
#pragma unroll
  for (int it = 0; it < 4; it++) {
    const int i = it * 8 + r;
    if (i >= NN) continue;
    const int ni = S.nodes[i];
    const int gr = A.fu[ni] + rv;
    if (A.dbc[gr]) continue;
    double *row = A.vals + A.rowptr[gr] + cv;
    const int *off = (rowT ? A.nbr_offT : A.nbr_off) + A.nbr_ptr[ni];
    const uint16_t *ns = nslot + i * NN;
#pragma unroll
    for (int jt = 0; jt < 4; jt++)
#pragma unroll
      for (int e2 = 0; e2 < 2; e2++) {
        const int j = jt * 8 + 2 * c + e2;
        if (j >= NN) continue;
        row[off[ns[j]]] += sc * acc[it * 4 + jt][e2];
      }
  }
}

// adds the shared diagonal term S1 + S2 to a 27 x 27 block
__device__ __forceinline__ void add_diag(double (&acc)[16][2], const Smem &S, int lane) {
  const int r = lane >> 2, c = lane & 3;
#pragma unroll
  for (int it = 0; it < 4; it++) {
    const int i = it * 8 + r;
    if (i >= NN) continue;
#pragma unroll
    for (int jt = 0; jt < 4; jt++)
#pragma unroll
      for (int e2 = 0; e2 < 2; e2++) {
        const int j = jt * 8 + 2 * c + e2;
        if (j < NN) acc[it * 4 + jt][e2] += S.S1[i][j] + S.S2[i][j];
      }
  }
}

__device__ __forceinline__ void store_block(const double (&acc)[16][2], double (*dst)[KP],
                                            int lane) {
  const int r = lane >> 2, c = lane & 3;
#pragma unroll
  for (int it = 0; it < 4; it++) {
    const int i = it * 8 + r;
    if (i >= NN) continue;
#pragma unroll
    for (int jt = 0; jt < 4; jt++)
#pragma unroll
      for (int e2 = 0; e2 < 2; e2++) {
        const int j = jt * 8 + 2 * c + e2;
        if (j < NN) dst[i][j] = acc[it * 4 + jt][e2];
      }
  }
}

// residual rows of the nodal equations (momentum, energy) of one element
template <bool ENERGY>
__device__ __forceinline__ void residual_rows(const Smem &S, const AsmArgs &A, int lane) {
  constexpr int DIM = 3;
  double accR[4][2];
#pragma unroll
  for (int it = 0; it < 4; it++) accR[it][0] = accR[it][1] = 0.0;
  prod41(accR, S.phi, S.cR, lane);
  prod41(accR, S.G[0], S.tR[0], lane);
  prod41(accR, S.G[1], S.tR[1], lane);
  prod41(accR, S.G[2], S.tR[2], lane);
  const int r = lane >> 2, c = lane & 3;
  if (c < 2) {
#pragma unroll
    for (int it = 0; it < 4; it++) {
      const int i = it * 8 + r;
      if (i >= NN) continue;
      const int f0 = A.fu[S.nodes[i]];
#pragma unroll
      for (int e2 = 0; e2 < 2; e2++) {
        const int n = 2 * c + e2;
        if (n == DIM && !ENERGY) continue;
        if (!A.dbc[f0 + n]) A.R[f0 + n] += accR[it][e2];
      }
    }
  }
}

// velocity block (a, b): phi^T(w_ab) phi + G_b mG_a^T
__device__ __forceinline__ void vel_block(double (&acc)[16][2], int a, int b, const Smem &S,
                                          int lane) {
  zero(acc);
  prod44<true>(acc, S.phi, S.w[W_AB + a * 3 + b], S.phi, lane);
  prod44<false>(acc, S.G[b], nullptr, S.mG[a], lane);
}

}  // namespace gm

template <bool ENERGY, bool JAC>
__global__ void __launch_bounds__(256, 2)
    assemble_gemm_kernel(AsmArgs A, const double *__restrict__ tab_iso,
                         const int *__restrict__ elems, int nelem) {
  using namespace gm;
  constexpr int DIM = 3;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem &S = *reinterpret_cast<Smem *>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const MaterialDev M = A.mat;
  const double *__restrict__ tab_dphi = A.tab_dphi;

  // every table starts at zero once: the padding rows and columns stay zero
  for (int t = tid; t < (int)(sizeof(Smem) / sizeof(double)); t += blockDim.x)
    reinterpret_cast<double *>(smem_raw)[t] = 0.0;
  __syncthreads();
  for (int t = tid; t < NQ * NN; t += blockDim.x) {
    const int q = t / NN, k = t - q * NN;
    S.phi[q * LD + k] = A.tab_phi[q * NN + k];
  }

  for (int ei = blockIdx.x; ei < nelem; ei += gridDim.x) {
    const int e = elems[ei];
    __syncthreads();  // the previous element's tables are consumed
    // ---- nodal data
    if (tid < NN) {
      const int k = tid;
      const int n = A.conn[(int64_t)e * NN + k];
      S.nodes[k] = n;
      const int f0 = A.fu[n];
#pragma unroll
      for (int j = 0; j < DIM; j++) {
        S.nod[k * LDS + j] = A.coords[(int64_t)n * DIM + j];
        S.nod[k * LDS + 3 + j] = A.x[f0 + j];
      }
      S.nod[k * LDS + 6] = ENERGY ? A.x[f0 + DIM] : 0.0;
      if (k == CENT)
        for (int l = 0; l < NP; l++) S.Pn[l] = A.x[f0 + A.pofs + l];
    }
    __syncthreads();
    // ---- isoparametric product: 14 row tiles x 7 k-steps
    {
      const int r = lane >> 2, c = lane & 3;
      for (int mt = warp; mt < NISO / 8; mt += 8) {
        double acc[2] = {0.0, 0.0};
#pragma unroll
        for (int ks = 0; ks < KP / 4; ks++) {
          const double a = __ldg(tab_iso + (mt * 8 + r) * KP + ks * 4 + c);
          const double b = S.nod[(ks * 4 + c) * LDS + r];
          dmma(acc, a, b);
        }
        const int row = mt * 8 + r;
        if (row < 4 * NQ) {
          const int d = row / NQ, q = row - d * NQ;
          S.F[2 * c][d][q] = acc[0];
          S.F[2 * c + 1][d][q] = acc[1];
        }
      }
    }
    __syncthreads();
    // ---- per quadrature point (warp 0): J^-1, det J, gradients, weights
    if (warp == 0) {
      const int q = lane;
      double rc[NP] = {0.0, 0.0, 0.0, 0.0};
      bool bad = false;
      if (q < NQ) {
        double Jm[3][3], Gh[3][3], Th[3], v[3];
#pragma unroll
        for (int r = 0; r < 3; r++) {
#pragma unroll
          for (int j = 0; j < 3; j++) {
            Jm[r][j] = S.F[j][1 + r][q];
            Gh[r][j] = S.F[3 + j][1 + r][q];
          }
          Th[r] = S.F[6][1 + r][q];
          v[r] = S.F[3 + r][0][q];
        }
        const double T = S.F[6][0][q];
        const double c00 = Jm[1][1] * Jm[2][2] - Jm[1][2] * Jm[2][1];
        const double c01 = Jm[1][0] * Jm[2][2] - Jm[1][2] * Jm[2][0];
        const double c02 = Jm[1][0] * Jm[2][1] - Jm[1][1] * Jm[2][0];
        const double det = Jm[0][0] * c00 - Jm[0][1] * c01 + Jm[0][2] * c02;
        bad = !(det > 0.0);
        const double id = 1.0 / det;
        double B[3][3];
        B[0][0] = c00 * id;
        B[0][1] = -(Jm[0][1] * Jm[2][2] - Jm[2][1] * Jm[0][2]) * id;
        B[0][2] = (Jm[0][1] * Jm[1][2] - Jm[1][1] * Jm[0][2]) * id;
        B[1][0] = -c01 * id;
        B[1][1] = (Jm[0][0] * Jm[2][2] - Jm[2][0] * Jm[0][2]) * id;
        B[1][2] = -(Jm[0][0] * Jm[1][2] - Jm[1][0] * Jm[0][2]) * id;
        B[2][0] = c02 * id;
        B[2][1] = -(Jm[0][0] * Jm[2][1] - Jm[2][0] * Jm[0][1]) * id;
        B[2][2] = (Jm[0][0] * Jm[1][1] - Jm[1][0] * Jm[0][1]) * id;
        const double dA = A.tab_w[q] * det;
        // gv[p][a] = d v_a / d x_p, gT[p] = dT / dx_p
        double gv[3][3], gT[3];
#pragma unroll
        for (int p = 0; p < 3; p++) {
#pragma unroll
          for (int a = 0; a < 3; a++)
            gv[p][a] = B[p][0] * Gh[0][a] + B[p][1] * Gh[1][a] + B[p][2] * Gh[2][a];
          gT[p] = B[p][0] * Th[0] + B[p][1] * Th[1] + B[p][2] * Th[2];
        }
        double psi[NP];
        psi[0] = 1.0;
        psi[1] = A.tab_pt[q % 3];
        psi[2] = A.tab_pt[(q % 9) / 3];
        psi[3] = A.tab_pt[q / 9];
        double P = 0.0;
#pragma unroll
        for (int l = 0; l < NP; l++) P = fma(S.Pn[l], psi[l], P);
        const double mu = M.viscosity, rho = M.density;
        const double divv = gv[0][0] + gv[1][1] + gv[2][2];
#pragma unroll
        for (int l = 0; l < NP; l++) {
          S.psidA[q * LDS + l] = psi[l] * dA;
          rc[l] = psi[l] * dA * divv;
        }
#pragma unroll
        for (int a = 0; a < 3; a++) {
#pragma unroll
          for (int b = 0; b < 3; b++) S.w[W_AB + a * 3 + b][q] = -rho * dA * gv[b][a];
          S.w[W_TV + a][q] = ENERGY ? -rho * M.heat_capacity * dA * gT[a] : 0.0;
          double f = M.source[a];
          if (M.source_model == GB_SOURCE_BOUSSINESQ)
            f = ENERGY ? M.density * M.source[a] * (-M.beta * (T - M.Tref)) : 0.0;
          const double adv = v[0] * gv[0][a] + v[1] * gv[1][a] + v[2] * gv[2][a];
          S.cR[q * LDS + a] = dA * (f - rho * adv);
#pragma unroll
          for (int p = 0; p < 3; p++)
            S.tR[p][q * LDS + a] = -dA * ((p == a ? -P : 0.0) + mu * (gv[a][p] + gv[p][a]));
        }
        S.w[W_DA][q] = dA;
        if (ENERGY) {
          S.cR[q * LDS + 3] = -rho * M.heat_capacity * dA * (v[0] * gT[0] + v[1] * gT[1] + v[2] * gT[2]);
#pragma unroll
          for (int p = 0; p < 3; p++) S.tR[p][q * LDS + 3] = -M.conductivity * dA * gT[p];
        }
#pragma unroll
        for (int p = 0; p < 3; p++) {
#pragma unroll
          for (int r = 0; r < 3; r++) S.Bq[q][p * 3 + r] = B[p][r];
          S.vq[q][p] = v[p];
        }
        S.dAq[q] = dA;
      }
      // continuity residual rows and the det J status
#pragma unroll
      for (int l = 0; l < NP; l++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) rc[l] += __shfl_xor_sync(0xffffffffu, rc[l], o);
      const unsigned anybad = __ballot_sync(0xffffffffu, bad);
      if (lane == 0) {
        if (anybad) {
          atomicAdd(A.status, 1);
          atomicMin(A.status + 1, e);
        }
        const int nc = S.nodes[CENT];
        const int g0 = A.fu[nc] + A.pofs;
#pragma unroll
        for (int l = 0; l < NP; l++)
          if (!A.dbc[g0 + l]) A.R[g0 + l] += rc[l];
      }
    }
    __syncthreads();
    // ---- operand tables: physical gradients, -mu dA G, CK
    for (int t = tid; t < NQ * NN; t += blockDim.x) {
      const int q = t / NN, k = t - q * NN;
      const double d0 = tab_dphi[t * 3], d1 = tab_dphi[t * 3 + 1], d2 = tab_dphi[t * 3 + 2];
      const double *B = S.Bq[q];
      const double g0 = B[0] * d0 + B[1] * d1 + B[2] * d2;
      const double g1 = B[3] * d0 + B[4] * d1 + B[5] * d2;
      const double g2 = B[6] * d0 + B[7] * d1 + B[8] * d2;
      const double dA = S.dAq[q];
      const double nm = -M.viscosity * dA;
      const int o = q * LD + k;
      S.G[0][o] = g0;
      S.G[1][o] = g1;
      S.G[2][o] = g2;
      if (!JAC) continue;
      S.mG[0][o] = nm * g0;
      S.mG[1][o] = nm * g1;
      S.mG[2][o] = nm * g2;
      S.cK[o] = -M.density * dA * (S.vq[q][0] * g0 + S.vq[q][1] * g1 + S.vq[q][2] * g2);
    }
    __syncthreads();

    const uint16_t *nslot = A.elem_nslot + (int64_t)e * NN * NN;
    double acc[16][2];
    // ---- stage A
    if (!JAC) {
      if (warp == 1) residual_rows<ENERGY>(S, A, lane);
      continue;
    }
    if (warp == 0) {
      zero(acc);
      prod44<false>(acc, S.G[0], nullptr, S.mG[0], lane);
      prod44<false>(acc, S.G[1], nullptr, S.mG[1], lane);
      prod44<false>(acc, S.G[2], nullptr, S.mG[2], lane);
      store_block(acc, S.S2, lane);
    } else if (warp == 1) {
      zero(acc);
      prod44<false>(acc, S.phi, nullptr, S.cK, lane);
      store_block(acc, S.S1, lane);
      if (ENERGY && (M.source_model == GB_SOURCE_BOUSSINESQ)) {
        zero(acc);
        prod44<true>(acc, S.phi, S.w[W_DA], S.phi, lane);
#pragma unroll
        for (int a = 0; a < 3; a++) {
          const double dfT = -M.density * M.source[a] * M.beta;
          if (dfT != 0.0) scatter<ENERGY>(acc, a, DIM, dfT, S, A, nslot, lane);
        }
      }
      residual_rows<ENERGY>(S, A, lane);
    } else if (warp == 2) {
      if (ENERGY) {
#pragma unroll 1
        for (int b = 0; b < 3; b++) {
          zero(acc);
          prod44<true>(acc, S.phi, S.w[W_TV + b], S.phi, lane);
          scatter<ENERGY>(acc, DIM, b, 1.0, S, A, nslot, lane);
        }
      } else {
        vel_block(acc, 0, 1, S, lane);
        scatter<ENERGY>(acc, 0, 1, 1.0, S, A, nslot, lane);
      }
    } else {
      // warps 3..7: off-diagonal velocity blocks
      constexpr int offd_e[5][2] = {{0, 1}, {0, 2}, {1, 0}, {1, 2}, {2, 0}};
      constexpr int offd_n[5][2] = {{0, 2}, {1, 0}, {1, 2}, {2, 0}, {2, 1}};
      const int a = ENERGY ? offd_e[warp - 3][0] : offd_n[warp - 3][0];
      const int b = ENERGY ? offd_e[warp - 3][1] : offd_n[warp - 3][1];
      vel_block(acc, a, b, S, lane);
      scatter<ENERGY>(acc, a, b, 1.0, S, A, nslot, lane);
    }
    __syncthreads();  // S1, S2 visible
    // ---- stage B
    if (warp == 0) {
      if (ENERGY) {
        // J_TT = Cp S1 + (k / mu) S2, with S2 still in this warp's accumulators
        const double kr = M.conductivity / M.viscosity;
        const int r = lane >> 2, c = lane & 3;
#pragma unroll
        for (int it = 0; it < 4; it++) {
          const int i = it * 8 + r;
#pragma unroll
          for (int jt = 0; jt < 4; jt++)
#pragma unroll
            for (int e2 = 0; e2 < 2; e2++) {
              const int j = jt * 8 + 2 * c + e2;
              const double s1 = (i < NN && j < NN) ? S.S1[i][j] : 0.0;
              acc[it * 4 + jt][e2] = fma(M.heat_capacity, s1, kr * acc[it * 4 + jt][e2]);
            }
        }
        scatter<ENERGY>(acc, DIM, DIM, 1.0, S, A, nslot, lane);
      }
    } else if (ENERGY ? (warp >= 3 && warp <= 5) : (warp >= 1 && warp <= 3)) {
      const int a = ENERGY ? warp - 3 : warp - 1;
      vel_block(acc, a, a, S, lane);
      add_diag(acc, S, lane);
      scatter<ENERGY>(acc, a, a, 1.0, S, A, nslot, lane);
    } else if (ENERGY && warp == 6) {
      vel_block(acc, 2, 1, S, lane);
      scatter<ENERGY>(acc, 2, 1, 1.0, S, A, nslot, lane);
    } else if (warp == 7) {
      // J_mP and its transpose J_cv, then the Dirichlet diagonals
      const int r = lane >> 2, c = lane & 3;
      const int nc = S.nodes[CENT];
      const int fc = A.fu[nc] + A.pofs;
      const int *offc = A.nbr_off + A.nbr_ptr[nc];
#pragma unroll 1
      for (int a = 0; a < 3; a++) {
        double accP[4][2];
#pragma unroll
        for (int it = 0; it < 4; it++) accP[it][0] = accP[it][1] = 0.0;
        prod41(accP, S.G[a], S.psidA, lane);
        if (c < 2) {
#pragma unroll
          for (int it = 0; it < 4; it++) {
            const int i = it * 8 + r;
            if (i >= NN) continue;
            const int ni = S.nodes[i];
            const int gr = A.fu[ni] + a;
            if (!A.dbc[gr]) {
              const int64_t base = A.rowptr[gr] + A.nbr_off[A.nbr_ptr[ni] + nslot[i * NN + CENT]] +
                                   A.pofs + 2 * c;
              A.vals[base] += accP[it][0];
              A.vals[base + 1] += accP[it][1];
            }
            const int oc = offc[nslot[CENT * NN + i]] + a;
#pragma unroll
            for (int e2 = 0; e2 < 2; e2++) {
              const int l = 2 * c + e2;
              if (!A.dbc[fc + l]) A.vals[A.rowptr[fc + l] + oc] += accP[it][e2];
            }
          }
        }
      }
      constexpr int NV = DIM + (ENERGY ? 1 : 0);
      for (int t = lane; t < NN * NV + NP; t += 32) {
        int k, var;
        if (t < NN * NV) {
          k = t / NV;
          var = t - k * NV;
        } else {
          k = CENT;
          var = A.pofs + t - NN * NV;
        }
        const int nk = S.nodes[k];
        const int gr = A.fu[nk] + var;
        if (!A.dbc[gr]) continue;
        const int s = nslot[k * NN + k];
        const int off = (ENERGY && var == DIM) ? A.nbr_offT[A.nbr_ptr[nk] + s]
                                               : A.nbr_off[A.nbr_ptr[nk] + s];
        A.vals[A.rowptr[gr] + off + var] += 1.0;
      }
    }
  }
}

size_t assemble_gemm_smem_bytes() { return sizeof(gm::Smem); }

void build_iso_table(const double *tab_phi, const double *tab_dphi, double *iso) {
  using namespace gm;
  for (int t = 0; t < NISO * KP; t++) iso[t] = 0.0;
  for (int d = 0; d < 4; d++)
    for (int q = 0; q < NQ; q++)
      for (int k = 0; k < NN; k++)
        iso[(d * NQ + q) * KP + k] =
            d == 0 ? tab_phi[q * NN + k] : tab_dphi[(q * NN + k) * 3 + d - 1];
}

template <bool ENERGY, bool JAC>
static cudaError_t launch_gemm_t(const AsmArgs &a, const double *tab_iso, const int *elems,
                                 int nelem, int grid_cap, cudaStream_t st) {
  const size_t sm = sizeof(gm::Smem);
  auto k = assemble_gemm_kernel<ENERGY, JAC>;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const int grid = nelem < grid_cap ? nelem : grid_cap;
  if (grid <= 0) return cudaSuccess;
  k<<<grid, 256, sm, st>>>(a, tab_iso, elems, nelem);
  return cudaGetLastError();
}

cudaError_t launch_assemble_gemm(const AsmArgs &a, bool energy, const double *tab_iso,
                                 const int *elems, int nelem, int grid_cap, cudaStream_t st) {
  if (a.vals)
    return energy ? launch_gemm_t<true, true>(a, tab_iso, elems, nelem, grid_cap, st)
                  : launch_gemm_t<false, true>(a, tab_iso, elems, nelem, grid_cap, st);
  return energy ? launch_gemm_t<true, false>(a, tab_iso, elems, nelem, grid_cap, st)
                : launch_gemm_t<false, false>(a, tab_iso, elems, nelem, grid_cap, st);
}

}  // namespace gb
