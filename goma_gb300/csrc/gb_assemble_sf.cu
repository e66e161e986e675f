// 3-D Q2/P1 element residual + analytic Jacobian (Newtonian Navier-Stokes,
// optional energy with a Boussinesq body force) with the fewest FP64
// operations: sum factorisation over the tensor-product HEX27 basis for
// every term whose test and trial functions are reference-element tensor
// products, and one symmetric product for the rest.
//
// Same physics and results (to rounding) as the scalar kernel of
// gb_assemble.cu: the reference's assemble_momentum
// (src/mm_fill_momentum.c:100, fluid_stress :2834), assemble_continuity
// (src/mm_fill_continuity.c:119), assemble_energy (src/mm_fill_energy.c:109),
// bouss_momentum_source (src/mm_std_models.c:125), the hard-set Dirichlet rows
// of put_dirichlet_in_matrix (src/bc_dirich.c:44) and the load_lec scatter
// (src/mm_fill.c:5175).
//
// Why: on GB300 FP64 runs at ~2 FMA per SM-cycle, on the scalar units and on
// the FP64 tensor path (mma.sync m8n8k4) alike, so the element kernel is
// bound by its count of FP64 operations, not by memory.  Per element:
//
//   field values and reference gradients at the 27 points: sum
//     factorisation, 3 passes over the 1-D factors (~5K FMA instead of 20K);
//   weighted mass matrices  M_w(i,j) = sum_q phi_i phi_j w(q)  for 13
//     weights (-rho dA dv_a/dx_b, -rho Cp dA dT/dx_b, dA) and the advection
//     term S1(i,j) = sum_q phi_i (-rho dA v . grad phi_j) written as three
//     such sums over reference derivatives: phi_i phi_j = prod_d
//     l_{i_d}(q_d) l_{j_d}(q_d), so each is three contractions of 243 + 729
//     + 2187 FMA instead of 19,683;
//   H((p,i),(r,j)) = sum_q dphi_i/dx_p dA dphi_j/dx_r, symmetric 81 x 81,
//     upper triangle only (3,321 entries x 27 FMA): gives the transpose
//     stress term -mu H((b,i),(a,j)) of J_ab, and through its trace the
//     viscous term of J_aa and the conduction term of J_TT.
//
//   J_ab   = M(-rho dA dv_a/dx_b) - mu H((b,i),(a,j)) + delta_ab (S1 - mu tr H)
//   J_TT   = Cp S1 - k tr H
//   J_Tb   = M(-rho Cp dA dT/dx_b),   J_aT = (df_a/dT) M(dA)
//   J_mP   = sum_q dphi_i/dx_a psi_l dA,   J_cv = J_mP^T
//
// That is ~195K FP64 operations per element against ~865K for the dense
// forms.  The scatter adds into the CSR values with red.global.add.f64: the
// add runs in L2 instead of on the SM's FP64 pipe, and since the elements of
// one colour share no CSR row every entry receives one add per launch, so
// the result is deterministic.  One CTA of 256 threads per element, two
// CTAs per SM, persistent over the colour's element list.
#include <cuda_runtime.h>

#include <cstdint>

#include "gb_device.h"

namespace gb {

namespace sf {

constexpr int NN = 27, NQ = 27, NP = 4, CENT = 20, NF = 7;
constexpr int NC = 16;  // sum-factorised contractions
enum { C_AB = 0, C_TV = 9, C_DA = 12, C_S1 = 13 };
constexpr int NH = 81 * 82 / 2;  // upper triangle of H

__device__ __forceinline__ int hrow(int P) { return P * 81 - (P * (P - 1)) / 2; }

struct Smem {
  double ell[2][3][3];   // [0] l_a(xi_g), [1] l'_a(xi_g)
  double pp[2][9][3];    // [0] l_a l_b, [1] l_a l'_b at xi_g, index a*3+b
  double phi[NQ][NN];    // phi_L(q), L lexicographic
  double W[NC][NQ];      // weights of the sum-factorised contractions
  double cR[4][NQ];      // residual: phi part (momentum a, energy 3)
  double tR[3][4][NQ];   // residual: gradient part [p][n][q]
  double psidA[NP][NQ];
  double Bq[NQ][9];      // J^-1 [p][r]
  double dAq[NQ];
  double G[3][NQ][NN];   // d phi_L / d x_p at q
  double cG[3][NQ][NN];  // dA * G
  double T2[NC][3][81];  // second stage of the sum factorisation
  union {
    double H[NH];
    double T1[NC][9][9];
    struct {
      double Xn[NF][NN];   // x y z u v w T at the nodes (lexicographic)
      double A[NF][2][NN];
      double B[NF][3][NN];
      double F[NF][4][NQ]; // value, d/dxi_1..3 at the points
      double Xd[4][NN];    // u v w T time derivatives at the nodes (transient)
    } iso;
  } X;
  double Pn[NP];
  int lex[NN];    // lexicographic index of local node k
  int loc[NN];    // local node of lexicographic index L
  int nodes[NN];  // global node of local node k
};

}  // namespace sf

template <bool ENERGY, bool JAC>
__global__ void __launch_bounds__(256, 2)
    assemble_sf_kernel(AsmArgs A, const SfTables *__restrict__ tb,
                       const int *__restrict__ elems, int nelem) {
  using namespace sf;
  constexpr int DIM = 3;
  constexpr int NV = DIM + (ENERGY ? 1 : 0);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem &S = *reinterpret_cast<Smem *>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nt = blockDim.x;
  const MaterialDev M = A.mat;

  // constant tables
  for (int t = tid; t < 18; t += nt) (&S.ell[0][0][0])[t] = (&tb->ell[0][0][0])[t];
  for (int t = tid; t < 54; t += nt) (&S.pp[0][0][0])[t] = (&tb->pp[0][0][0])[t];
  for (int t = tid; t < NQ * NN; t += nt) (&S.phi[0][0])[t] = (&tb->phi[0][0])[t];
  for (int t = tid; t < NN; t += nt) {
    S.lex[t] = tb->lex[t];
    S.loc[t] = tb->loc[t];
  }

  for (int ei = blockIdx.x; ei < nelem; ei += gridDim.x) {
    const int e = elems[ei];
    const double rho_e = A.elem_rho ? A.elem_rho[e] : M.density;
    __syncthreads();  // the previous element is done with shared memory
    // ---- nodal data (lexicographic order)
    if (tid < NN) {
      const int k = tid, L = S.lex[k];
      const int n = A.conn[(int64_t)e * NN + k];
      S.nodes[k] = n;
      const int f0 = A.fu[n];
#pragma unroll
      for (int j = 0; j < DIM; j++) {
        S.X.iso.Xn[j][L] = A.coords[(int64_t)n * DIM + j];
        S.X.iso.Xn[3 + j][L] = A.x[f0 + j];
      }
      S.X.iso.Xn[6][L] = ENERGY ? A.x[f0 + DIM] : 0.0;
      if (k == CENT)
        for (int l = 0; l < NP; l++) S.Pn[l] = A.x[f0 + A.pofs + l];
      if (A.xdot) {
#pragma unroll
        for (int j = 0; j < DIM; j++) S.X.iso.Xd[j][L] = A.xdot[f0 + j];
        S.X.iso.Xd[3][L] = ENERGY ? A.xdot[f0 + DIM] : 0.0;
      }
    }
    __syncthreads();
    // ---- values and reference gradients at the points: three passes
    for (int t = tid; t < NF * 2 * 27; t += nt) {  // contract a1 -> q1 (l, l')
      const int f = t / 54, v = (t / 27) % 2, r = t % 27;
      const int a3 = r / 9, a2 = (r / 3) % 3, q1 = r % 3;
      const double *x = &S.X.iso.Xn[f][3 * a2 + 9 * a3];
      const double(*E)[3] = S.ell[v];
      S.X.iso.A[f][v][r] = E[0][q1] * x[0] + E[1][q1] * x[1] + E[2][q1] * x[2];
      (void)q1;
    }
    __syncthreads();
    for (int t = tid; t < NF * 3 * 27; t += nt) {  // contract a2 -> q2
      const int f = t / 81, w = (t / 27) % 3, r = t % 27;
      const int a3 = r / 9, q2 = (r / 3) % 3, q1 = r % 3;
      const int src = w == 2 ? 1 : 0;
      const double(*E)[3] = S.ell[w == 1 ? 1 : 0];
      const double *a = &S.X.iso.A[f][src][a3 * 9 + q1];
      S.X.iso.B[f][w][r] = E[0][q2] * a[0] + E[1][q2] * a[3] + E[2][q2] * a[6];
    }
    __syncthreads();
    for (int t = tid; t < NF * 4 * 27; t += nt) {  // contract a3 -> q3
      const int f = t / 108, d = (t / 27) % 4, q = t % 27;
      const int q3 = q / 9, q2 = (q / 3) % 3, q1 = q % 3;
      // d = 0 value, 1 d/dxi_1, 2 d/dxi_2, 3 d/dxi_3
      const int src = d == 1 ? 2 : (d == 2 ? 1 : 0);
      const double(*E)[3] = S.ell[d == 3 ? 1 : 0];
      const double *b = &S.X.iso.B[f][src][q2 * 3 + q1];
      S.X.iso.F[f][d][q] = E[0][q3] * b[0] + E[1][q3] * b[9] + E[2][q3] * b[18];
    }
    __syncthreads();
    // ---- per quadrature point (warp 0)
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
            Jm[r][j] = S.X.iso.F[j][1 + r][q];
            Gh[r][j] = S.X.iso.F[3 + j][1 + r][q];
          }
          Th[r] = S.X.iso.F[6][1 + r][q];
          v[r] = S.X.iso.F[3 + r][0][q];
        }
        const double T = S.X.iso.F[6][0][q];
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
        double gv[3][3], gT[3];  // gv[p][a] = d v_a / d x_p
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
        const double mu = M.viscosity, rho = rho_e;
        const double divv = gv[0][0] + gv[1][1] + gv[2][2];
        // time derivatives at the point (transient; load_fv's fv_dot)
        double vd[4] = {0.0, 0.0, 0.0, 0.0};
        if (A.xdot)
          for (int L = 0; L < NN; L++) {
            const double ph = S.phi[q][L];
#pragma unroll
            for (int c = 0; c < 4; c++) vd[c] = fma(ph, S.X.iso.Xd[c][L], vd[c]);
          }
#pragma unroll
        for (int l = 0; l < NP; l++) {
          S.psidA[l][q] = psi[l] * dA;
          rc[l] = psi[l] * dA * divv;
        }
#pragma unroll
        for (int a = 0; a < 3; a++) {
#pragma unroll
          for (int b = 0; b < 3; b++) S.W[C_AB + a * 3 + b][q] = -rho * dA * gv[b][a];
          S.W[C_TV + a][q] = ENERGY ? -rho * M.heat_capacity * dA * gT[a] : 0.0;
          S.W[C_S1 + a][q] = -rho * dA * (v[0] * B[0][a] + v[1] * B[1][a] + v[2] * B[2][a]);
          double f = M.source[a];
          if (M.source_model == GB_SOURCE_BOUSSINESQ)
            f = ENERGY ? rho * M.source[a] * (-M.beta * (T - M.Tref)) : 0.0;
          const double adv = v[0] * gv[0][a] + v[1] * gv[1][a] + v[2] * gv[2][a];
          // with the mass term -rho v_dot_a (src/mm_fill_momentum.c:471-500)
          S.cR[a][q] = dA * (f - rho * (adv + vd[a]));
#pragma unroll
          for (int p = 0; p < 3; p++)
            S.tR[p][a][q] = -dA * ((p == a ? -P : 0.0) + mu * (gv[a][p] + gv[p][a]));
        }
        S.W[C_DA][q] = dA;
        S.cR[3][q] = ENERGY ? -rho * M.heat_capacity * dA *
                                  (v[0] * gT[0] + v[1] * gT[1] + v[2] * gT[2] + vd[3])
                            : 0.0;
#pragma unroll
        for (int p = 0; p < 3; p++) S.tR[p][3][q] = ENERGY ? -M.conductivity * dA * gT[p] : 0.0;
#pragma unroll
        for (int p = 0; p < 3; p++)
#pragma unroll
          for (int r = 0; r < 3; r++) S.Bq[q][p * 3 + r] = B[p][r];
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
        const int g0 = A.fu[S.nodes[CENT]] + A.pofs;
#pragma unroll
        for (int l = 0; l < NP; l++)
          if (!A.dbc[g0 + l]) atomicAdd(A.R + g0 + l, rc[l]);
      }
    }
    __syncthreads();
    // ---- physical gradients; first stage of the sum factorisation
    for (int t = tid; t < NQ * NN; t += nt) {
      const int q = t / NN, L = t - q * NN;
      const double *d = &tb->dref[q][L][0];
      const double d0 = __ldg(d), d1 = __ldg(d + 1), d2 = __ldg(d + 2);
      const double *B = S.Bq[q];
      const double g0 = B[0] * d0 + B[1] * d1 + B[2] * d2;
      const double g1 = B[3] * d0 + B[4] * d1 + B[5] * d2;
      const double g2 = B[6] * d0 + B[7] * d1 + B[8] * d2;
      S.G[0][q][L] = g0;
      S.G[1][q][L] = g1;
      S.G[2][q][L] = g2;
      if (JAC) {
        const double dA = S.dAq[q];
        S.cG[0][q][L] = dA * g0;
        S.cG[1][q][L] = dA * g1;
        S.cG[2][q][L] = dA * g2;
      }
    }
    if (JAC) {
      for (int t = tid; t < NC * 81; t += nt) {
        const int c = t / 81, r = t % 81, q12 = r / 9, ab3 = r % 9;
        const double *pp = S.pp[c == C_S1 + 2 ? 1 : 0][ab3];
        const double *w = &S.W[c][q12];
        S.X.T1[c][q12][ab3] = pp[0] * w[0] + pp[1] * w[9] + pp[2] * w[18];
      }
    }
    __syncthreads();
    // ---- second stage; residual rows, J_mP / J_cv, Dirichlet diagonals
    if (JAC) {
      for (int t = tid; t < NC * 243; t += nt) {
        const int c = t / 243, r = t % 243, q1 = r / 81, ab23 = r % 81;
        const int ab2 = ab23 / 9, ab3 = ab23 % 9;
        const double *pp = S.pp[c == C_S1 + 1 ? 1 : 0][ab2];
        S.T2[c][q1][ab23] = pp[0] * S.X.T1[c][q1][ab3] + pp[1] * S.X.T1[c][q1 + 3][ab3] +
                            pp[2] * S.X.T1[c][q1 + 6][ab3];
      }
    }
    {
      const int nres = 4 * NN, njmp = JAC ? 3 * NN * NP : 0, ndir = JAC ? NN * NV + NP : 0;
      const int nc = S.nodes[CENT];
      for (int t = tid; t < nres + njmp + ndir; t += nt) {
        if (t < nres) {
          const int n = t / NN, L = t % NN;
          if (n == 3 && !ENERGY) continue;
          double s = 0.0;
#pragma unroll 3
          for (int q = 0; q < NQ; q++) {
            s = fma(S.phi[q][L], S.cR[n][q], s);
            s = fma(S.G[0][q][L], S.tR[0][n][q], s);
            s = fma(S.G[1][q][L], S.tR[1][n][q], s);
            s = fma(S.G[2][q][L], S.tR[2][n][q], s);
          }
          const int gr = A.fu[S.nodes[S.loc[L]]] + n;
          if (!A.dbc[gr]) atomicAdd(A.R + gr, s);
        } else if (t < nres + njmp) {
          const int u = t - nres, a = u / (NN * NP), L = (u / NP) % NN, l = u % NP;
          double s = 0.0;
#pragma unroll 3
          for (int q = 0; q < NQ; q++) s = fma(S.G[a][q][L], S.psidA[l][q], s);
          const int k = S.loc[L], nk = S.nodes[k];
          const uint16_t *ns = A.elem_nslot + (int64_t)e * NN * NN;
          const int gr = A.fu[nk] + a;
          if (!A.dbc[gr])
            atomicAdd(A.vals + A.rowptr[gr] + A.nbr_off[A.nbr_ptr[nk] + ns[k * NN + CENT]] +
                          A.pofs + l, s);
          const int gc = A.fu[nc] + A.pofs + l;
          if (!A.dbc[gc])
            atomicAdd(A.vals + A.rowptr[gc] + A.nbr_off[A.nbr_ptr[nc] + ns[CENT * NN + k]] + a, s);
        } else {
          const int u = t - nres - njmp;
          int k, var;
          if (u < NN * NV) {
            k = u / NV;
            var = u - k * NV;
          } else {
            k = CENT;
            var = A.pofs + u - NN * NV;
          }
          const int nk = S.nodes[k];
          const int gr = A.fu[nk] + var;
          if (!A.dbc[gr]) continue;
          const int s = A.elem_nslot[(int64_t)e * NN * NN + k * NN + k];
          const int off = (ENERGY && var == DIM) ? A.nbr_offT[A.nbr_ptr[nk] + s]
                                                 : A.nbr_off[A.nbr_ptr[nk] + s];
          atomicAdd(A.vals + A.rowptr[gr] + off + var, 1.0);
        }
      }
    }
    if (!JAC) continue;
    __syncthreads();
    // ---- H, upper triangle
    for (int t = tid; t < NH; t += nt) {
      const int pr = tb->hmap[t];
      const int P = pr >> 7, R = pr & 127;
      const int p = P / NN, i = P - p * NN, r = R / NN, j = R - r * NN;
      const double *gi = &S.G[p][0][i], *gj = &S.cG[r][0][j];
      double s0 = 0.0, s1 = 0.0, s2 = 0.0;
#pragma unroll
      for (int q = 0; q < NQ; q += 3) {
        s0 = fma(gi[q * NN], gj[q * NN], s0);
        s1 = fma(gi[(q + 1) * NN], gj[(q + 1) * NN], s1);
        s2 = fma(gi[(q + 2) * NN], gj[(q + 2) * NN], s2);
      }
      S.X.H[t] = (s0 + s1) + s2;
    }
    __syncthreads();
    // ---- node pairs: combine and scatter
    {
      const double mu = M.viscosity, Cp = M.heat_capacity, kc = M.conductivity;
      double dfT[3];
#pragma unroll
      for (int a = 0; a < 3; a++)
        dfT[a] = (ENERGY && M.source_model == GB_SOURCE_BOUSSINESQ)
                     ? -rho_e * M.source[a] * M.beta
                     : 0.0;
      const uint16_t *ns = A.elem_nslot + (int64_t)e * NN * NN;
      for (int t = tid; t < NN * NN; t += nt) {
        const int ki = t / NN, kj = t - ki * NN;
        const int Li = S.lex[ki], Lj = S.lex[kj];
        const int a1 = Li % 3, a2 = (Li / 3) % 3, a3 = Li / 9;
        const int b1 = Lj % 3, b2 = (Lj / 3) % 3, b3 = Lj / 9;
        const int ab1 = a1 * 3 + b1, ab23 = (a2 * 3 + b2) * 9 + a3 * 3 + b3;
        auto stage3 = [&](int c) {
          const double *pp = S.pp[c == C_S1 ? 1 : 0][ab1];
          return pp[0] * S.T2[c][0][ab23] + pp[1] * S.T2[c][1][ab23] + pp[2] * S.T2[c][2][ab23];
        };
        auto h = [&](int P, int R) {
          return P <= R ? S.X.H[hrow(P) + R - P] : S.X.H[hrow(R) + P - R];
        };
        const double S1 = stage3(C_S1) + stage3(C_S1 + 1) + stage3(C_S1 + 2);
        const double trH = h(Li, Lj) + h(NN + Li, NN + Lj) + h(2 * NN + Li, 2 * NN + Lj);
        const int ni = S.nodes[ki];
        const int fi = A.fu[ni];
        const int nb = A.nbr_ptr[ni] + ns[ki * NN + kj];
        const bool tr = A.mass_c != 0.0;
        const double mdA = (ENERGY || tr) ? stage3(C_DA) : 0.0;
        // the mass terms' sensitivity -(1 + 2 theta) / dt rho M(dA)
        // (src/mm_fill_momentum.c:1586-1590), times Cp on the energy row
        const double Mt = tr ? -A.mass_c * rho_e * mdA : 0.0;
        const double D = fma(-mu, trH, S1) + Mt;
#pragma unroll
        for (int a = 0; a < 3; a++) {
          const int gr = fi + a;
          if (A.dbc[gr]) continue;
          double *row = A.vals + A.rowptr[gr] + A.nbr_off[nb];
#pragma unroll
          for (int b = 0; b < 3; b++) {
            double v = fma(-mu, h(b * NN + Li, a * NN + Lj), stage3(C_AB + a * 3 + b));
            if (a == b) v += D;
            atomicAdd(row + b, v);
          }
          if (ENERGY) atomicAdd(row + DIM, dfT[a] * mdA);
        }
        if (ENERGY) {
          const int gr = fi + DIM;
          if (!A.dbc[gr]) {
            double *row = A.vals + A.rowptr[gr] + A.nbr_offT[nb];
#pragma unroll
            for (int b = 0; b < 3; b++) atomicAdd(row + b, stage3(C_TV + b));
            atomicAdd(row + DIM, fma(Cp, S1 + Mt, -kc * trH));
          }
        }
      }
    }
  }
}

void build_sf_tables(const double *tab_phi, const double *tab_dphi, const int (*loc27)[3],
                     const double *ell, const double *dell, SfTables &T) {
  using namespace sf;
  for (int a = 0; a < 3; a++)
    for (int g = 0; g < 3; g++) {
      T.ell[0][a][g] = ell[a * 3 + g];
      T.ell[1][a][g] = dell[a * 3 + g];
    }
  for (int a = 0; a < 3; a++)
    for (int b = 0; b < 3; b++)
      for (int g = 0; g < 3; g++) {
        T.pp[0][a * 3 + b][g] = ell[a * 3 + g] * ell[b * 3 + g];
        T.pp[1][a * 3 + b][g] = ell[a * 3 + g] * dell[b * 3 + g];
      }
  for (int k = 0; k < NN; k++) {
    const int L = loc27[k][0] + 3 * loc27[k][1] + 9 * loc27[k][2];
    T.lex[k] = L;
    T.loc[L] = k;
  }
  for (int q = 0; q < NQ; q++)
    for (int L = 0; L < NN; L++) {
      const int k = T.loc[L];
      T.phi[q][L] = tab_phi[q * NN + k];
      for (int r = 0; r < 3; r++) T.dref[q][L][r] = tab_dphi[(q * NN + k) * 3 + r];
    }
  int e = 0;
  for (int P = 0; P < 81; P++)
    for (int R = P; R < 81; R++) T.hmap[e++] = (uint16_t)((P << 7) | R);
}

size_t assemble_sf_smem_bytes() { return sizeof(sf::Smem); }

template <bool ENERGY, bool JAC>
static cudaError_t launch_sf_t(const AsmArgs &a, const SfTables *tb, const int *elems,
                               int nelem, int grid_cap, cudaStream_t st) {
  const size_t sm = sizeof(sf::Smem);
  auto k = assemble_sf_kernel<ENERGY, JAC>;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const int grid = nelem < grid_cap ? nelem : grid_cap;
  if (grid <= 0) return cudaSuccess;
  k<<<grid, 256, sm, st>>>(a, tb, elems, nelem);
  return cudaGetLastError();
}

cudaError_t launch_assemble_sf(const AsmArgs &a, bool energy, const SfTables *tb,
                               const int *elems, int nelem, int grid_cap, cudaStream_t st) {
  if (a.vals)
    return energy ? launch_sf_t<true, true>(a, tb, elems, nelem, grid_cap, st)
                  : launch_sf_t<false, true>(a, tb, elems, nelem, grid_cap, st);
  return energy ? launch_sf_t<true, false>(a, tb, elems, nelem, grid_cap, st)
                : launch_sf_t<false, false>(a, tb, elems, nelem, grid_cap, st);
}

}  // namespace gb
