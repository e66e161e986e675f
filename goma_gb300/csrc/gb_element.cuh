// Element-level definitions shared by the scalar-FP64 and the DMMA element
// kernels: Q2/P1 sizes, the per-quadrature-point record and its set-up.
#pragma once
#include <cuda_runtime.h>

#include "gb_device.h"

namespace gb {

template <int DIM>
struct Q2 {
  static constexpr int NN = DIM == 2 ? 9 : 27;
  static constexpr int NQ = NN;
  static constexpr int NP = DIM + 1;
  static constexpr int CENT = DIM == 2 ? 8 : 20;
  static constexpr int TPE = DIM == 2 ? 81 : 243;  // threads per element
  static constexpr int EPB = DIM == 2 ? 3 : 1;     // elements per CTA
  static constexpr int PPT = NN * NN / TPE;        // (i,j) pairs per thread
};

// per-quadrature-point record in shared memory
template <int DIM>
struct QP {
  double dA;
  double B[DIM][DIM];
  double v[DIM];
  double gv[DIM][DIM];  // gv[p][a] = d v_a / d x_p
  double gam[DIM][DIM];
  double T, gT[DIM];
  double P;
  double mu;
  double cmu;  // (d mu / d gammadot) / gammadot, 0 when not Carreau or gd = 0
  double f[DIM];
  double dfT[DIM];
  double psi[DIM + 1];
  double hs, dhs;  // heat source and its T sensitivity
  int bad;
};

// Quadrature-point set-up (one thread per point), for an element of density
// rho: isoparametric map
// (beer_belly, src/mm_fill_util.c:140), J^-1 and det J, field values and
// gradients (load_fv / load_fv_grads, src/load_field_variables.c:128,
// :2049), viscosity (src/mm_viscosity.c:108, Carreau :981, shear rate
// src/mm_fill_util.c:4564) and body force (src/mm_std_models.c:125).
template <int DIM, bool ENERGY, bool CARREAU>
__device__ __forceinline__ void qp_setup(const double (*X)[DIM], const double (*U)[DIM],
                                         const double *Tn, const double *Pn, int q,
                                         const double *__restrict__ tab_phi,
                                         const double *__restrict__ tab_dphi,
                                         const double *__restrict__ tab_w,
                                         const double *__restrict__ tab_pt, const MaterialDev &M,
                                         double rho, QP<DIM> &Q) {
  constexpr int NN = Q2<DIM>::NN, NP = Q2<DIM>::NP;
    double Jm[DIM][DIM], Gh[DIM][DIM], Th[DIM];
#pragma unroll
    for (int i = 0; i < DIM; i++) {
      Th[i] = 0.0;
#pragma unroll
      for (int j = 0; j < DIM; j++) Jm[i][j] = Gh[i][j] = 0.0;
    }
    double v[DIM], T = 0.0;
#pragma unroll
    for (int a = 0; a < DIM; a++) v[a] = 0.0;
    for (int k = 0; k < NN; k++) {
      const double ph = tab_phi[q * NN + k];
      double dph[DIM];
#pragma unroll
      for (int i = 0; i < DIM; i++) dph[i] = tab_dphi[(q * NN + k) * DIM + i];
#pragma unroll
      for (int i = 0; i < DIM; i++) {
#pragma unroll
        for (int j = 0; j < DIM; j++) {
          Jm[i][j] = fma(dph[i], X[k][j], Jm[i][j]);
          Gh[i][j] = fma(dph[i], U[k][j], Gh[i][j]);
        }
        if (ENERGY) Th[i] = fma(dph[i], Tn[k], Th[i]);
      }
#pragma unroll
      for (int a = 0; a < DIM; a++) v[a] = fma(ph, U[k][a], v[a]);
      if (ENERGY) T = fma(ph, Tn[k], T);
    }
    double det, B[DIM][DIM];
    if (DIM == 2) {
      det = Jm[0][0] * Jm[1][1] - Jm[0][1] * Jm[1][0];
      B[0][0] = Jm[1][1] / det;
      B[1][1] = Jm[0][0] / det;
      B[0][1] = -Jm[0][1] / det;
      B[1][0] = -Jm[1][0] / det;
    } else {
      const double c00 = Jm[1][1] * Jm[2][2] - Jm[1][2] * Jm[2][1];
      const double c01 = Jm[1][0] * Jm[2][2] - Jm[1][2] * Jm[2][0];
      const double c02 = Jm[1][0] * Jm[2][1] - Jm[1][1] * Jm[2][0];
      det = Jm[0][0] * c00 - Jm[0][1] * c01 + Jm[0][2] * c02;
      B[0][0] = c00 / det;
      B[0][1] = -(Jm[0][1] * Jm[2][2] - Jm[2][1] * Jm[0][2]) / det;
      B[0][2] = (Jm[0][1] * Jm[1][2] - Jm[1][1] * Jm[0][2]) / det;
      B[1][0] = -c01 / det;
      B[1][1] = (Jm[0][0] * Jm[2][2] - Jm[2][0] * Jm[0][2]) / det;
      B[1][2] = -(Jm[0][0] * Jm[1][2] - Jm[1][0] * Jm[0][2]) / det;
      B[2][0] = c02 / det;
      B[2][1] = -(Jm[0][0] * Jm[2][1] - Jm[2][0] * Jm[0][1]) / det;
      B[2][2] = (Jm[0][0] * Jm[1][1] - Jm[1][0] * Jm[0][1]) / det;
    }
    Q.bad = !(det > 0.0);
    Q.dA = tab_w[q] * det;
#pragma unroll
    for (int p = 0; p < DIM; p++)
#pragma unroll
      for (int i = 0; i < DIM; i++) Q.B[p][i] = B[p][i];
    // gv[p][a] = sum_i B[p][i] Gh[i][a]; gT[p] = sum_i B[p][i] Th[i]
    double gv[DIM][DIM], gT[DIM];
#pragma unroll
    for (int p = 0; p < DIM; p++) {
      gT[p] = 0.0;
#pragma unroll
      for (int a = 0; a < DIM; a++) {
        double s2 = 0.0;
#pragma unroll
        for (int i = 0; i < DIM; i++) s2 = fma(B[p][i], Gh[i][a], s2);
        gv[p][a] = s2;
      }
      if (ENERGY)
#pragma unroll
        for (int i = 0; i < DIM; i++) gT[p] = fma(B[p][i], Th[i], gT[p]);
    }
    double gam[DIM][DIM];
#pragma unroll
    for (int a = 0; a < DIM; a++)
#pragma unroll
      for (int b = 0; b < DIM; b++) gam[a][b] = gv[a][b] + gv[b][a];
    double mu = M.viscosity, cmu = 0.0;
    if (CARREAU) {
      double s2 = 0.0;
#pragma unroll
      for (int a = 0; a < DIM; a++)
#pragma unroll
        for (int b = 0; b < DIM; b++) s2 = fma(gam[a][b], gam[b][a], s2);
      const double gd = sqrt(0.5 * fabs(s2));
      const bool nz = gd > 1.0e-298;
      const double lg = M.lambda * gd;
      const double val2 = nz ? pow(lg, M.aexp) : 0.0;
      mu = M.mu_inf + (M.mu0 - M.mu_inf) * pow(1.0 + val2, (M.nexp - 1.0) / M.aexp);
      const double val = nz ? pow(lg, M.aexp - 1.0) : 0.0;
      const double val1 = pow(1.0 + val2, (M.nexp - 1.0 - M.aexp) / M.aexp);
      const double dmu = (M.mu0 - M.mu_inf) * (M.nexp - 1.0) * M.lambda * val * val1;
      cmu = nz ? dmu / gd : 0.0;
    }
    double P = 0.0, psi[NP];
    psi[0] = 1.0;
    const int is = q % 3, it = (q % 9) / 3, iu = q / 9;
    psi[1] = tab_pt[is];
    psi[2] = tab_pt[it];
    if (DIM == 3) psi[3] = tab_pt[iu];
#pragma unroll
    for (int l = 0; l < NP; l++) P = fma(Pn[l], psi[l], P);
#pragma unroll
    for (int l = 0; l < NP; l++) Q.psi[l] = psi[l];
#pragma unroll
    for (int a = 0; a < DIM; a++) {
      Q.v[a] = v[a];
      if (ENERGY) Q.gT[a] = gT[a];
#pragma unroll
      for (int b = 0; b < DIM; b++) {
        Q.gv[a][b] = gv[a][b];
        Q.gam[a][b] = gam[a][b];
      }
      double f = 0.0, dfT = 0.0;
      if (M.source_model == GB_SOURCE_BOUSSINESQ) {
        if (ENERGY) {
          f = rho * M.source[a] * (-M.beta * (T - M.Tref));
          dfT = -rho * M.source[a] * M.beta;
        }
      } else {
        f = M.source[a];
      }
      Q.f[a] = f;
      Q.dfT[a] = dfT;
    }
    // heat source (heat_source, src/mm_fill_energy.c:1724; the exponential
    // one is a USER model, src/user_mp.c:472)
    double hs = 0.0, dhs = 0.0;
    if (ENERGY) {
      if (M.hsm == GB_HEAT_SOURCE_CONSTANT) {
        hs = M.hs[0];
      } else if (M.hsm == GB_HEAT_SOURCE_EXPONENTIAL) {
        hs = M.hs[0] * exp(M.hs[1] * T);
        dhs = M.hs[1] * hs;
      }
    }
    Q.hs = hs;
    Q.dhs = dhs;
    Q.T = T;
    Q.P = P;
    Q.mu = mu;
    Q.cmu = cmu;
}

}  // namespace gb
