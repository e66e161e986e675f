// Species rows of the element residual and analytic Jacobian (dilute
// species, Galerkin; steady, or with the time-derivative terms of a
// transient step), in FP64 on sm_103a, with the coloured CSR scatter.
//
// Replaces, for these rows, assemble_mass_transport
// (src/mm_fill_species.c:194) with get_continuous_species_terms (:9739),
// fickian_flux (:12414) and the CONSTANT / USER species sources
// (:10117, :10146; the USER body is the Arrhenius rate of the problem
// description).  The species variable form is SPECIES_UNDEFINED_FORM (the
// reader's default, src/mm_as_alloc.c:140), so coeff_rho = 1:
//   R_w[i] = sum_q dA [ -phi_i (v . grad Y_w) + grad phi_i . (-D_w grad Y_w)
//                       + phi_i S_w ]
//   dR_w[i]/dY_w1[j] = dA [ (w == w1) (-phi_i v . grad phi_j
//                                     - D_w grad phi_i . grad phi_j)
//                           + phi_i phi_j dS_w/dY_w1 ]
//   dR_w[i]/dv_b[j]  = -dA phi_i phi_j dY_w/dx_b
//   dR_w[i]/dT[j]    =  dA phi_i phi_j dS_w/dT
// The momentum, continuity and energy rows do not depend on the species
// (constant density, no heat of reaction), so the flow kernels need not
// know about them; this kernel runs after the flow kernel of the same
// colour and writes only species rows.
//
// Work decomposition mirrors the flow kernel: one CTA per element in 3-D,
// three in 2-D; phase 1 per quadrature point (geometry, fields, source),
// phase 2 per (quadrature point, node) (physical gradients), phase 3 per
// (i, j) node pairs, one species row block at a time to bound registers,
// then the scatter.  Elements of a colour share no node: no atomics.
#include <cuda_runtime.h>

#include <cstdint>

#include "gb_device.h"
#include "gb_element.cuh"

namespace gb {

namespace sp {

constexpr int MS = GB_MAX_SPECIES;

template <int DIM>
struct QPs {
  double dA;
  double B[DIM][DIM];
  double v[DIM];
  double gY[MS][DIM];
  double S[MS], dSdT[MS], dSdY[MS][MS];
  double Yd[MS];  // time derivatives (transient)
};

template <int DIM>
struct QNs {
  double phi;
  double g[DIM];
  double vg;  // v . grad phi
};

template <int DIM>
struct Elem {
  double X[Q2<DIM>::NN][DIM];
  double U[Q2<DIM>::NN][DIM];
  double Tn[Q2<DIM>::NN];
  double Yn[MS][Q2<DIM>::NN];
  double Ydn[MS][Q2<DIM>::NN];  // nodal time derivatives (transient)
  int nodes[Q2<DIM>::NN];
  int e;
  QPs<DIM> qp[Q2<DIM>::NQ];
  QNs<DIM> qn[Q2<DIM>::NQ][Q2<DIM>::NN];
};

}  // namespace sp

template <int DIM, bool ENERGY, bool JAC>
__global__ void __launch_bounds__(256)
    assemble_species_kernel(AsmArgs A, const int *__restrict__ elems, int nelem) {
  using C = Q2<DIM>;
  using sp::MS;
  constexpr int NN = C::NN, NQ = C::NQ, TPE = C::TPE, EPB = C::EPB, PPT = C::PPT;
  constexpr int OY = DIM + (ENERGY ? 1 : 0);  // offset of Y_0 among a node's unknowns
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using Elem = sp::Elem<DIM>;
  Elem *S = reinterpret_cast<Elem *>(smem_raw);
  const int tid = threadIdx.x;
  const int slot = tid / TPE;
  const int lt = tid - slot * TPE;
  const int ebase = blockIdx.x * EPB;
  const bool thread_live = tid < TPE * EPB && ebase + slot < nelem;
  const double *__restrict__ tab_phi = A.tab_phi;
  const double *__restrict__ tab_dphi = A.tab_dphi;
  const MaterialDev &M = A.mat;
  const int ns = M.nspec;

  // ---- load element data
  for (int t = tid; t < EPB * NN; t += blockDim.x) {
    const int s = t / NN, k = t - s * NN;
    if (ebase + s >= nelem) continue;
    const int e = elems[ebase + s];
    const int n = A.conn[(int64_t)e * NN + k];
    Elem &E = S[s];
    E.nodes[k] = n;
    if (k == 0) E.e = e;
    const int f0 = A.fu[n];
#pragma unroll
    for (int j = 0; j < DIM; j++) {
      E.X[k][j] = A.coords[(int64_t)n * DIM + j];
      E.U[k][j] = A.x[f0 + j];
    }
    E.Tn[k] = ENERGY ? A.x[f0 + DIM] : 0.0;
    for (int w = 0; w < ns; w++) E.Yn[w][k] = A.x[f0 + OY + w];
    for (int w = 0; w < ns; w++) E.Ydn[w][k] = A.xdot ? A.xdot[f0 + OY + w] : 0.0;
  }
  __syncthreads();

  // ---- phase 1: one thread per quadrature point
  for (int t = tid; t < EPB * NQ; t += blockDim.x) {
    const int s = t / NQ, q = t - s * NQ;
    if (ebase + s >= nelem) continue;
    Elem &E = S[s];
    sp::QPs<DIM> &Q = E.qp[q];
    double Jm[DIM][DIM], v[DIM], T = 0.0, Y[MS], Yh[MS][DIM];
#pragma unroll
    for (int i = 0; i < DIM; i++) {
      v[i] = 0.0;
#pragma unroll
      for (int j = 0; j < DIM; j++) Jm[i][j] = 0.0;
    }
#pragma unroll
    for (int w = 0; w < MS; w++) {
      Y[w] = 0.0;
#pragma unroll
      for (int i = 0; i < DIM; i++) Yh[w][i] = 0.0;
    }
    for (int k = 0; k < NN; k++) {
      const double ph = tab_phi[q * NN + k];
      double dph[DIM];
#pragma unroll
      for (int i = 0; i < DIM; i++) dph[i] = tab_dphi[(q * NN + k) * DIM + i];
#pragma unroll
      for (int i = 0; i < DIM; i++)
#pragma unroll
        for (int j = 0; j < DIM; j++) Jm[i][j] = fma(dph[i], E.X[k][j], Jm[i][j]);
#pragma unroll
      for (int a = 0; a < DIM; a++) v[a] = fma(ph, E.U[k][a], v[a]);
      if (ENERGY) T = fma(ph, E.Tn[k], T);
#pragma unroll
      for (int w = 0; w < MS; w++) {
        if (w >= ns) break;
        const double yk = E.Yn[w][k];
        Y[w] = fma(ph, yk, Y[w]);
#pragma unroll
        for (int i = 0; i < DIM; i++) Yh[w][i] = fma(dph[i], yk, Yh[w][i]);
      }
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
    Q.dA = A.tab_w[q] * det;
#pragma unroll
    for (int p = 0; p < DIM; p++) {
      Q.v[p] = v[p];
#pragma unroll
      for (int i = 0; i < DIM; i++) Q.B[p][i] = B[p][i];
    }
#pragma unroll
    for (int w = 0; w < MS; w++) {
      if (w >= ns) break;
#pragma unroll
      for (int p = 0; p < DIM; p++) {
        double g = 0.0;
#pragma unroll
        for (int i = 0; i < DIM; i++) g = fma(B[p][i], Yh[w][i], g);
        Q.gY[w][p] = g;
      }
      // source and its sensitivities (CONSTANT: src/mm_fill_species.c:10117;
      // USER Arrhenius S = nu k0 exp(-E/T) Y_s: :10146-10190)
      double Sw = 0.0, dT = 0.0;
      for (int w1 = 0; w1 < MS; w1++) Q.dSdY[w][w1] = 0.0;
      if (M.ssm[w] == GB_SPECIES_SOURCE_CONSTANT) {
        Sw = M.ssp[w][0];
      } else if (M.ssm[w] == GB_SPECIES_SOURCE_ARRHENIUS) {
        const int src = (int)M.ssp[w][3];
        const double r = M.ssp[w][0] * exp(-M.ssp[w][1] / T);
        double ys = 0.0;
        for (int w1 = 0; w1 < MS; w1++)
          if (w1 == src) ys = Y[w1];
        Sw = M.ssp[w][2] * r * ys;
        dT = Sw * M.ssp[w][1] / (T * T);
        Q.dSdY[w][src] = M.ssp[w][2] * r;
      }
      Q.S[w] = Sw;
      Q.dSdT[w] = dT;
      double yd = 0.0;
      if (A.xdot)
        for (int k = 0; k < NN; k++) yd = fma(tab_phi[q * NN + k], E.Ydn[w][k], yd);
      Q.Yd[w] = yd;
    }
  }
  __syncthreads();

  // ---- phase 2: one thread per (quadrature point, node)
  for (int t = tid; t < EPB * NQ * NN; t += blockDim.x) {
    const int s = t / (NQ * NN), r = t - s * (NQ * NN), q = r / NN, k = r - q * NN;
    if (ebase + s >= nelem) continue;
    Elem &E = S[s];
    const sp::QPs<DIM> &Q = E.qp[q];
    sp::QNs<DIM> &W = E.qn[q][k];
    double dph[DIM], vg = 0.0;
#pragma unroll
    for (int i = 0; i < DIM; i++) dph[i] = tab_dphi[(q * NN + k) * DIM + i];
#pragma unroll
    for (int p = 0; p < DIM; p++) {
      double g = 0.0;
#pragma unroll
      for (int i = 0; i < DIM; i++) g = fma(Q.B[p][i], dph[i], g);
      W.g[p] = g;
      vg = fma(Q.v[p], g, vg);
    }
    W.phi = tab_phi[q * NN + k];
    W.vg = vg;
  }
  __syncthreads();
  if (!thread_live) return;

  Elem &E = S[slot];
  const int e = E.e;
  const int *nodes = E.nodes;
  const uint16_t *nslot = A.elem_nslot + (int64_t)e * NN * NN;

  // ---- residual rows (w, i): one thread each; Dirichlet rows get their
  // diagonal 1 instead (put_dirichlet_in_matrix, src/bc_dirich.c:44)
  if (lt < ns * NN) {
    const int w = lt / NN, i = lt - (lt / NN) * NN;
    const double nD = -M.diff[w];
    double Racc = 0.0;
    for (int q = 0; q < NQ; q++) {
      const sp::QPs<DIM> &Q = E.qp[q];
      const sp::QNs<DIM> &Wi = E.qn[q][i];
      double vgY = 0.0, dif = 0.0;
#pragma unroll
      for (int p = 0; p < DIM; p++) {
        vgY = fma(Q.v[p], Q.gY[w][p], vgY);
        dif = fma(Wi.g[p], nD * Q.gY[w][p], dif);
      }
      // with the mass term -Y_dot_w phi_i dA (coeff_rho = 1,
      // src/mm_fill_species.c:525-551)
      Racc += (-(vgY + Q.Yd[w]) * Wi.phi + dif + Q.S[w] * Wi.phi) * Q.dA;
    }
    const int node = nodes[i];
    const int gr = A.fu[node] + OY + w;
    if (A.dbc[gr]) {
      if (JAC) {
        const int s = nslot[i * NN + i];
        A.vals[A.rowptr[gr] + A.nbr_off[A.nbr_ptr[node] + s] + OY + w] += 1.0;
      }
    } else {
      A.R[gr] += Racc;
    }
  }
  if (!JAC) return;

  // ---- Jacobian node pairs, one species row block at a time
  const int pi = lt / (NN / PPT);
  const int pj0 = lt - pi * (NN / PPT);
  const int ni = nodes[pi];
  const int nb0 = A.nbr_ptr[ni];
  for (int w = 0; w < ns; w++) {
    const int gr = A.fu[ni] + OY + w;
    if (A.dbc[gr]) continue;  // uniform per thread: the row belongs to node pi
    const double nD = -M.diff[w];
    double JYY[PPT][MS], JYv[PPT][DIM], JYT[PPT];
#pragma unroll
    for (int m = 0; m < PPT; m++) {
      JYT[m] = 0.0;
#pragma unroll
      for (int b = 0; b < DIM; b++) JYv[m][b] = 0.0;
#pragma unroll
      for (int w1 = 0; w1 < MS; w1++) JYY[m][w1] = 0.0;
    }
    for (int q = 0; q < NQ; q++) {
      const sp::QPs<DIM> &Q = E.qp[q];
      const sp::QNs<DIM> &Wi = E.qn[q][pi];
      const double dA = Q.dA;
      double ngY[DIM], dSdY[MS];
#pragma unroll
      for (int b = 0; b < DIM; b++) ngY[b] = -Q.gY[w][b];
#pragma unroll
      for (int w1 = 0; w1 < MS; w1++) dSdY[w1] = Q.dSdY[w][w1];
      const double dSdT = Q.dSdT[w];
#pragma unroll
      for (int m = 0; m < PPT; m++) {
        const sp::QNs<DIM> &Wj = E.qn[q][pj0 + m * (NN / PPT)];
        double dot = 0.0;
#pragma unroll
        for (int p = 0; p < DIM; p++) dot = fma(Wi.g[p], Wj.g[p], dot);
        const double pij = Wi.phi * Wj.phi * dA;
        // with the mass term's sensitivity -(1 + 2 theta) / dt phi_i phi_j dA
        const double diag = fma(-Wi.phi, Wj.vg, nD * dot) * dA - A.mass_c * pij;
#pragma unroll
        for (int w1 = 0; w1 < MS; w1++)
          JYY[m][w1] = fma(dSdY[w1], pij, JYY[m][w1] + (w1 == w ? diag : 0.0));
#pragma unroll
        for (int b = 0; b < DIM; b++) JYv[m][b] = fma(ngY[b], pij, JYv[m][b]);
        JYT[m] = fma(dSdT, pij, JYT[m]);
      }
    }
    const int64_t rb = A.rowptr[gr];
#pragma unroll
    for (int m = 0; m < PPT; m++) {
      const int pj = pj0 + m * (NN / PPT);
      const int64_t base = rb + A.nbr_off[nb0 + nslot[pi * NN + pj]];
#pragma unroll
      for (int b = 0; b < DIM; b++) A.vals[base + b] += JYv[m][b];
      if (ENERGY) A.vals[base + DIM] += JYT[m];
#pragma unroll
      for (int w1 = 0; w1 < MS; w1++)
        if (w1 < ns) A.vals[base + OY + w1] += JYY[m][w1];
    }
  }
}

template <int DIM, bool ENERGY, bool JAC>
static cudaError_t launch_species_t(const AsmArgs &a, const int *elems, int nelem,
                                    cudaStream_t st) {
  using C = Q2<DIM>;
  const size_t sm = sizeof(sp::Elem<DIM>) * C::EPB;
  auto k = assemble_species_kernel<DIM, ENERGY, JAC>;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  const int grid = (nelem + C::EPB - 1) / C::EPB;
  if (grid == 0) return cudaSuccess;
  k<<<grid, 256, sm, st>>>(a, elems, nelem);
  return cudaGetLastError();
}

cudaError_t launch_assemble_species(const AsmArgs &a, int dim, bool energy, bool jac,
                                    const int *elems, int nelem, cudaStream_t st) {
#define GB_DISPATCH(D, EN, JA) \
  if (dim == D && energy == EN && jac == JA) return launch_species_t<D, EN, JA>(a, elems, nelem, st);
  GB_DISPATCH(2, false, true)
  GB_DISPATCH(2, true, true)
  GB_DISPATCH(3, false, true)
  GB_DISPATCH(3, true, true)
  GB_DISPATCH(2, false, false)
  GB_DISPATCH(2, true, false)
  GB_DISPATCH(3, false, false)
  GB_DISPATCH(3, true, false)
#undef GB_DISPATCH
  return cudaErrorInvalidValue;
}

}  // namespace gb
