// Element residual + analytic Jacobian assembly for Q2/P1 Navier-Stokes
// (+ energy, Boussinesq, Carreau-Yasuda) with the coloured CSR scatter, in
// FP64 on sm_103a.
//
// Replaces matrix_fill_full / matrix_fill (src/mm_fill.c:158, :317) for
// these physics: assemble_momentum (src/mm_fill_momentum.c:100),
// fluid_stress (:2834), assemble_continuity (src/mm_fill_continuity.c:119),
// assemble_energy (src/mm_fill_energy.c:109), the hard-set Dirichlet rows of
// put_dirichlet_in_matrix (src/bc_dirich.c:44) and the load_lec scatter
// (src/mm_fill.c:5175) -- the scatter's per-entry linear search becomes a
// slot computed from the node graph.
//
// Work decomposition (one CTA per element in 3-D, three per CTA in 2-D):
//   phase 1  one thread per quadrature point: isoparametric map, J^-1,
//            det J, field values and gradients, viscosity, body force;
//   phase 2  one thread per (quadrature point, node): physical basis
//            gradients and the per-node coefficients of the Jacobian terms;
//   phase 3  one thread per 1 (2-D) or 3 (3-D) (i, j) node pairs: all
//            velocity/temperature blocks of J(i, j) accumulated in
//            registers over the quadrature points, read from shared memory;
//            the first dim*nn+nn+dim+1 threads also own one residual row and
//            the J_m_P / J_c_v pressure couplings;
//   phase 4  coloured read-modify-write into the CSR values and R: elements
//            of one colour share no node, hence no CSR row, so the scatter
//            needs no atomics and is deterministic.
// The dominant cost is the FP64 pipe (phase 3); global traffic is the
// matrix read-modify-write.
#include <cuda_runtime.h>

#include <cstdint>

#include "gb_device.h"
#include "gb_element.cuh"

namespace gb {

// per-(quadrature point, node) record
template <int DIM, bool CARREAU>
struct QN {
  double phi;
  double g[DIM];   // physical gradient
  double cK;       // -rho dA (v . grad phi)
  double cT;       // -rho Cp dA (v . grad phi)
  double gm[CARREAU ? DIM : 1];  // grad phi . gamma_a
};

// shared-memory record of one element: nodal data, per-quadrature-point
// records, per-(quadrature point, node) records
template <int DIM, bool CARREAU>
struct ElemSmem {
  double X[Q2<DIM>::NN][DIM];
  double U[Q2<DIM>::NN][DIM];
  double Tn[Q2<DIM>::NN];
  double Pn[Q2<DIM>::NP];
  double Ud[Q2<DIM>::NN][DIM];  // nodal time derivatives (transient)
  double Tdn[Q2<DIM>::NN];
  double vd[Q2<DIM>::NQ][DIM];  // the same at the quadrature points
  double Td[Q2<DIM>::NQ];
  int nodes[Q2<DIM>::NN];
  int e;
  double rho;  // density of this element
  QP<DIM> qp[Q2<DIM>::NQ];
  QN<DIM, CARREAU> qn[Q2<DIM>::NQ][Q2<DIM>::NN];
};

template <int DIM, bool ENERGY, bool CARREAU, bool JAC>
__global__ void __launch_bounds__(256)
    assemble_kernel(AsmArgs A, const int *__restrict__ elems, int nelem) {
  using C = Q2<DIM>;
  constexpr int NN = C::NN, NQ = C::NQ, NP = C::NP, TPE = C::TPE, EPB = C::EPB, PPT = C::PPT;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using Elem = ElemSmem<DIM, CARREAU>;
  Elem *S = reinterpret_cast<Elem *>(smem_raw);
  const int tid = threadIdx.x;
  const int slot = tid / TPE;
  const int lt = tid - slot * TPE;
  const int ebase = blockIdx.x * EPB;
  const bool thread_live = tid < TPE * EPB && ebase + slot < nelem;
  const double *__restrict__ tab_phi = A.tab_phi;    // [NQ][NN]
  const double *__restrict__ tab_dphi = A.tab_dphi;  // [NQ][NN][DIM]
  const MaterialDev M = A.mat;

  // ---- load element data
  for (int t = tid; t < EPB * NN; t += blockDim.x) {
    const int s = t / NN, k = t - s * NN;
    if (ebase + s >= nelem) continue;
    const int e = elems[ebase + s];
    const int n = A.conn[(int64_t)e * NN + k];
    Elem &E = S[s];
    E.nodes[k] = n;
    if (k == 0) {
      E.e = e;
      E.rho = A.elem_rho ? A.elem_rho[e] : M.density;
    }
    const int f0 = A.fu[n];
#pragma unroll
    for (int j = 0; j < DIM; j++) {
      E.X[k][j] = A.coords[(int64_t)n * DIM + j];
      E.U[k][j] = A.x[f0 + j];
    }
    if (ENERGY) E.Tn[k] = A.x[f0 + DIM];
    if (k == C::CENT)
      for (int l = 0; l < NP; l++) E.Pn[l] = A.x[f0 + A.pofs + l];
    if (A.xdot) {
#pragma unroll
      for (int j = 0; j < DIM; j++) E.Ud[k][j] = A.xdot[f0 + j];
      E.Tdn[k] = ENERGY ? A.xdot[f0 + DIM] : 0.0;
    }
  }
  __syncthreads();

  // ---- phase 1: one thread per quadrature point
  for (int t = tid; t < EPB * NQ; t += blockDim.x) {
    const int s = t / NQ, q = t - s * NQ;
    if (ebase + s >= nelem) continue;
    Elem &E = S[s];
    qp_setup<DIM, ENERGY, CARREAU>(E.X, E.U, E.Tn, E.Pn, q, tab_phi, tab_dphi, A.tab_w, A.tab_pt,
                                   M, E.rho, E.qp[q]);
    if (A.xdot) {  // v_dot and T_dot at the point (load_fv's fv_dot)
      double vd[DIM], Td = 0.0;
#pragma unroll
      for (int a = 0; a < DIM; a++) vd[a] = 0.0;
      for (int k = 0; k < NN; k++) {
        const double ph = tab_phi[q * NN + k];
#pragma unroll
        for (int a = 0; a < DIM; a++) vd[a] = fma(ph, E.Ud[k][a], vd[a]);
        if (ENERGY) Td = fma(ph, E.Tdn[k], Td);
      }
#pragma unroll
      for (int a = 0; a < DIM; a++) E.vd[q][a] = vd[a];
      E.Td[q] = Td;
    }
  }
  __syncthreads();

  // ---- phase 2: one thread per (quadrature point, node)
  for (int t = tid; t < EPB * NQ * NN; t += blockDim.x) {
    const int s = t / (NQ * NN), r = t - s * (NQ * NN), q = r / NN, k = r - q * NN;
    if (ebase + s >= nelem) continue;
    Elem &E = S[s];
    const QP<DIM> &Q = E.qp[q];
    QN<DIM, CARREAU> &W = E.qn[q][k];
    double g[DIM], dph[DIM];
#pragma unroll
    for (int i = 0; i < DIM; i++) dph[i] = tab_dphi[(q * NN + k) * DIM + i];
    double vg = 0.0;
#pragma unroll
    for (int p = 0; p < DIM; p++) {
      double s2 = 0.0;
#pragma unroll
      for (int i = 0; i < DIM; i++) s2 = fma(Q.B[p][i], dph[i], s2);
      g[p] = s2;
      W.g[p] = s2;
      vg = fma(Q.v[p], s2, vg);
    }
    W.phi = tab_phi[q * NN + k];
    W.cK = -E.rho * Q.dA * vg;
    if (ENERGY) W.cT = -E.rho * M.heat_capacity * Q.dA * vg;
    if (CARREAU) {
#pragma unroll
      for (int a = 0; a < DIM; a++) {
        double s2 = 0.0;
#pragma unroll
        for (int p = 0; p < DIM; p++) s2 = fma(g[p], Q.gam[a][p], s2);
        W.gm[a] = s2;
      }
    }
  }
  __syncthreads();
  if (!thread_live) return;

  Elem &E = S[slot];
  const int e = E.e;

  // ---- phase 3: accumulate
  // residual / pressure-coupling ownership
  constexpr int NRM = DIM * NN;  // momentum rows
  const bool own_m = lt < NRM;
  const bool own_T = ENERGY && lt >= NRM && lt < NRM + NN;
  const bool own_c = lt >= NRM + (ENERGY ? NN : 0) && lt < NRM + (ENERGY ? NN : 0) + NP;
  const int ra = lt / NN, ri = lt - (lt / NN) * NN;  // momentum row (a, i)
  const int rT = lt - NRM;                           // energy row i
  const int rc = lt - NRM - (ENERGY ? NN : 0);       // continuity row l
  double Racc = 0.0;
  double JmP[NP];
#pragma unroll
  for (int l = 0; l < NP; l++) JmP[l] = 0.0;

  // pairs
  const int pi = lt / (NN / PPT);
  const int pj0 = lt - pi * (NN / PPT);
  double Jv[PPT][DIM][DIM], JTT[PPT], JTv[PPT][DIM], JvT[PPT][DIM];
#pragma unroll
  for (int m = 0; m < PPT; m++) {
    JTT[m] = 0.0;
#pragma unroll
    for (int a = 0; a < DIM; a++) {
      JTv[m][a] = JvT[m][a] = 0.0;
#pragma unroll
      for (int b = 0; b < DIM; b++) Jv[m][a][b] = 0.0;
    }
  }
  bool bad = false;
  for (int q = 0; q < NQ; q++) {
    const QP<DIM> &Q = E.qp[q];
    const double dA = Q.dA;
    bad |= Q.bad;
    // residual rows
    if (own_m) {
      const QN<DIM, CARREAU> &Wi = E.qn[q][ri];
      double adv = 0.0;
#pragma unroll
      for (int p = 0; p < DIM; p++) adv = fma(Q.v[p], Q.gv[p][ra], adv);
      adv = adv * E.rho * (-Wi.phi * dA);
      double dif = 0.0;
#pragma unroll
      for (int p = 0; p < DIM; p++)
        dif = fma(Wi.g[p], (p == ra ? -Q.P : 0.0) + Q.mu * Q.gam[ra][p], dif);
      dif *= -dA;
      const double src = Q.f[ra] * (Wi.phi * dA);
      // mass term -rho v_dot_a phi_i dA (src/mm_fill_momentum.c:471-500)
      const double mass = A.xdot ? -E.rho * E.vd[q][ra] * (Wi.phi * dA) : 0.0;
      Racc += mass + adv + dif + src;
      if (JAC) {
#pragma unroll
        for (int l = 0; l < NP; l++) JmP[l] = fma(Wi.g[ra] * Q.psi[l], dA, JmP[l]);
      }
    } else if (own_T) {
      const QN<DIM, CARREAU> &Wi = E.qn[q][rT];
      double vgT = 0.0, dif = 0.0;
#pragma unroll
      for (int p = 0; p < DIM; p++) {
        vgT = fma(Q.v[p], Q.gT[p], vgT);
        dif = fma(Wi.g[p], -M.conductivity * Q.gT[p], dif);
      }
      // with the mass term -rho Cp T_dot phi_i dA (src/mm_fill_energy.c:315-381)
      // and the heat source phi_i h dA (:374-378)
      const double Tt = A.xdot ? vgT + E.Td[q] : vgT;
      Racc += Tt * (-Wi.phi * E.rho * M.heat_capacity * dA) + dif * dA + Q.hs * (Wi.phi * dA);
    } else if (own_c) {
      double divv = 0.0;
#pragma unroll
      for (int a = 0; a < DIM; a++) divv += Q.gv[a][a];
      Racc += divv * (Q.psi[rc] * dA);
    }
    if (!JAC) continue;
    // Jacobian node pairs
    const QN<DIM, CARREAU> &Wi = E.qn[q][pi];
    const double nmu = -Q.mu * dA;
    double ti[DIM];
#pragma unroll
    for (int b = 0; b < DIM; b++) ti[b] = nmu * Wi.g[b];
    const double nkdA = -M.conductivity * dA;
    // the mass terms' sensitivity -(1 + 2 theta) / dt rho phi_i phi_j dA
    // (src/mm_fill_momentum.c:1586-1590), times Cp on the energy rows
    const double nmc = -A.mass_c * E.rho;
#pragma unroll
    for (int m = 0; m < PPT; m++) {
      const int pj = pj0 + m * (NN / PPT);
      const QN<DIM, CARREAU> &Wj = E.qn[q][pj];
      double dot = 0.0;
#pragma unroll
      for (int p = 0; p < DIM; p++) dot = fma(Wi.g[p], Wj.g[p], dot);
      const double pij = Wi.phi * Wj.phi * dA;
      const double prho = -E.rho * pij;
      const double K = fma(nmc, pij, fma(Wi.phi, Wj.cK, nmu * dot));
#pragma unroll
      for (int a = 0; a < DIM; a++)
#pragma unroll
        for (int b = 0; b < DIM; b++) {
          double val = fma(prho, Q.gv[b][a], ti[b] * Wj.g[a]);
          if (a == b) val += K;
          if (CARREAU) val = fma(Wi.gm[a], -dA * Q.cmu * Wj.gm[b], val);
          Jv[m][a][b] += val;
        }
      if (ENERGY) {
        JTT[m] += fma(nmc * M.heat_capacity + Q.dhs, pij, fma(Wi.phi, Wj.cT, nkdA * dot));
        const double pc = -E.rho * M.heat_capacity * pij;
#pragma unroll
        for (int b = 0; b < DIM; b++) {
          JTv[m][b] = fma(pc, Q.gT[b], JTv[m][b]);
          JvT[m][b] = fma(pij, Q.dfT[b], JvT[m][b]);
        }
      }
    }
  }
  if (bad && lt == 0) {
    atomicAdd(A.status, 1);
    atomicMin(A.status + 1, e);
  }

  // ---- phase 4: coloured scatter (no other element of this colour
  // touches these rows)
  const int *nodes = E.nodes;
  const uint16_t *nslot = A.elem_nslot + (int64_t)e * NN * NN;
  // residual + Dirichlet diagonal + pressure couplings
  if (own_m || own_T || own_c) {
    int gr, node, k, rowvar;
    if (own_m) {
      k = ri;
      node = nodes[ri];
      gr = A.fu[node] + ra;
      rowvar = ra;
    } else if (own_T) {
      k = rT;
      node = nodes[rT];
      gr = A.fu[node] + DIM;
      rowvar = DIM;
    } else {
      k = C::CENT;
      node = nodes[C::CENT];
      gr = A.fu[node] + A.pofs + rc;
      rowvar = A.pofs + rc;
    }
    const bool dir = A.dbc[gr] != 0;
    if (!dir) A.R[gr] += Racc;
    if (JAC) {
      const int64_t rb = A.rowptr[gr];
      const int nb0 = A.nbr_ptr[node];
      const bool rowT = ENERGY && rowvar == DIM;
      if (dir) {
        const int s = nslot[k * NN + k];
        const int off = rowT ? A.nbr_offT[nb0 + s] : A.nbr_off[nb0 + s];
        A.vals[rb + off + rowvar] += 1.0;
      } else if (own_m) {
        // J_m_P: row (a, i), columns P_l at the centroid node
        const int s = nslot[k * NN + C::CENT];
        const int64_t base = rb + A.nbr_off[nb0 + s] + A.pofs;
#pragma unroll
        for (int l = 0; l < NP; l++) A.vals[base + l] += JmP[l];
      }
    }
  }
  if (JAC && own_m) {
    // J_c_v = transpose of J_m_P: rows P_l at the centroid, column (a, i)
    const int nc = nodes[C::CENT];
    const int s = nslot[C::CENT * NN + ri];
    const int nb0 = A.nbr_ptr[nc];
    const int off = A.nbr_off[nb0 + s] + ra;
#pragma unroll
    for (int l = 0; l < NP; l++) {
      const int gr = A.fu[nc] + A.pofs + l;
      if (A.dbc[gr]) continue;
      A.vals[A.rowptr[gr] + off] += JmP[l];
    }
  }
  if (!JAC) return;
  {
    const int ni = nodes[pi];
    const int fi = A.fu[ni];
    const int nb0 = A.nbr_ptr[ni];
#pragma unroll
    for (int m = 0; m < PPT; m++) {
      const int pj = pj0 + m * (NN / PPT);
      const int s = nslot[pi * NN + pj];
      const int off = A.nbr_off[nb0 + s];
#pragma unroll
      for (int a = 0; a < DIM; a++) {
        const int gr = fi + a;
        if (A.dbc[gr]) continue;
        const int64_t base = A.rowptr[gr] + off;
#pragma unroll
        for (int b = 0; b < DIM; b++) A.vals[base + b] += Jv[m][a][b];
        if (ENERGY) A.vals[base + DIM] += JvT[m][a];
      }
      if (ENERGY) {
        const int gr = fi + DIM;
        if (!A.dbc[gr]) {
          const int64_t base = A.rowptr[gr] + A.nbr_offT[nb0 + s];
#pragma unroll
          for (int b = 0; b < DIM; b++) A.vals[base + b] += JTv[m][b];
          A.vals[base + DIM] += JTT[m];
        }
      }
    }
  }
}

template <int DIM, bool ENERGY, bool CARREAU, bool JAC>
static size_t smem_bytes() {
  using C = Q2<DIM>;
  return sizeof(ElemSmem<DIM, CARREAU>) * C::EPB;
}

template <int DIM, bool ENERGY, bool CARREAU, bool JAC>
static cudaError_t launch_t(const AsmArgs &a, const int *elems, int nelem, cudaStream_t st) {
  using C = Q2<DIM>;
  const size_t sm = smem_bytes<DIM, ENERGY, CARREAU, JAC>();
  auto k = assemble_kernel<DIM, ENERGY, CARREAU, JAC>;
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

size_t assemble_smem_bytes(int dim, bool energy, bool carreau) {
  if (dim == 2) {
    if (energy)
      return carreau ? smem_bytes<2, true, true, true>() : smem_bytes<2, true, false, true>();
    return carreau ? smem_bytes<2, false, true, true>() : smem_bytes<2, false, false, true>();
  }
  if (energy)
    return carreau ? smem_bytes<3, true, true, true>() : smem_bytes<3, true, false, true>();
  return carreau ? smem_bytes<3, false, true, true>() : smem_bytes<3, false, false, true>();
}

cudaError_t launch_assemble(const AsmArgs &a, int dim, bool energy, bool carreau, bool jac,
                            const int *elems, int nelem, cudaStream_t st) {
#define GB_DISPATCH(D, EN, CA, JA)                                    \
  if (dim == D && energy == EN && carreau == CA && jac == JA)         \
    return launch_t<D, EN, CA, JA>(a, elems, nelem, st);
  GB_DISPATCH(2, false, false, true)
  GB_DISPATCH(2, false, true, true)
  GB_DISPATCH(2, true, false, true)
  GB_DISPATCH(2, true, true, true)
  GB_DISPATCH(3, false, false, true)
  GB_DISPATCH(3, false, true, true)
  GB_DISPATCH(3, true, false, true)
  GB_DISPATCH(3, true, true, true)
  GB_DISPATCH(2, false, false, false)
  GB_DISPATCH(2, false, true, false)
  GB_DISPATCH(2, true, false, false)
  GB_DISPATCH(2, true, true, false)
  GB_DISPATCH(3, false, false, false)
  GB_DISPATCH(3, false, true, false)
  GB_DISPATCH(3, true, false, false)
  GB_DISPATCH(3, true, true, false)
#undef GB_DISPATCH
  return cudaErrorInvalidValue;
}

}  // namespace gb
