// Device-side argument blocks shared by the kernels and the host driver.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/gb_problem.h"

namespace gb {

struct MaterialDev {
  double density, viscosity, mu0, mu_inf, lambda, aexp, nexp;
  double heat_capacity, conductivity;
  int source_model;
  double source[3];
  double beta, Tref;
  // species w < nspec: Fickian diffusivity and source (GB_SPECIES_SOURCE_*;
  // CONSTANT ssp[w][0], ARRHENIUS k0, E, nu, s)
  int nspec;
  double diff[GB_MAX_SPECIES];
  int ssm[GB_MAX_SPECIES];
  double ssp[GB_MAX_SPECIES][4];
  // energy heat source (GB_HEAT_SOURCE_*): CONSTANT hs[0], EXPONENTIAL
  // hs[0] exp(hs[1] T)
  int hsm;
  double hs[2];
};

// Everything the assembly kernel reads or writes.  Device pointers.
struct AsmArgs {
  const double *coords;  // num_nodes * dim
  const int *conn;       // num_elems * nn
  const int *fu;         // num_nodes + 1
  const uint8_t *dbc;    // N
  const int64_t *rowptr; // N + 1
  const int *nbr_ptr;
  const int *nbr_off;
  const int *nbr_offT;
  const uint16_t *elem_nslot;  // num_elems * nn * nn
  const double *tab_phi;       // nq * nn
  const double *tab_dphi;      // nq * nn * dim
  const double *tab_w;         // nq
  const double *tab_pt;        // 3 Gauss abscissae (+pt, 0, -pt)
  const double *x;             // N
  double *R;                   // N
  double *vals;                // nnz (CSR, diagonal in row); NULL: residual only
  int *status;                 // [0] non-positive det J count, [1] first such element
  const double *elem_rho;      // per-element density (overrides mat.density); NULL: none
  int pofs;                    // offset of the first P1 pressure at a centroid node
                               // (= nodal fields per node: dim + energy + species)
  // transient terms: the time derivative (N; NULL: steady) and the mass
  // coefficient (1 + 2 theta) / delta_t of its sensitivity
  const double *xdot;
  double mass_c;
  MaterialDev mat;
};

// Integrated boundary conditions, one entry per element side (the cards of
// gb_problem_desc expanded): element, Exodus side number, GB_IBC_* type and
// the card's two values.  Device pointers.
struct SideArgs {
  int num_sides;
  const int *elem;
  const int *side;
  const int *type;
  const double *val;  // 2 per side
};

cudaError_t launch_assemble(const AsmArgs &a, int dim, bool energy, bool carreau, bool jac,
                            const int *elems, int nelem, cudaStream_t st);
// the side terms (gb_assemble_bc.cu); launched after the element kernels
cudaError_t launch_assemble_sides(const AsmArgs &a, const SideArgs &s, int dim, bool energy,
                                  cudaStream_t st);
size_t assemble_smem_bytes(int dim, bool energy, bool carreau);
// species rows (gb_assemble_species.cu); launched after the flow kernel of
// the same colour
cudaError_t launch_assemble_species(const AsmArgs &a, int dim, bool energy, bool jac,
                                    const int *elems, int nelem, cudaStream_t st);
// 3-D Jacobian contractions on the FP64 tensor pipe (gb_assemble_tc.cu)
cudaError_t launch_assemble_tc(const AsmArgs &a, bool energy, bool carreau, const int *elems,
                               int nelem, int grid_cap, cudaStream_t st);
// Constant tables of the sum-factorised 3-D kernel (gb_assemble_sf.cu), one
// device copy per context: 1-D Lagrange factors at the Gauss points and their
// pair products, phi and reference gradients in lexicographic node order, the
// local <-> lexicographic node maps, and the (row, column) list of the upper
// triangle of the 81 x 81 gradient product.
struct SfTables {
  double ell[2][3][3];
  double pp[2][9][3];
  double phi[27][27];
  double dref[27][27][3];
  int lex[27];
  int loc[27];
  uint16_t hmap[81 * 82 / 2];
};
void build_sf_tables(const double *tab_phi, const double *tab_dphi, const int (*loc27)[3],
                     const double *ell, const double *dell, SfTables &T);
cudaError_t launch_assemble_sf(const AsmArgs &a, bool energy, const SfTables *tb,
                               const int *elems, int nelem, int grid_cap, cudaStream_t st);
size_t assemble_sf_smem_bytes();
// 3-D Newtonian residual + Jacobian as dense DMMA products (gb_assemble_gemm.cu);
// tab_iso is build_iso_table's [112][28] table on the device
cudaError_t launch_assemble_gemm(const AsmArgs &a, bool energy, const double *tab_iso,
                                 const int *elems, int nelem, int grid_cap, cudaStream_t st);
size_t assemble_gemm_smem_bytes();
void build_iso_table(const double *tab_phi, const double *tab_dphi, double *iso);

}  // namespace gb
