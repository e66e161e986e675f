/* CPU oracle for the Q2/P1 Newton hot path -- TEST INFRASTRUCTURE ONLY.
 * See gb_oracle.h for scope.  Every routine names the reference code it
 * restates; the restatement is pinned by tests/test_oracle_golden.py
 * against vectors the reference produced (tests/golden/make_golden.py). */
#include "gb_oracle.h"

#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

struct orc_problem {
  gb_problem_desc d; /* copy; the arrays below are owned copies */
  double *coords;
  int *conn;
  int nn;       /* nodes per element: 9 or 27 */
  int centroid; /* local index of the centroid node: 8 or 20 */
  int nvn;      /* nodal fields per node: dim + energy + species */
  int ns;       /* species */
  int npres;    /* P1 pressure unknowns per element: dim + 1 */
  int nloc;     /* nvn * nn + npres */
  int N;
  int *fu;    /* first unknown per node, num_nodes + 1 */
  int *ija;   /* MSR pattern */
  long msr_len;
  int *dbc;   /* per unknown: -1, or index of the Dirichlet card (datum: -2) */
  double *dbc_val;
  /* transient: the time derivative xdot (NULL when steady) and the mass
   * coefficient (1 + 2 theta) / delta_t of its sensitivity */
  const double *xdot;
  double mass_c;
  /* integrated boundary conditions (owned copies) and, per element, its
   * (card, side) pairs: eibc_ptr[e] .. eibc_ptr[e+1]-1 */
  int *ibc_type, *ibc_ptr, *ibc_elem, *ibc_side;
  double *ibc_value;
  int *eibc_ptr, *eibc_card, *eibc_side;
};

/* ---------------------------------------------------------------- basis */

/* Gauss-Legendre constants as the reference writes them
 * (src/el_elm_info.c:1642 and :3484-3485). */
static const double GQ_PT = 0.77459666924148340428;
static const double GQ_W0 = 0.55555555555555555556;
static const double GQ_W1 = 0.88888888888888888888;

static const int LOC9[9][2] = {{0, 0}, {2, 0}, {2, 2}, {0, 2}, {1, 0},
                               {2, 1}, {1, 2}, {0, 1}, {1, 1}};
static const int LOC27[27][3] = {
    {0, 0, 0}, {2, 0, 0}, {2, 2, 0}, {0, 2, 0}, {0, 0, 2}, {2, 0, 2}, {2, 2, 2},
    {0, 2, 2}, {1, 0, 0}, {2, 1, 0}, {1, 2, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 1},
    {2, 2, 1}, {0, 2, 1}, {1, 0, 2}, {2, 1, 2}, {1, 2, 2}, {0, 1, 2}, {1, 1, 1},
    {1, 1, 0}, {1, 1, 2}, {0, 1, 1}, {2, 1, 1}, {1, 0, 1}, {1, 2, 1}};

/* 1-D quadratic Lagrange polynomials on the nodes -1, 0, +1 */
static double lag(int g, double s) {
  return g == 0 ? 0.5 * s * (s - 1.0) : (g == 1 ? 1.0 - s * s : 0.5 * s * (s + 1.0));
}
static double dlag(int g, double s) { return g == 0 ? s - 0.5 : (g == 1 ? -2.0 * s : s + 0.5); }

/* Quadrature point iq in the reference order (src/el_elm_info.c:1748 for
 * QUAD9, :1802 for HEX27): s runs fastest from +sqrt(3/5) down, then t,
 * then u; weight = w_s * w_t * w_u (src/el_elm_info.c:3554, :3646). */
static void quad_point(int dim, int iq, double xi[3], double *w) {
  static const double pt[3] = {0.77459666924148340428, 0.0, -0.77459666924148340428};
  static const double wt[3] = {0.55555555555555555556, 0.88888888888888888888,
                               0.55555555555555555556};
  int is = iq % 3, it = (iq % 9) / 3, iu = iq / 9;
  (void)GQ_PT;
  (void)GQ_W0;
  (void)GQ_W1;
  xi[0] = pt[is];
  xi[1] = pt[it];
  xi[2] = dim == 3 ? pt[iu] : 0.0;
  *w = dim == 3 ? wt[is] * wt[it] * wt[iu] : wt[is] * wt[it];
}

/* phi and d(phi)/d(xi) of the Q2 basis at xi */
static void q2_basis(int dim, const double xi[3], double *phi, double (*dphi)[3]) {
  if (dim == 2) {
    for (int k = 0; k < 9; k++) {
      int gx = LOC9[k][0], gy = LOC9[k][1];
      double ls = lag(gx, xi[0]), lt = lag(gy, xi[1]);
      phi[k] = ls * lt;
      dphi[k][0] = dlag(gx, xi[0]) * lt;
      dphi[k][1] = ls * dlag(gy, xi[1]);
      dphi[k][2] = 0.0;
    }
  } else {
    for (int k = 0; k < 27; k++) {
      int gx = LOC27[k][0], gy = LOC27[k][1], gz = LOC27[k][2];
      double ls = lag(gx, xi[0]), lt = lag(gy, xi[1]), lu = lag(gz, xi[2]);
      phi[k] = ls * lt * lu;
      dphi[k][0] = dlag(gx, xi[0]) * lt * lu;
      dphi[k][1] = ls * dlag(gy, xi[1]) * lu;
      dphi[k][2] = ls * lt * dlag(gz, xi[2]);
    }
  }
}

/* ---------------------------------------------------------------- setup */

static int cmp_int(const void *a, const void *b) {
  int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}

/* DOF numbering (src/mm_unknown_map.c:758, Index_Solution :5268): node by
 * node in node order; at every node the velocity components, then T, then
 * the species Y_0.., and at an element's centroid node its dim+1 P1
 * pressure unknowns (variable types in ascending order,
 * include/rf_fem_const.h:174-200).
 * Sparsity (src/exo_conn.c:204 build_node_node, src/mm_fill_util.c:3229
 * find_MSR_problem_graph): unknown i couples with every unknown of every
 * node sharing an element with its node; a centroid node also couples with
 * the centroid nodes of the face neighbours of its element
 * (src/exo_conn.c:300-330).  Off-diagonal columns ascend. */
orc_problem *orc_create(const gb_problem_desc *desc) {
  orc_problem *p = (orc_problem *)calloc(1, sizeof(*p));
  if (!p) return NULL;
  p->d = *desc;
  const int dim = desc->dim, nnod = desc->num_nodes, ne = desc->num_elems;
  p->nn = dim == 2 ? 9 : 27;
  p->centroid = dim == 2 ? 8 : 20;
  p->ns = desc->num_species > 0 ? desc->num_species : 0;
  p->nvn = dim + (desc->energy ? 1 : 0) + p->ns;
  p->npres = dim + 1;
  p->nloc = p->nvn * p->nn + p->npres;
  p->coords = (double *)malloc(sizeof(double) * (size_t)nnod * dim);
  p->conn = (int *)malloc(sizeof(int) * (size_t)ne * p->nn);
  memcpy(p->coords, desc->coords, sizeof(double) * (size_t)nnod * dim);
  memcpy(p->conn, desc->conn, sizeof(int) * (size_t)ne * p->nn);
  p->d.coords = p->coords;
  p->d.conn = p->conn;

  /* centroid flag and unknowns per node */
  int *is_cent = (int *)calloc((size_t)nnod, sizeof(int));
  int *cent_elem = (int *)malloc(sizeof(int) * (size_t)nnod);
  for (int i = 0; i < nnod; i++) cent_elem[i] = -1;
  for (int e = 0; e < ne; e++) {
    int c = p->conn[e * p->nn + p->centroid];
    is_cent[c] = 1;
    cent_elem[c] = e;
  }
  p->fu = (int *)malloc(sizeof(int) * (size_t)(nnod + 1));
  p->fu[0] = 0;
  for (int i = 0; i < nnod; i++) p->fu[i + 1] = p->fu[i] + p->nvn + (is_cent[i] ? p->npres : 0);
  p->N = p->fu[nnod];

  /* node -> elements */
  int *ne_ptr = (int *)calloc((size_t)nnod + 1, sizeof(int));
  for (int e = 0; e < ne; e++)
    for (int k = 0; k < p->nn; k++) ne_ptr[p->conn[e * p->nn + k] + 1]++;
  for (int i = 0; i < nnod; i++) ne_ptr[i + 1] += ne_ptr[i];
  int *ne_list = (int *)malloc(sizeof(int) * (size_t)ne_ptr[nnod]);
  int *fill = (int *)calloc((size_t)nnod, sizeof(int));
  for (int e = 0; e < ne; e++)
    for (int k = 0; k < p->nn; k++) {
      int n = p->conn[e * p->nn + k];
      ne_list[ne_ptr[n] + fill[n]++] = e;
    }
  /* face neighbours: elements sharing a mid-side node (QUAD9 local 4..7,
   * HEX27 local 21..26) */
  const int side0 = dim == 2 ? 4 : 21, side1 = dim == 2 ? 8 : 27;

  /* node -> neighbour nodes, then rows */
  int maxnb = 8 * p->nn + 16;
  int *nb = (int *)malloc(sizeof(int) * (size_t)maxnb);
  int **nbl = (int **)malloc(sizeof(int *) * (size_t)nnod);
  int *nbn = (int *)malloc(sizeof(int) * (size_t)nnod);
  for (int n = 0; n < nnod; n++) {
    int cnt = 0;
    for (int q = ne_ptr[n]; q < ne_ptr[n + 1]; q++) {
      int e = ne_list[q];
      for (int k = 0; k < p->nn; k++) {
        int m = p->conn[e * p->nn + k], dup = 0;
        for (int r = 0; r < cnt; r++)
          if (nb[r] == m) {
            dup = 1;
            break;
          }
        if (!dup) nb[cnt++] = m;
      }
    }
    if (is_cent[n] && ne_ptr[n + 1] - ne_ptr[n] == 1) {
      int e = cent_elem[n];
      for (int k = side0; k < side1; k++) {
        int m = p->conn[e * p->nn + k];
        for (int q = ne_ptr[m]; q < ne_ptr[m + 1]; q++) {
          int f = ne_list[q];
          if (f == e) continue;
          int c = p->conn[f * p->nn + p->centroid], dup = 0;
          for (int r = 0; r < cnt; r++)
            if (nb[r] == c) {
              dup = 1;
              break;
            }
          if (!dup) nb[cnt++] = c;
        }
      }
    }
    qsort(nb, (size_t)cnt, sizeof(int), cmp_int);
    nbl[n] = (int *)malloc(sizeof(int) * (size_t)cnt);
    memcpy(nbl[n], nb, sizeof(int) * (size_t)cnt);
    nbn[n] = cnt;
  }
  /* Interaction mask (src/mm_unknown_map.c:1125 set_interaction_masks):
   * every equation couples with every variable except energy with
   * pressure (:1692; momentum :1226, species :1761 and continuity :2276 list
   * pressure).  An unknown's variable: offset < nvn is a nodal field
   * (offset == dim is T when energy is on), offset >= nvn is pressure. */
  long off = 0;
  for (int pass = 0; pass < 2; pass++) {
    long pos = p->N + 1;
    for (int n = 0; n < nnod; n++) {
      for (int i = p->fu[n]; i < p->fu[n + 1]; i++) {
        const int row_is_T = desc->energy && (i - p->fu[n]) == dim;
        if (pass) p->ija[i] = (int)pos;
        for (int r = 0; r < nbn[n]; r++) {
          int mm = nbl[n][r];
          for (int j = p->fu[mm]; j < p->fu[mm + 1]; j++) {
            if (j == i) continue;
            if (row_is_T && (j - p->fu[mm]) >= p->nvn) continue;
            if (pass) p->ija[pos] = j;
            pos++;
          }
        }
      }
    }
    if (!pass) {
      off = pos - (p->N + 1);
      p->msr_len = (long)p->N + 1 + off;
      /* beyond the reference's 32-bit MSR indexing: no pattern, element-level
       * use only (orc_element, orc_element_dofs, residual-only fills) */
      if (p->msr_len > INT_MAX) {
        p->ija = NULL;
        break;
      }
      p->ija = (int *)malloc(sizeof(int) * (size_t)p->msr_len);
    } else {
      p->ija[p->N] = (int)pos;
    }
  }

  /* integrated boundary conditions: owned copies, then per element */
  {
    const int nc = desc->num_ibc > 0 ? desc->num_ibc : 0;
    const int ns = nc ? desc->ibc_ptr[nc] : 0;
    p->ibc_type = (int *)malloc(sizeof(int) * (size_t)(nc + 1));
    p->ibc_value = (double *)malloc(sizeof(double) * (size_t)(2 * nc + 1));
    p->ibc_ptr = (int *)calloc((size_t)nc + 1, sizeof(int));
    p->ibc_elem = (int *)malloc(sizeof(int) * (size_t)(ns + 1));
    p->ibc_side = (int *)malloc(sizeof(int) * (size_t)(ns + 1));
    if (nc) {
      memcpy(p->ibc_type, desc->ibc_type, sizeof(int) * (size_t)nc);
      memcpy(p->ibc_value, desc->ibc_value, sizeof(double) * (size_t)(2 * nc));
      memcpy(p->ibc_ptr, desc->ibc_ptr, sizeof(int) * (size_t)(nc + 1));
      memcpy(p->ibc_elem, desc->ibc_elem, sizeof(int) * (size_t)ns);
      memcpy(p->ibc_side, desc->ibc_side, sizeof(int) * (size_t)ns);
    }
    p->d.num_ibc = nc;
    p->d.ibc_type = p->ibc_type;
    p->d.ibc_value = p->ibc_value;
    p->d.ibc_ptr = p->ibc_ptr;
    p->d.ibc_elem = p->ibc_elem;
    p->d.ibc_side = p->ibc_side;
    p->eibc_ptr = (int *)calloc((size_t)ne + 1, sizeof(int));
    p->eibc_card = (int *)malloc(sizeof(int) * (size_t)(ns + 1));
    p->eibc_side = (int *)malloc(sizeof(int) * (size_t)(ns + 1));
    for (int k = 0; k < ns; k++) p->eibc_ptr[p->ibc_elem[k] + 1]++;
    for (int e2 = 0; e2 < ne; e2++) p->eibc_ptr[e2 + 1] += p->eibc_ptr[e2];
    int *cnt = (int *)calloc((size_t)ne + 1, sizeof(int));
    for (int c = 0; c < nc; c++)
      for (int k = p->ibc_ptr[c]; k < p->ibc_ptr[c + 1]; k++) {
        const int el = p->ibc_elem[k], slot = p->eibc_ptr[el] + cnt[el]++;
        p->eibc_card[slot] = c;
        p->eibc_side[slot] = p->ibc_side[k];
      }
    free(cnt);
  }

  /* Dirichlet cards in order: a later card overwrites (src/mm_bc.c:132) */
  p->dbc = (int *)malloc(sizeof(int) * (size_t)p->N);
  p->dbc_val = (double *)calloc((size_t)p->N, sizeof(double));
  for (int i = 0; i < p->N; i++) p->dbc[i] = -1;
  for (int c = 0; c < desc->num_bc; c++) {
    int var = desc->bc_var[c], offv;
    if (var == GB_VAR_T) {
      if (!desc->energy) continue;
      offv = dim;
    } else if (var >= GB_VAR_Y(0)) {
      if (var - GB_VAR_Y(0) >= p->ns) continue;
      offv = dim + (desc->energy ? 1 : 0) + (var - GB_VAR_Y(0));
    } else if (var == GB_VAR_P) {
      /* first pressure unknown of a centroid node: PRESSURE DATUM of that
         element (src/mm_bc.c:418), one per independent member of a batch */
      offv = p->nvn;
    } else {
      offv = var;
    }
    for (int q = desc->bc_ptr[c]; q < desc->bc_ptr[c + 1]; q++) {
      int n = desc->bc_nodes[q];
      p->dbc[p->fu[n] + offv] = c;
      p->dbc_val[p->fu[n] + offv] = desc->bc_value[c];
    }
  }
  if (desc->pressure_datum_elem >= 0 && desc->pressure_datum_elem < ne) {
    int c = p->conn[desc->pressure_datum_elem * p->nn + p->centroid];
    int i = p->fu[c] + p->nvn;
    p->dbc[i] = -2;
    p->dbc_val[i] = desc->pressure_datum_value;
  }

  for (int n = 0; n < nnod; n++) free(nbl[n]);
  free(nbl);
  free(nbn);
  free(nb);
  free(fill);
  free(ne_list);
  free(ne_ptr);
  free(is_cent);
  free(cent_elem);
  return p;
}

void orc_destroy(orc_problem *p) {
  if (!p) return;
  free(p->coords);
  free(p->conn);
  free(p->fu);
  free(p->ija);
  free(p->dbc);
  free(p->dbc_val);
  free(p->ibc_type);
  free(p->ibc_value);
  free(p->ibc_ptr);
  free(p->ibc_elem);
  free(p->ibc_side);
  free(p->eibc_ptr);
  free(p->eibc_card);
  free(p->eibc_side);
  free(p);
}

int orc_num_unknowns(const orc_problem *p) { return p->N; }
long orc_msr_len(const orc_problem *p) { return p->msr_len; }
void orc_msr_pattern(const orc_problem *p, int *ija) {
  if (!p->ija) return;
  memcpy(ija, p->ija, sizeof(int) * (size_t)p->msr_len);
}
void orc_first_unknown(const orc_problem *p, int *fu) {
  memcpy(fu, p->fu, sizeof(int) * (size_t)(p->d.num_nodes + 1));
}
void orc_dirichlet_mask(const orc_problem *p, int *mask) {
  for (int i = 0; i < p->N; i++) mask[i] = p->dbc[i] != -1;
}
void orc_dirichlet_init(const orc_problem *p, double *x) {
  for (int i = 0; i < p->N; i++)
    if (p->dbc[i] != -1) x[i] = p->dbc_val[i];
}
int orc_local_size(const orc_problem *p) { return p->nloc; }

void orc_element_dofs(const orc_problem *p, int e, int *g) {
  const int nn = p->nn, dim = p->d.dim;
  const int *cn = p->conn + (size_t)e * nn;
  for (int a = 0; a < dim; a++)
    for (int k = 0; k < nn; k++) g[a * nn + k] = p->fu[cn[k]] + a;
  if (p->d.energy)
    for (int k = 0; k < nn; k++) g[dim * nn + k] = p->fu[cn[k]] + dim;
  const int oy = dim + (p->d.energy ? 1 : 0);
  for (int w = 0; w < p->ns; w++)
    for (int k = 0; k < nn; k++) g[(oy + w) * nn + k] = p->fu[cn[k]] + oy + w;
  for (int l = 0; l < p->npres; l++) g[p->nvn * nn + l] = p->fu[cn[p->centroid]] + p->nvn + l;
}

/* ------------------------------------------------------------- element */

/* One element's residual and Jacobian.  Follows, per quadrature point:
 *   geometry            beer_belly           src/mm_fill_util.c:140
 *   field values/grads  load_fv, load_fv_grads src/load_field_variables.c
 *   viscosity           viscosity / carreau_viscosity, calc_shearrate
 *                       src/mm_viscosity.c:108,:981, src/mm_fill_util.c:4564
 *   stress Pi = -P I + mu gamma and its derivatives
 *                       fluid_stress          src/mm_fill_momentum.c:2834
 *   body force          bouss_momentum_source src/mm_std_models.c:125
 *   momentum R, J_m_v, J_m_P, J_m_T           src/mm_fill_momentum.c:471-2116
 *   continuity R, J_c_v                       src/mm_fill_continuity.c:430-700
 *   energy R, J_e_T, J_e_v (Fourier flux)     src/mm_fill_energy.c:315-560,
 *                                             heat_flux :1629
 *   species R, J_s_c, J_s_v, J_s_T (Galerkin, steady, SPECIES_UNDEFINED_FORM
 *   so coeff_rho = 1; Fickian flux -D grad Y; CONSTANT or Arrhenius source)
 *                                             src/mm_fill_species.c:194-1710,
 *                                             fickian_flux :12414, sources
 *                                             :10100-10190
 * then the hard-set Dirichlet rows of put_dirichlet_in_matrix
 * (src/bc_dirich.c:44): row zeroed, diagonal DIRICHLET_PENALTY = 1,
 * residual 0. */
/* The integrated boundary conditions of one element side (apply_integrated_bc,
 * src/bc_integ.c): Gauss points on the side (find_surf_st,
 * src/el_elm_info.c:1987), sdet and the outward normal from the side's
 * tangents, R_i += w phi_i sdet func, J_ij += w phi_i sdet dfunc/dx_j. */
static void side_terms(const orc_problem *p, int card, int side, const double (*X)[3],
                       const double *Tn, double *Re, double *Je) {
  const int dim = p->d.dim, nn = p->nn, nloc = p->nloc, oT = dim * nn;
  /* side -> fixed reference coordinate and its value */
  static const int fix2[4][2] = {{1, -1}, {0, 1}, {1, 1}, {0, -1}};
  static const int fix3[6][2] = {{1, -1}, {0, 1}, {1, 1}, {0, -1}, {2, -1}, {2, 1}};
  const int fi = dim == 2 ? fix2[side - 1][0] : fix3[side - 1][0];
  const double fv = dim == 2 ? fix2[side - 1][1] : fix3[side - 1][1];
  int fr[2], nf = 0;
  for (int r = 0; r < dim; r++)
    if (r != fi) fr[nf++] = r;
  const double g[3] = {GQ_PT, 0.0, -GQ_PT}, gw[3] = {GQ_W0, GQ_W1, GQ_W0};
  const int type = p->ibc_type[card];
  const double v0 = p->ibc_value[2 * card], v1 = p->ibc_value[2 * card + 1];
  const int nq = dim == 2 ? 3 : 9;
  /* element centre (for the outward orientation) */
  double xc[3] = {0, 0, 0};
  {
    double xi0[3] = {0, 0, 0}, phc[27], dphc[27][3];
    q2_basis(dim, xi0, phc, dphc);
    for (int k = 0; k < nn; k++)
      for (int j = 0; j < dim; j++) xc[j] += phc[k] * X[k][j];
  }
  for (int iq = 0; iq < nq; iq++) {
    double xi[3] = {0, 0, 0}, w;
    xi[fi] = fv;
    xi[fr[0]] = g[iq % 3];
    w = gw[iq % 3];
    if (dim == 3) {
      xi[fr[1]] = g[iq / 3];
      w *= gw[iq / 3];
    }
    double phi[27], dphi[27][3];
    q2_basis(dim, xi, phi, dphi);
    double t[2][3] = {{0, 0, 0}, {0, 0, 0}}, xq[3] = {0, 0, 0}, T = 0.0;
    for (int k = 0; k < nn; k++) {
      for (int j = 0; j < dim; j++) {
        xq[j] += phi[k] * X[k][j];
        for (int m = 0; m < nf; m++) t[m][j] += dphi[k][fr[m]] * X[k][j];
      }
      T += phi[k] * Tn[k];
    }
    double n[3] = {0, 0, 0}, sdet;
    if (dim == 2) {
      sdet = sqrt(t[0][0] * t[0][0] + t[0][1] * t[0][1]);
      n[0] = t[0][1] / sdet;
      n[1] = -t[0][0] / sdet;
    } else {
      double c[3] = {t[0][1] * t[1][2] - t[0][2] * t[1][1], t[0][2] * t[1][0] - t[0][0] * t[1][2],
                     t[0][0] * t[1][1] - t[0][1] * t[1][0]};
      sdet = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
      for (int j = 0; j < 3; j++) n[j] = c[j] / sdet;
    }
    double o = 0.0;
    for (int j = 0; j < dim; j++) o += n[j] * (xq[j] - xc[j]);
    if (o < 0.0)
      for (int j = 0; j < dim; j++) n[j] = -n[j];
    const double ws = w * sdet;
    for (int i = 0; i < nn; i++) {
      const double wi = ws * phi[i];
      if (type == GB_IBC_QSIDE) {
        Re[oT + i] += wi * v0;
      } else if (type == GB_IBC_QCONV) {
        Re[oT + i] += wi * v0 * (v1 - T);
        for (int j = 0; j < nn; j++) Je[(size_t)(oT + i) * nloc + oT + j] += wi * (-v0 * phi[j]);
      } else if (type == GB_IBC_FLOW_PRESSURE) {
        for (int a = 0; a < dim; a++) Re[a * nn + i] += wi * (-v0 * n[a]);
      }
    }
  }
}

int orc_element(const orc_problem *p, int e, const double *x, double *Re, double *Je,
                int apply_bc) {
  const int nn = p->nn, dim = p->d.dim, nloc = p->nloc, nq = dim == 2 ? 9 : 27;
  const int en = p->d.energy, npr = p->npres, ns = p->ns;
  const int oT = dim * nn, oP = p->nvn * nn, oY = (dim + (en ? 1 : 0)) * nn;
  const gb_material *m = &p->d.mat;
  const int *cn = p->conn + (size_t)e * nn;
  int status = 0;
  double X[27][3], U[27][3], Tn[27], Pn[4], Yn[GB_MAX_SPECIES][27];
  /* nodal time derivatives of the transient terms (zero when steady) */
  double Ud[27][3], Tdn[27], Ydn[GB_MAX_SPECIES][27];
  const double *xd = p->xdot, mc = p->xdot ? p->mass_c : 0.0;
  int g[27 * (4 + GB_MAX_SPECIES) + 4];
  orc_element_dofs(p, e, g);
  for (int k = 0; k < nn; k++) {
    for (int j = 0; j < dim; j++) X[k][j] = p->coords[(size_t)cn[k] * dim + j];
    for (int a = 0; a < dim; a++) U[k][a] = x[g[a * nn + k]];
    Tn[k] = en ? x[g[oT + k]] : 0.0;
    for (int w = 0; w < ns; w++) Yn[w][k] = x[g[oY + w * nn + k]];
    for (int a = 0; a < dim; a++) Ud[k][a] = xd ? xd[g[a * nn + k]] : 0.0;
    Tdn[k] = (en && xd) ? xd[g[oT + k]] : 0.0;
    for (int w = 0; w < ns; w++) Ydn[w][k] = xd ? xd[g[oY + w * nn + k]] : 0.0;
  }
  for (int l = 0; l < npr; l++) Pn[l] = x[g[oP + l]];
  memset(Re, 0, sizeof(double) * (size_t)nloc);
  memset(Je, 0, sizeof(double) * (size_t)nloc * nloc);
#define JE(r, c) Je[(size_t)(r) * nloc + (c)]

  for (int iq = 0; iq < nq; iq++) {
    double xi[3], wq, phi[27], dphi[27][3], gphi[27][3];
    quad_point(dim, iq, xi, &wq);
    q2_basis(dim, xi, phi, dphi);
    /* J[i][j] = sum_k dphi_k/dxi_i * x_k,j ; B = J^-1 */
    double Jm[3][3] = {{0}}, B[3][3] = {{0}}, det;
    for (int i = 0; i < dim; i++)
      for (int j = 0; j < dim; j++) {
        double s = 0.0;
        for (int k = 0; k < nn; k++) s += dphi[k][i] * X[k][j];
        Jm[i][j] = s;
      }
    if (dim == 2) {
      det = Jm[0][0] * Jm[1][1] - Jm[0][1] * Jm[1][0];
      B[0][0] = Jm[1][1] / det;
      B[1][1] = Jm[0][0] / det;
      B[0][1] = -Jm[0][1] / det;
      B[1][0] = -Jm[1][0] / det;
    } else {
      det = Jm[0][0] * (Jm[1][1] * Jm[2][2] - Jm[1][2] * Jm[2][1]) -
            Jm[0][1] * (Jm[1][0] * Jm[2][2] - Jm[1][2] * Jm[2][0]) +
            Jm[0][2] * (Jm[1][0] * Jm[2][1] - Jm[1][1] * Jm[2][0]);
      B[0][0] = (Jm[1][1] * Jm[2][2] - Jm[2][1] * Jm[1][2]) / det;
      B[0][1] = -(Jm[0][1] * Jm[2][2] - Jm[2][1] * Jm[0][2]) / det;
      B[0][2] = (Jm[0][1] * Jm[1][2] - Jm[1][1] * Jm[0][2]) / det;
      B[1][0] = -(Jm[1][0] * Jm[2][2] - Jm[2][0] * Jm[1][2]) / det;
      B[1][1] = (Jm[0][0] * Jm[2][2] - Jm[2][0] * Jm[0][2]) / det;
      B[1][2] = -(Jm[0][0] * Jm[1][2] - Jm[1][0] * Jm[0][2]) / det;
      B[2][0] = (Jm[1][0] * Jm[2][1] - Jm[2][0] * Jm[1][1]) / det;
      B[2][1] = -(Jm[0][0] * Jm[2][1] - Jm[2][0] * Jm[0][1]) / det;
      B[2][2] = (Jm[0][0] * Jm[1][1] - Jm[1][0] * Jm[0][1]) / det;
    }
    if (!(det > 0.0)) status = -1;
    /* grad phi_k (physical) = B * dphi/dxi:  d/dx_p = sum_i B[p][i] d/dxi_i */
    for (int k = 0; k < nn; k++)
      for (int pp = 0; pp < dim; pp++) {
        double s = 0.0;
        for (int i = 0; i < dim; i++) s += B[pp][i] * dphi[k][i];
        gphi[k][pp] = s;
      }
    /* P1 pressure basis {1, s, t[, u]} in reference coordinates */
    double psi[4];
    psi[0] = 1.0;
    for (int i = 0; i < dim; i++) psi[1 + i] = xi[i];
    const double dA = wq * det;

    /* fields */
    double v[3] = {0}, gv[3][3] = {{0}}, T = 0.0, gT[3] = {0}, P = 0.0;
    for (int k = 0; k < nn; k++) {
      for (int a = 0; a < dim; a++) {
        v[a] += U[k][a] * phi[k];
        for (int pp = 0; pp < dim; pp++) gv[pp][a] += U[k][a] * gphi[k][pp];
      }
      if (en) {
        T += Tn[k] * phi[k];
        for (int pp = 0; pp < dim; pp++) gT[pp] += Tn[k] * gphi[k][pp];
      }
    }
    for (int l = 0; l < npr; l++) P += Pn[l] * psi[l];
    double Y[GB_MAX_SPECIES] = {0}, gY[GB_MAX_SPECIES][3] = {{0}};
    for (int w = 0; w < ns; w++)
      for (int k = 0; k < nn; k++) {
        Y[w] += Yn[w][k] * phi[k];
        for (int pp = 0; pp < dim; pp++) gY[w][pp] += Yn[w][k] * gphi[k][pp];
      }
    /* time derivatives at the point (load_fv: fv_dot, src/load_field_variables.c) */
    double vd[3] = {0, 0, 0}, Td = 0.0, Yd[GB_MAX_SPECIES] = {0};
    for (int k = 0; k < nn; k++) {
      for (int a = 0; a < dim; a++) vd[a] += Ud[k][a] * phi[k];
      Td += Tdn[k] * phi[k];
      for (int w = 0; w < ns; w++) Yd[w] += Ydn[w][k] * phi[k];
    }
    double divv = 0.0;
    for (int a = 0; a < dim; a++) divv += gv[a][a];
    double gam[3][3];
    for (int a = 0; a < dim; a++)
      for (int b = 0; b < dim; b++) gam[a][b] = gv[a][b] + gv[b][a];

    /* viscosity and d mu / d v_{b,j} */
    double mu, dmu_dgd = 0.0, gd = 0.0;
    if (m->viscosity_model == GB_VISC_CARREAU) {
      double s = 0.0;
      for (int a = 0; a < dim; a++)
        for (int b = 0; b < dim; b++) s += gam[a][b] * gam[b][a];
      gd = sqrt(0.5 * fabs(s));
      double val2 = gd > 1.0e-298 ? pow(m->lambda * gd, m->aexp) : 0.0;
      mu = m->mu_inf + (m->mu0 - m->mu_inf) * pow(1.0 + val2, (m->nexp - 1.0) / m->aexp);
      double val = gd > 1.0e-298 ? pow(m->lambda * gd, m->aexp - 1.0) : 0.0;
      double val1 = pow(1.0 + val2, (m->nexp - 1.0 - m->aexp) / m->aexp);
      dmu_dgd = (m->mu0 - m->mu_inf) * (m->nexp - 1.0) * m->lambda * val * val1;
    } else {
      mu = m->viscosity;
    }
    /* dmu_v[b][j] = dmu/dgd * (sum_p dphi_j/dx_p gam[b][p]) / gd */
    double dmu_v[3][27];
    for (int b = 0; b < dim; b++)
      for (int j = 0; j < nn; j++) {
        double s = 0.0;
        if (m->viscosity_model == GB_VISC_CARREAU && gd != 0.0 && gd > 1.0e-298) {
          for (int pp = 0; pp < dim; pp++) s += gphi[j][pp] * gam[b][pp];
          s = dmu_dgd * (s / gd);
        }
        dmu_v[b][j] = s;
      }
    double Pi[3][3];
    for (int a = 0; a < dim; a++)
      for (int b = 0; b < dim; b++) Pi[a][b] = (a == b ? -P : 0.0) + mu * gam[a][b];

    /* body force f and df/dT_j = dfT[a] * phi_j */
    double f[3] = {0, 0, 0}, dfT[3] = {0, 0, 0};
    if (m->momentum_source_model == GB_SOURCE_BOUSSINESQ) {
      if (en)
        for (int a = 0; a < dim; a++) {
          f[a] = m->density * m->momentum_source[a] *
                 (-m->volume_expansion * (T - m->reference_temperature));
          dfT[a] = -m->density * m->momentum_source[a] * m->volume_expansion;
        }
    } else {
      for (int a = 0; a < dim; a++) f[a] = m->momentum_source[a];
    }
    const double rho = m->density, rcp = m->density * m->heat_capacity, kc = m->conductivity;
    /* heat source (heat_source, src/mm_fill_energy.c:1724): CONSTANT, or the
     * USER model c0 exp(c1 T) (usr_heat_source, src/user_mp.c:472) */
    double hsrc = 0.0, dhsrc = 0.0;
    if (m->heat_source_model == GB_HEAT_SOURCE_CONSTANT) {
      hsrc = m->heat_source[0];
    } else if (m->heat_source_model == GB_HEAT_SOURCE_EXPONENTIAL) {
      hsrc = m->heat_source[0] * exp(m->heat_source[1] * T);
      dhsrc = m->heat_source[1] * hsrc;
    }

    /* momentum */
    for (int a = 0; a < dim; a++) {
      double adv_a = 0.0;
      for (int pp = 0; pp < dim; pp++) adv_a += v[pp] * gv[pp][a];
      for (int i = 0; i < nn; i++) {
        const int ri = a * nn + i;
        double adv = adv_a * rho * (-phi[i] * dA);
        double dif = 0.0;
        for (int pp = 0; pp < dim; pp++) dif += gphi[i][pp] * Pi[a][pp];
        dif *= -dA;
        double src = f[a] * (phi[i] * dA);
        /* mass term -rho v_dot_a phi_i dA (src/mm_fill_momentum.c:471-500) */
        double mass = -rho * vd[a] * phi[i] * dA;
        Re[ri] += mass + adv + dif + src;
        /* its sensitivity -(1 + 2 theta) / dt rho phi_i phi_j dA (:1586-1590) */
        if (mc != 0.0)
          for (int j = 0; j < nn; j++) JE(ri, a * nn + j) += -mc * rho * phi[i] * phi[j] * dA;
        /* J_m_v */
        double gi_dot_gam = 0.0;
        for (int pp = 0; pp < dim; pp++) gi_dot_gam += gphi[i][pp] * gam[a][pp];
        for (int b = 0; b < dim; b++)
          for (int j = 0; j < nn; j++) {
            double adv_j = phi[j] * gv[b][a];
            if (a == b)
              for (int pp = 0; pp < dim; pp++) adv_j += v[pp] * gphi[j][pp];
            adv_j *= rho * (-phi[i] * dA);
            double dd = mu * gphi[i][b] * gphi[j][a];
            if (a == b)
              for (int pp = 0; pp < dim; pp++) dd += mu * gphi[i][pp] * gphi[j][pp];
            dd += dmu_v[b][j] * gi_dot_gam;
            dd *= -dA;
            JE(ri, b * nn + j) += adv_j + dd;
          }
        /* J_m_P */
        for (int l = 0; l < npr; l++) JE(ri, oP + l) += gphi[i][a] * psi[l] * dA;
        /* J_m_T */
        if (en)
          for (int j = 0; j < nn; j++) JE(ri, oT + j) += phi[i] * (dfT[a] * phi[j]) * dA;
      }
    }
    /* continuity */
    for (int l = 0; l < npr; l++) {
      const int rl = oP + l;
      Re[rl] += divv * (psi[l] * dA);
      for (int b = 0; b < dim; b++)
        for (int j = 0; j < nn; j++) JE(rl, b * nn + j) += psi[l] * gphi[j][b] * dA;
    }
    /* energy */
    if (en) {
      double vgT = 0.0;
      for (int pp = 0; pp < dim; pp++) vgT += v[pp] * gT[pp];
      for (int i = 0; i < nn; i++) {
        const int ri = oT + i;
        double adv = vgT * (-phi[i] * rcp * dA);
        double dif = 0.0;
        for (int pp = 0; pp < dim; pp++) dif += gphi[i][pp] * (-kc * gT[pp]);
        dif *= dA;
        /* mass term -rho Cp T_dot phi_i dA (src/mm_fill_energy.c:315-381),
         * heat source phi_i h dA (:374-378) */
        Re[ri] += adv + dif - rcp * Td * phi[i] * dA + hsrc * phi[i] * dA;
        for (int j = 0; j < nn; j++) JE(ri, oT + j) += dhsrc * phi[i] * phi[j] * dA;
        if (mc != 0.0)
          for (int j = 0; j < nn; j++) JE(ri, oT + j) += -mc * rcp * phi[i] * phi[j] * dA;
        for (int j = 0; j < nn; j++) {
          double vgj = 0.0, gij = 0.0;
          for (int pp = 0; pp < dim; pp++) {
            vgj += v[pp] * gphi[j][pp];
            gij += gphi[i][pp] * gphi[j][pp];
          }
          JE(ri, oT + j) += rcp * vgj * (-phi[i] * dA) - kc * gij * dA;
          for (int b = 0; b < dim; b++)
            JE(ri, b * nn + j) += rcp * phi[j] * gT[b] * (-phi[i] * dA);
        }
      }
    }
    /* species: source S_w and its sensitivities (usr_species_source /
     * CONSTANT, src/mm_fill_species.c:10117,:10146-10190) */
    for (int w = 0; w < ns; w++) {
      double S = 0.0, dSdT = 0.0, dSdY[GB_MAX_SPECIES] = {0};
      const double *sp = m->species_source[w];
      if (m->species_source_model[w] == GB_SPECIES_SOURCE_CONSTANT) {
        S = sp[0];
      } else if (m->species_source_model[w] == GB_SPECIES_SOURCE_ARRHENIUS) {
        const int src = (int)sp[3];
        const double r = sp[0] * exp(-sp[1] / T);
        S = sp[2] * r * Y[src];
        dSdT = S * sp[1] / (T * T);
        dSdY[src] = sp[2] * r;
      }
      const double D = m->diffusivity[w];
      double vgY = 0.0;
      for (int pp = 0; pp < dim; pp++) vgY += v[pp] * gY[w][pp];
      for (int i = 0; i < nn; i++) {
        const int ri = oY + w * nn + i;
        /* advection -phi_i (v . grad Y_w), diffusion grad phi_i . (-D grad Y_w),
         * source phi_i S_w (:572-665) */
        double dif = 0.0;
        for (int pp = 0; pp < dim; pp++) dif += gphi[i][pp] * (-D * gY[w][pp]);
        Re[ri] += -vgY * phi[i] * dA + dif * dA + S * phi[i] * dA;
        /* mass term -Y_dot_w phi_i dA, with the advection term's unit
         * coefficient (src/mm_fill_species.c:525-551) */
        Re[ri] += -Yd[w] * phi[i] * dA;
        if (mc != 0.0)
          for (int j = 0; j < nn; j++) JE(ri, oY + w * nn + j) += -mc * phi[i] * phi[j] * dA;
        for (int j = 0; j < nn; j++) {
          double vgj = 0.0, gij = 0.0;
          for (int pp = 0; pp < dim; pp++) {
            vgj += v[pp] * gphi[j][pp];
            gij += gphi[i][pp] * gphi[j][pp];
          }
          const double pij = phi[i] * phi[j] * dA;
          /* J_s_c (:760-904): advection and diffusion on the diagonal species,
           * the source on every species it depends on */
          JE(ri, oY + w * nn + j) += -phi[i] * vgj * dA - D * gij * dA;
          for (int w1 = 0; w1 < ns; w1++)
            if (dSdY[w1] != 0.0) JE(ri, oY + w1 * nn + j) += dSdY[w1] * pij;
          /* J_s_v (:906-1000): d(v . grad Y_w)/d v_b = phi_j dY_w/dx_b */
          for (int b = 0; b < dim; b++) JE(ri, b * nn + j) += -gY[w][b] * pij;
          /* J_s_T: source only (constant diffusivity) */
          if (en && dSdT != 0.0) JE(ri, oT + j) += dSdT * pij;
        }
      }
    }
  }
  /* integrated boundary conditions of this element's sides */
  for (int k = p->eibc_ptr[e]; k < p->eibc_ptr[e + 1]; k++)
    side_terms(p, p->eibc_card[k], p->eibc_side[k], (const double (*)[3])X, Tn, Re, Je);
  if (apply_bc) {
    for (int r = 0; r < nloc; r++) {
      if (p->dbc[g[r]] == -1) continue;
      for (int c = 0; c < nloc; c++) JE(r, c) = 0.0;
      JE(r, r) = 1.0;
      Re[r] = 0.0;
    }
  }
#undef JE
  return status;
}

/* Scatter of load_lec (src/mm_fill.c:5241): a[diag] / a[off-diag slot]
 * += element entries, elements in order. */
/* The element loop of matrix_fill_full (src/mm_fill.c:158-312) over either
 * the range [e0, e1) (elems == NULL) or the list elems[e0 .. e1). */
static int fill_elements(const orc_problem *p, const double *x, double *R, double *a,
                         const int *elems, int e0, int e1) {
  const int nloc = p->nloc;
  double *Re = (double *)malloc(sizeof(double) * (size_t)nloc);
  double *Je = (double *)malloc(sizeof(double) * (size_t)nloc * nloc);
  int g[27 * (4 + GB_MAX_SPECIES) + 4];
  int status = 0;
  for (int k = e0; k < e1; k++) {
    const int e = elems ? elems[k] : k;
    if (orc_element(p, e, x, Re, Je, 1) != 0) status = -1;
    orc_element_dofs(p, e, g);
    for (int r = 0; r < nloc; r++) {
      const int gr = g[r];
      R[gr] += Re[r];
      if (!a) continue;
      const int s0 = p->ija[gr], s1 = p->ija[gr + 1];
      for (int c = 0; c < nloc; c++) {
        const int gc = g[c];
        const double v = Je[(size_t)r * nloc + c];
        if (gc == gr) {
          a[gr] += v;
          continue;
        }
        int lo = s0, hi = s1 - 1; /* columns ascend: bisection */
        while (lo <= hi) {
          int mid = (lo + hi) >> 1;
          if (p->ija[mid] < gc)
            lo = mid + 1;
          else
            hi = mid - 1;
        }
        if (lo >= s1 || p->ija[lo] != gc) {
          /* masked pair (energy row, pressure column): always zero */
          if (v == 0.0) continue;
          fprintf(stderr, "oracle: missing MSR slot (%d,%d)\n", gr, gc);
          abort();
        }
        a[lo] += v;
      }
    }
  }
  free(Re);
  free(Je);
  return status;
}

void orc_set_transient(orc_problem *p, const double *xdot, double mass_c) {
  p->xdot = xdot;
  p->mass_c = mass_c;
}

int orc_matrix_fill(const orc_problem *p, const double *x, double *R, double *a, int e0, int e1) {
  if (a && !p->ija) return -2;
  return fill_elements(p, x, R, a, NULL, e0, e1);
}

int orc_matrix_fill_list(const orc_problem *p, const double *x, double *R, double *a,
                         const int *elems, int n) {
  if (a && !p->ija) return -2;
  return fill_elements(p, x, R, a, elems, 0, n);
}

/* Greedy element colouring: each element takes the smallest colour that no
 * element sharing one of its nodes has taken yet, in element order. */
int orc_element_colors(const orc_problem *p, int *color) {
  const int ne = p->d.num_elems, nn = p->nn;
  unsigned long long *used =
      (unsigned long long *)calloc((size_t)p->d.num_nodes, sizeof(unsigned long long));
  if (!used) return -1;
  int ncol = 0;
  for (int e = 0; e < ne; e++) {
    unsigned long long m = 0;
    for (int k = 0; k < nn; k++) m |= used[p->conn[(size_t)e * nn + k]];
    int c = 0;
    while (c < 64 && (m >> c) & 1ULL) c++;
    if (c == 64) {
      free(used);
      return -1;
    }
    color[e] = c;
    if (c + 1 > ncol) ncol = c + 1;
    for (int k = 0; k < nn; k++) used[p->conn[(size_t)e * nn + k]] |= 1ULL << c;
  }
  free(used);
  return ncol;
}

/* row_sum_scale_MSR (src/sl_matrix_util.c:506) */
void orc_row_sum_scale(const orc_problem *p, double *a, double *R, double *scale) {
  for (int i = 0; i < p->N; i++) {
    double s = fabs(a[i]);
    for (int k = p->ija[i]; k < p->ija[i + 1]; k++) s += fabs(a[k]);
    if (fabs(a[i]) > 1.0e-200) s = a[i] < 0.0 ? -s : s;
    if (s == 0.0) s = 1.0; /* the reference warns and keeps going */
    scale[i] = s;
    R[i] = R[i] / s;
    a[i] = a[i] / s;
    for (int k = p->ija[i]; k < p->ija[i + 1]; k++) a[k] /= s;
  }
}

/* ILU(0) of an MSR matrix with a pivot floor, row by row in the IKJ order
 * (Saad, Iterative Methods for Sparse Linear Systems, 2nd ed., Alg. 10.4):
 * row i is eliminated with the finished rows k < i of its pattern, fill
 * outside the pattern is dropped, then a pivot below tau in magnitude
 * becomes +-tau.  The reference's preconditioner is AztecOO's ILU(0)
 * (third-party, not in the reference tree); this restates the published
 * algorithm to check the GPU factors. */
int orc_ilu0(const orc_problem *p, const double *a, double tau, double *lu) {
  const int N = p->N;
  const int *ija = p->ija;
  memcpy(lu, a, sizeof(double) * (size_t)p->msr_len);
  long *pos = (long *)malloc(sizeof(long) * (size_t)N);
  if (!pos) return -1;
  for (int j = 0; j < N; j++) pos[j] = -1;
  for (int i = 0; i < N; i++) {
    pos[i] = i;
    for (int k = ija[i]; k < ija[i + 1]; k++) pos[ija[k]] = k;
    for (int k = ija[i]; k < ija[i + 1]; k++) {
      const int j = ija[k];
      if (j >= i) break; /* off-diagonal columns ascend */
      const double l = lu[k] / lu[j];
      lu[k] = l;
      for (int kk = ija[j]; kk < ija[j + 1]; kk++) {
        const int c = ija[kk];
        if (c <= j || pos[c] < 0) continue;
        lu[pos[c]] -= l * lu[kk];
      }
    }
    if (fabs(lu[i]) < tau) lu[i] = lu[i] < 0.0 ? -tau : tau;
    pos[i] = -1;
    for (int k = ija[i]; k < ija[i + 1]; k++) pos[ija[k]] = -1;
  }
  free(pos);
  return 0;
}

/* Banded Gaussian elimination with partial pivoting on the MSR system
 * (the oracle's stand-in for the Krylov solve; only converged fields are
 * compared). */
static int band_solve(int N, const int *ija, const double *a, double *xb) {
  int kl = 0, ku = 0;
  for (int i = 0; i < N; i++)
    for (int k = ija[i]; k < ija[i + 1]; k++) {
      int j = ija[k];
      if (i - j > kl) kl = i - j;
      if (j - i > ku) ku = j - i;
    }
  const long w = 2L * kl + ku + 1;
  double *Bd = (double *)calloc((size_t)N * (size_t)w, sizeof(double));
  if (!Bd) return -1;
#define BD(i, j) Bd[(size_t)(i) * (size_t)w + (size_t)((j) - (i) + kl)]
  for (int i = 0; i < N; i++) {
    BD(i, i) = a[i];
    for (int k = ija[i]; k < ija[i + 1]; k++) BD(i, ija[k]) += a[k];
  }
  for (int c = 0; c < N; c++) {
    int last = c + kl < N - 1 ? c + kl : N - 1, piv = c;
    double best = fabs(BD(c, c));
    for (int r = c + 1; r <= last; r++)
      if (fabs(BD(r, c)) > best) {
        best = fabs(BD(r, c));
        piv = r;
      }
    if (best == 0.0) {
      free(Bd);
      return -1;
    }
    int cmax = c + kl + ku < N - 1 ? c + kl + ku : N - 1;
    if (piv != c) {
      for (int j = c; j <= cmax; j++) {
        double t = BD(c, j);
        BD(c, j) = BD(piv, j);
        BD(piv, j) = t;
      }
      double t = xb[c];
      xb[c] = xb[piv];
      xb[piv] = t;
    }
    for (int r = c + 1; r <= last; r++) {
      double fct = BD(r, c) / BD(c, c);
      if (fct == 0.0) continue;
      BD(r, c) = 0.0;
      for (int j = c + 1; j <= cmax; j++) BD(r, j) -= fct * BD(c, j);
      xb[r] -= fct * xb[c];
    }
  }
  for (int i = N - 1; i >= 0; i--) {
    int cmax = i + kl + ku < N - 1 ? i + kl + ku : N - 1;
    double s = xb[i];
    for (int j = i + 1; j <= cmax; j++) s -= BD(i, j) * xb[j];
    xb[i] = s / BD(i, i);
  }
#undef BD
  free(Bd);
  return 0;
}

/* Newton loop of solve_nonlinear_problem (src/mm_sol_nonlinear.c:1108):
 * assemble, row-sum scale, converged when after at least one update the
 * scaled residual has L2 and L-infinity norms below tol (:1482-1486),
 * otherwise solve and take the full step x -= dx (:2553-2557). */
/* Newton with the banded direct solve; with xdot (transient) the time
 * derivative follows every update, xdot -= (1 + 2 theta) / dt * dx
 * (src/mm_sol_nonlinear.c:2553-2562). */
static int newton_impl(const orc_problem *p, double *x, double *xdot, int max_it, double tol,
                       double *norms) {
  const int N = p->N;
  double *R = (double *)malloc(sizeof(double) * (size_t)N);
  double *a = (double *)malloc(sizeof(double) * (size_t)p->msr_len);
  double *sc = (double *)malloc(sizeof(double) * (size_t)N);
  int result = -1;
  for (int it = 0; it < max_it; it++) {
    memset(R, 0, sizeof(double) * (size_t)N);
    memset(a, 0, sizeof(double) * (size_t)p->msr_len);
    if (orc_matrix_fill(p, x, R, a, 0, p->d.num_elems) != 0) break;
    orc_row_sum_scale(p, a, R, sc);
    double l2 = 0.0, loo = 0.0;
    for (int i = 0; i < N; i++) {
      l2 += R[i] * R[i];
      if (fabs(R[i]) > loo) loo = fabs(R[i]);
    }
    l2 = sqrt(l2);
    if (norms) norms[it] = l2;
    if (!isfinite(l2)) break;
    if (it > 0 && l2 < tol && loo < tol) {
      result = it;
      break;
    }
    if (band_solve(N, p->ija, a, R) != 0) break;
    for (int i = 0; i < N; i++) x[i] -= R[i];
    if (xdot)
      for (int i = 0; i < N; i++) xdot[i] -= p->mass_c * R[i];
  }
  free(R);
  free(a);
  free(sc);
  return result;
}

int orc_newton(const orc_problem *p, double *x, int max_it, double tol, double *norms) {
  return newton_impl(p, x, NULL, max_it, tol, norms);
}

int orc_newton_transient(orc_problem *p, double *x, double *xdot, double mass_c, int max_it,
                         double tol, double *norms) {
  orc_set_transient(p, xdot, mass_c);
  const int r = newton_impl(p, x, xdot, max_it, tol, norms);
  orc_set_transient(p, NULL, 0.0);
  return r;
}

/* y = A x for an MSR matrix (src/sl_auxutil.c:373, MV_MSR). */
static void msr_matvec(int N, const int *ija, const double *a, const double *x, double *y) {
  for (int i = 0; i < N; i++) {
    double s = a[i] * x[i];
    for (int k = ija[i]; k < ija[i + 1]; k++) s += a[k] * x[ija[k]];
    y[i] = s;
  }
}

/* z = (LU)^-1 z in place with ILU(0) factors in the MSR layout: unit lower
 * triangle below the diagonal, U on and above it. */
static void ilu0_apply(int N, const int *ija, const double *lu, double *z) {
  for (int i = 0; i < N; i++) {
    double s = z[i];
    for (int k = ija[i]; k < ija[i + 1] && ija[k] < i; k++) s -= lu[k] * z[ija[k]];
    z[i] = s;
  }
  for (int i = N - 1; i >= 0; i--) {
    double s = z[i];
    for (int k = ija[i + 1] - 1; k >= ija[i] && ija[k] > i; k--) s -= lu[k] * z[ija[k]];
    z[i] = s / lu[i];
  }
}

static double dot(int N, const double *x, const double *y) {
  double s = 0.0;
  for (int i = 0; i < N; i++) s += x[i] * y[i];
  return s;
}

/* Restarted GMRES(m), right-preconditioned, modified Gram-Schmidt and
 * Givens rotations (Saad, Iterative Methods for Sparse Linear Systems, 2nd
 * ed., Alg. 9.5).  The reference's Krylov solver is AztecOO's GMRES with
 * ILU(0) on one subdomain (third-party, Trilinos, not in the reference
 * tree; options from src/sl_util.c:417,556); this restates the published
 * algorithm so a CPU Krylov solve can be timed next to the GPU's. */
int orc_gmres_ilu0(const orc_problem *p, const double *a, const double *lu, const double *b,
                   double *x, int m, int maxit, double tol, int *its, double *relres) {
  const int N = p->N;
  const int *ija = p->ija;
  double *V = (double *)malloc(sizeof(double) * (size_t)N * (size_t)(m + 1));
  double *z = (double *)malloc(sizeof(double) * (size_t)N);
  double *w = (double *)malloc(sizeof(double) * (size_t)N);
  double *H = (double *)calloc((size_t)(m + 1) * (size_t)m, sizeof(double));
  double *cs = (double *)malloc(sizeof(double) * (size_t)m);
  double *sn = (double *)malloc(sizeof(double) * (size_t)m);
  double *g = (double *)malloc(sizeof(double) * (size_t)(m + 1));
  double *yv = (double *)malloc(sizeof(double) * (size_t)m);
  int result = -1, k_total = 0;
  double rel = 1.0;
  if (!V || !z || !w || !H || !cs || !sn || !g || !yv) goto done;
  for (int i = 0; i < N; i++) x[i] = 0.0;
  const double bnorm = sqrt(dot(N, b, b));
  if (bnorm == 0.0) {
    result = 0;
    rel = 0.0;
    goto done;
  }
  memcpy(w, b, sizeof(double) * (size_t)N); /* r0 = b - A 0 */
  result = 1;
  while (k_total < maxit) {
    const double beta = sqrt(dot(N, w, w));
    rel = beta / bnorm;
    if (rel <= tol) {
      result = 0;
      break;
    }
    for (int i = 0; i < N; i++) V[i] = w[i] / beta;
    for (int i = 0; i <= m; i++) g[i] = 0.0;
    g[0] = beta;
    int j = 0;
    for (; j < m && k_total < maxit; j++) {
      double *vj = V + (size_t)j * N, *vn = V + (size_t)(j + 1) * N;
      memcpy(z, vj, sizeof(double) * (size_t)N);
      ilu0_apply(N, ija, lu, z);
      msr_matvec(N, ija, a, z, vn);
      for (int i = 0; i <= j; i++) {
        const double *vi = V + (size_t)i * N;
        const double h = dot(N, vn, vi);
        H[i * m + j] = h;
        for (int q = 0; q < N; q++) vn[q] -= h * vi[q];
      }
      const double hn = sqrt(dot(N, vn, vn));
      H[(j + 1) * m + j] = hn;
      if (hn > 0.0)
        for (int q = 0; q < N; q++) vn[q] /= hn;
      for (int i = 0; i < j; i++) { /* earlier rotations on column j */
        const double t = cs[i] * H[i * m + j] + sn[i] * H[(i + 1) * m + j];
        H[(i + 1) * m + j] = -sn[i] * H[i * m + j] + cs[i] * H[(i + 1) * m + j];
        H[i * m + j] = t;
      }
      const double hd = H[j * m + j], hs = H[(j + 1) * m + j];
      const double r = sqrt(hd * hd + hs * hs);
      cs[j] = r > 0.0 ? hd / r : 1.0;
      sn[j] = r > 0.0 ? hs / r : 0.0;
      H[j * m + j] = r;
      H[(j + 1) * m + j] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      k_total++;
      if (fabs(g[j + 1]) <= tol * bnorm) {
        j++;
        break;
      }
    }
    /* y = H^-1 g (upper triangular, j columns), x += M^-1 V y */
    for (int i = j - 1; i >= 0; i--) {
      double s = g[i];
      for (int c = i + 1; c < j; c++) s -= H[i * m + c] * yv[c];
      yv[i] = H[i * m + i] != 0.0 ? s / H[i * m + i] : 0.0;
    }
    for (int q = 0; q < N; q++) z[q] = 0.0;
    for (int i = 0; i < j; i++) {
      const double *vi = V + (size_t)i * N;
      for (int q = 0; q < N; q++) z[q] += yv[i] * vi[q];
    }
    ilu0_apply(N, ija, lu, z);
    for (int q = 0; q < N; q++) x[q] += z[q];
    msr_matvec(N, ija, a, x, w); /* true residual for the restart */
    for (int q = 0; q < N; q++) w[q] = b[q] - w[q];
  }
  if (result == 1) {
    rel = sqrt(dot(N, w, w)) / bnorm;
    if (rel <= tol) result = 0;
  }
done:
  if (its) *its = k_total;
  if (relres) *relres = rel;
  free(V);
  free(z);
  free(w);
  free(H);
  free(cs);
  free(sn);
  free(g);
  free(yv);
  return result;
}

/* Newton loop of solve_nonlinear_problem (src/mm_sol_nonlinear.c:1108) as in
 * orc_newton, with the linear solve done by ILU(0)-GMRES(m) on the row-sum
 * scaled system (the reference's AZTECOO case, :1805). */
int orc_newton_gmres(const orc_problem *p, double *x, int max_it, double tol, double lin_tol,
                     int m, int lin_maxit, double tau, int *linear_its, double *norms) {
  const int N = p->N;
  double *R = (double *)malloc(sizeof(double) * (size_t)N);
  double *dx = (double *)malloc(sizeof(double) * (size_t)N);
  double *a = (double *)malloc(sizeof(double) * (size_t)p->msr_len);
  double *lu = (double *)malloc(sizeof(double) * (size_t)p->msr_len);
  double *sc = (double *)malloc(sizeof(double) * (size_t)N);
  int result = -1, lin_total = 0;
  if (!R || !dx || !a || !lu || !sc) goto done;
  for (int it = 0; it < max_it; it++) {
    memset(R, 0, sizeof(double) * (size_t)N);
    memset(a, 0, sizeof(double) * (size_t)p->msr_len);
    if (orc_matrix_fill(p, x, R, a, 0, p->d.num_elems) != 0) break;
    orc_row_sum_scale(p, a, R, sc);
    double l2 = 0.0, loo = 0.0;
    for (int i = 0; i < N; i++) {
      l2 += R[i] * R[i];
      if (fabs(R[i]) > loo) loo = fabs(R[i]);
    }
    l2 = sqrt(l2);
    if (norms) norms[it] = l2;
    if (!isfinite(l2)) break;
    if (it > 0 && l2 < tol && loo < tol) {
      result = it;
      break;
    }
    if (orc_ilu0(p, a, tau, lu) != 0) break;
    int its = 0;
    if (orc_gmres_ilu0(p, a, lu, R, dx, m, lin_maxit, lin_tol, &its, NULL) < 0) break;
    lin_total += its;
    for (int i = 0; i < N; i++) x[i] -= dx[i];
  }
done:
  if (linear_its) *linear_its = lin_total;
  free(R);
  free(dx);
  free(a);
  free(lu);
  free(sc);
  return result;
}

/* ------------------------------------------------- mesh generator access */
#include "mesh_gen.h"

int orc_mesh_sizes(const char *spec, int *num_nodes, int *num_elems, int *set_total) {
  gb_mesh m;
  if (gb_mesh_build_from_spec(&m, spec) != 0) return -1;
  *num_nodes = m.num_nodes;
  *num_elems = m.num_elems;
  *set_total = 0;
  for (int s = 0; s < m.num_sets; s++) *set_total += m.set_len[s];
  gb_mesh_free(&m);
  return 0;
}

int orc_mesh_fill(const char *spec, double *coords, int *conn, int *set_len, int *set_nodes) {
  gb_mesh m;
  if (gb_mesh_build_from_spec(&m, spec) != 0) return -1;
  for (int i = 0; i < m.num_nodes; i++) {
    coords[(size_t)i * m.dim + 0] = m.x[i];
    coords[(size_t)i * m.dim + 1] = m.y[i];
    if (m.dim == 3) coords[(size_t)i * m.dim + 2] = m.z[i];
  }
  memcpy(conn, m.conn, sizeof(int) * (size_t)m.num_elems * m.nodes_per_elem);
  int off = 0;
  for (int s = 0; s < m.num_sets; s++) {
    set_len[s] = m.set_len[s];
    memcpy(set_nodes + off, m.set_nodes[s], sizeof(int) * (size_t)m.set_len[s]);
    off += m.set_len[s];
  }
  gb_mesh_free(&m);
  return 0;
}
