/* Problem description shared by the GB300 Newton library (libgbnewton.so)
 * and its CPU oracle: a Q2/P1 finite-element mesh, one material and its
 * strong (Dirichlet) boundary conditions, as plain arrays.
 *
 * It carries what the reference reads from its input deck, material file
 * and Exodus mesh for the path this library replaces:
 *   - mesh: coordinates and QUAD9/HEX27 connectivity in the Exodus/Goma local
 *     node order (src/rf_shape.c:361 BIQUAD_QUAD, :1105 TRIQUAD_HEX);
 *   - equations: momentum (Q2), continuity (P1 discontinuous pressure,
 *     basis {1,s,t[,u]} in reference coordinates), optional energy (Q2),
 *     optional dilute species (Q2, "EQ = species_bulk", FICKIAN flux with
 *     constant diffusivity, SPECIES_UNDEFINED_FORM; assemble_mass_transport
 *     src/mm_fill_species.c:194, fickian_flux :12414);
 *   - material: density, Newtonian or Carreau-Yasuda viscosity
 *     (src/mm_viscosity.c:981), heat capacity, Fourier conductivity,
 *     CONSTANT or BOUSSINESQ momentum source (src/mm_std_models.c:125);
 *   - heat source of the energy equation: CONSTANT, or c0 exp(c1 T) as a
 *     USER model (usr_heat_source, src/user_mp.c:472);
 *   - species sources: CONSTANT, or the Arrhenius rate of a USER model
 *     (usr_species_source, src/user_mp.c:598, called from
 *     src/mm_fill_species.c:10146):  S_w = nu k0 exp(-E/T) Y_s;
 *   - "BC = U|V|W|T NS <id> <value>" and "BC = Y NS <id> <w> <value>"
 *     cards in deck order
 *     (src/mm_input_bc.c), hard-set Dirichlet (src/bc_dirich.c:44), and the
 *     PRESSURE DATUM card (src/mm_input_bc.c:3215, src/mm_bc.c:388).
 */
#ifndef GB_PROBLEM_H
#define GB_PROBLEM_H

#ifdef __cplusplus
extern "C" {
#endif

/* Variable numbering follows the reference's variable types
 * (include/rf_fem_const.h:174-200). */
#define GB_VAR_U1 0
#define GB_VAR_U2 1
#define GB_VAR_U3 2
#define GB_VAR_T 3
#define GB_VAR_P 9
/* species w (the reference's MASS_FRACTION variable, sub-variable w) */
#define GB_VAR_Y(w) (100 + (w))

#define GB_MAX_SPECIES 4

#define GB_SPECIES_SOURCE_NONE 0
#define GB_SPECIES_SOURCE_CONSTANT 1
#define GB_SPECIES_SOURCE_ARRHENIUS 2

#define GB_VISC_NEWTONIAN 0
#define GB_VISC_CARREAU 1

#define GB_SOURCE_CONSTANT 0
#define GB_SOURCE_BOUSSINESQ 1

/* "Heat Source" of the energy equation (heat_source, src/mm_fill_energy.c:
 * 1724): none, CONSTANT h = c0, or the USER model (usr_heat_source,
 * src/user_mp.c:472) h = c0 exp(c1 T), the Frank-Kamenetskii / Bratu
 * source; R_T[i] += phi_i h dA, J_TT += phi_i dh/dT phi_j dA
 * (src/mm_fill_energy.c:374-381, :477-481). */
#define GB_HEAT_SOURCE_NONE 0
#define GB_HEAT_SOURCE_CONSTANT 1
#define GB_HEAT_SOURCE_EXPONENTIAL 2

/* Integrated (weak) boundary conditions on element sides, as
 * apply_integrated_bc adds them (src/mm_fill.c:2976, src/bc_integ.c):
 * R[row of node i] += sum_q w_q phi_i(q) sdet(q) func(q) over the side's
 * Gauss points (3 on a QUAD9 edge, 3 x 3 on a HEX27 face,
 * src/el_elm_info.c:1987), rows with a Dirichlet card left to that card:
 *   QSIDE          energy, func = q (value[0])                 (:1518)
 *   QCONV          energy, func = h (T_inf - T), dfunc/dT_j = -h phi_j
 *                  (h = value[0], T_inf = value[1]; qrad_surf without
 *                  radiation, src/mm_ns_bc.c:15145)
 *   FLOW_PRESSURE  momentum a, func = -P n_a (P = value[0]; flow_n_dot_T_hydro,
 *                  src/mm_ns_bc.c:6057), n the outward unit normal */
#define GB_IBC_QSIDE 1
#define GB_IBC_QCONV 2
#define GB_IBC_FLOW_PRESSURE 3

typedef struct gb_material {
  double density;          /* "Density = CONSTANT" */
  int viscosity_model;     /* GB_VISC_* ("Liquid Constitutive Equation") */
  double viscosity;        /* Newtonian "Viscosity = CONSTANT" */
  double mu0;              /* Carreau "Low Rate Viscosity" */
  double mu_inf;           /* Carreau "High Rate Viscosity" */
  double lambda;           /* Carreau "Time Constant" */
  double aexp;             /* Carreau "Aexp" */
  double nexp;             /* Carreau "Power Law Exponent" */
  double heat_capacity;    /* "Heat Capacity = CONSTANT" */
  double conductivity;     /* "Conductivity = CONSTANT" (Fourier heat flux) */
  int momentum_source_model;     /* GB_SOURCE_* ("Navier-Stokes Source") */
  double momentum_source[3];     /* constant force or gravity vector */
  double volume_expansion;       /* "Volume Expansion = CONSTANT" (beta) */
  double reference_temperature;  /* "Reference Temperature = CONSTANT" */
  /* species w < num_species of the problem */
  double diffusivity[GB_MAX_SPECIES];        /* "Diffusivity = CONSTANT w D" */
  int species_source_model[GB_MAX_SPECIES];  /* GB_SPECIES_SOURCE_* ("Species Source") */
  /* CONSTANT: [0] = S.  ARRHENIUS: k0, E, nu, s with S_w = nu k0 exp(-E/T) Y_s
   * (needs the energy equation, T > 0). */
  double species_source[GB_MAX_SPECIES][4];
  int heat_source_model;   /* GB_HEAT_SOURCE_* ("Heat Source") */
  double heat_source[2];   /* c0, c1 */
} gb_material;

typedef struct gb_problem_desc {
  int dim;        /* 2 (QUAD9) or 3 (HEX27) */
  int num_nodes;
  int num_elems;
  const double *coords; /* num_nodes * dim, interleaved (x, y[, z]) */
  const int *conn;      /* num_elems * (9 | 27), 0-based node ids */
  int energy;           /* 1: solve the energy equation (variable T) */
  int num_species;      /* "Number of bulk species" (dilute: one equation each) */
  gb_material mat;
  /* Dirichlet cards, applied in order (a later card wins on a shared
   * node): card c sets variable bc_var[c] to bc_value[c] on the nodes
   * bc_nodes[bc_ptr[c] .. bc_ptr[c+1]-1].  bc_var: GB_VAR_U1..U3, GB_VAR_T
   * or GB_VAR_Y(w); GB_VAR_P on element centroid nodes pins the element's
   * first pressure unknown, as PRESSURE DATUM does for one element
   * (several independent problems held in one description each need one). */
  int num_bc;
  const int *bc_var;
  const double *bc_value;
  const int *bc_ptr;
  const int *bc_nodes;
  /* PRESSURE DATUM: element (0-based) whose first pressure unknown is
   * pinned to pressure_datum_value; -1 for none. */
  int pressure_datum_elem;
  double pressure_datum_value;
  /* Integrated boundary conditions (GB_IBC_*): card c of type ibc_type[c]
   * with values ibc_value[2c], ibc_value[2c+1] on the sides ibc_ptr[c] ..
   * ibc_ptr[c+1]-1; side k is element ibc_elem[k] (0-based), Exodus side
   * ibc_side[k]: 1..4 on a QUAD9 (t = -1, s = +1, t = +1, s = -1), 1..6 on a
   * HEX27 (t = -1, s = +1, t = +1, s = -1, u = -1, u = +1).  num_ibc 0: none. */
  int num_ibc;
  const int *ibc_type;
  const double *ibc_value;
  const int *ibc_ptr;
  const int *ibc_elem;
  const int *ibc_side;
} gb_problem_desc;

#ifdef __cplusplus
}
#endif
#endif
