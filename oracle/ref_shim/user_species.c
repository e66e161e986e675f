/* Arrhenius species source for the reference-as-oracle build (test
 * infrastructure).
 *
 * The reference's user routine usr_species_source (src/user_mp.c:598) is a
 * template that stops with "No user_defined species source model
 * implemented" (:618); a deck that names "Species Source = USER" must supply
 * the body.  The recipe links with -Wl,--wrap=usr_species_source, so the
 * call in get_continuous_species_terms (src/mm_fill_species.c:10146) lands
 * here.  Parameters of the card "Species Source = USER w k0 E nu s":
 *     S_w = nu * k0 * exp(-E / T) * Y_s
 * with its sensitivities to T and Y_s, stored where the template stores
 * them (mp->species_source[w], mp->d_species_source[TEMPERATURE] and
 * [MAX_VARIABLE_TYPES + s]); every other sensitivity is zero. */
#include <math.h>

#include "std.h"
#include "el_elm.h"
#include "mm_as.h"
#include "mm_as_structs.h"
#include "mm_mp.h"
#include "mm_mp_structs.h"
#include "rf_fem_const.h"

int __wrap_usr_species_source(int w, dbl *param) {
  const double k0 = param[0], E = param[1], nu = param[2];
  const int s = (int)param[3];
  const double T = fv->T, Y = fv->c[s];
  const double r = k0 * exp(-E / T);
  int a;
  mp->species_source[w] = nu * r * Y;
  mp->d_species_source[TEMPERATURE] = nu * r * Y * E / (T * T);
  mp->d_species_source[VOLTAGE] = 0.0;
  for (a = 0; a < DIM; a++) {
    mp->d_species_source[VELOCITY1 + a] = 0.0;
    mp->d_species_source[MESH_DISPLACEMENT1 + a] = 0.0;
  }
  for (a = 0; a < MAX_CONC; a++) mp->d_species_source[MAX_VARIABLE_TYPES + a] = 0.0;
  mp->d_species_source[MAX_VARIABLE_TYPES + s] = nu * r;
  return 0;
}
