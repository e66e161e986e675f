/* Exponential heat source for the reference-as-oracle build (test
 * infrastructure).
 *
 * The reference's user routine usr_heat_source (src/user_mp.c:472) is a
 * template that stops with "No user_defined heat source model implemented"
 * (:491); a deck that names "Heat Source = USER" must supply the body.  The
 * recipe links with -Wl,--wrap=usr_heat_source, so the call in heat_source
 * (src/mm_fill_energy.c:1766) lands here.  Parameters of the card
 * "Heat Source = USER c0 c1":
 *     h = c0 exp(c1 T)   (the Frank-Kamenetskii / Bratu source)
 * with dh/dT stored where the template stores it
 * (mp->d_heat_source[TEMPERATURE]); every other sensitivity is zero. */
#include <math.h>

#include "std.h"
#include "el_elm.h"
#include "mm_as.h"
#include "mm_as_structs.h"
#include "mm_mp.h"
#include "mm_mp_structs.h"
#include "rf_fem_const.h"

int __wrap_usr_heat_source(dbl *param, dbl time) {
  (void)time;
  const double h = param[0] * exp(param[1] * fv->T);
  int a;
  mp->heat_source = h;
  mp->d_heat_source[TEMPERATURE] = param[1] * h;
  mp->d_heat_source[VOLTAGE] = 0.0;
  for (a = 0; a < DIM; a++) {
    mp->d_heat_source[VELOCITY1 + a] = 0.0;
    mp->d_heat_source[MESH_DISPLACEMENT1 + a] = 0.0;
  }
  for (a = 0; a < MAX_CONC; a++) mp->d_heat_source[MAX_VARIABLE_TYPES + a] = 0.0;
  return 0;
}
