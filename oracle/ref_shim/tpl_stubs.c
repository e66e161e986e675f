/* Third-party entry points the reference links against (NetCDF, LAPACK,
 * Trilinos wrappers, ghost-element and level-set helpers written in C++).
 * None is on the oracle's path: each aborts loudly if it is ever reached,
 * except fix_output(), which merges per-rank result files and has nothing
 * to do for a single rank, and the destructor of the (absent) matrix object. */
#include <stdio.h>
#include <stdlib.h>

#define GB_UNREACHED(name)                                                     \
  int name() {                                                                 \
    fprintf(stderr, "reference oracle: %s is outside the oracle path\n", #name); \
    abort();                                                                   \
    return -1;                                                                 \
  }
GB_UNREACHED(nc_open)
GB_UNREACHED(nc_close)
GB_UNREACHED(nc_inq_dimid)
GB_UNREACHED(nc_inq_dimlen)
GB_UNREACHED(nc_inq_varid)
GB_UNREACHED(nc_get_var)
GB_UNREACHED(nc_put_var)
GB_UNREACHED(nc_def_dim)
GB_UNREACHED(nc_def_var)
GB_UNREACHED(nc_enddef)
GB_UNREACHED(nc_redef)
GB_UNREACHED(nc_strerror)
GB_UNREACHED(dsyev_)
GB_UNREACHED(fix_exo_file)
GB_UNREACHED(GomaSparseMatrix_SetProblemGraph)
GB_UNREACHED(GomaSparseMatrix_CreateFromFormat)
GB_UNREACHED(GomaSparseMatrix_LoadLec)
GB_UNREACHED(amesos2_solve)
GB_UNREACHED(setup_ghost_to_base)
GB_UNREACHED(generate_ghost_elems)
GB_UNREACHED(fluidity_viscosity)
GB_UNREACHED(fluidity_source)
GB_UNREACHED(fluidity_equilibrium_surf)
GB_UNREACHED(facet_based_reinitialization)
GB_UNREACHED(find_current_distances)

void fix_output(void) {}

/* The MSR path owns no GomaSparseMatrix object; the reference's clean-up
 * still calls the destructor on the empty handle. */
int GomaSparseMatrix_Destroy(void *matrix) {
  (void)matrix;
  return 0;
}
