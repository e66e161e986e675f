/* Empty Aztec surface for compiling the reference Goma sources into the CPU
 * oracle (test infrastructure).  The oracle replaces the Krylov solve. */
#ifndef GB_REF_SHIM_AZ_AZTEC_H
#define GB_REF_SHIM_AZ_AZTEC_H
#endif
