#!/bin/bash
# Builds the reference Goma C sources, unmodified, into oracle/_ref/goma_ref
# (test infrastructure: the checker that pins the CPU oracle, never shipped).
# The sources are compiled where they lie under the reference tree; the
# shims under oracle/ref_shim/ stand in for MPI (one rank), Exodus II (an
# in-memory structured mesh), NetCDF/LAPACK/Trilinos (unreached) and the
# Sparse 1.3 direct solver.  Outputs go only to oracle/_ref/.
#   usage: oracle/build_ref.sh [reference root; default $GOMA_REFERENCE,
#          else /root/reference]
set -euo pipefail
REF=${1:-${GOMA_REFERENCE:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT=$HERE/_ref
SHIM=$HERE/ref_shim
if [ ! -d "$REF/src" ]; then
  echo "build_ref: no reference tree at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT/obj"
DEFS="-DMDE=27 -DMAX_CONC=4 -DMAX_PROB_VAR=15 -DMAX_EXTERNAL_FIELD=4 -DMAX_NUMBER_MATLS=9 \
 -DCOMPILER_64BIT -DTRILINOS -DPARALLEL -DNO_CHEBYSHEV_PLEASE"
CFLAGS="-std=gnu11 -O2 -g -w -fcommon -fno-strict-aliasing $DEFS -I$SHIM/include -I$REF/include"
# every reference C file except the stand-alone fix tool and the Sparse-1.3
# wrapper (replaced by ref_shim/band_lu.c)
SRCS=$(ls "$REF"/src/*.c "$REF"/src/bc/*.c "$REF"/src/gds/*.c "$REF"/src/util/*.c |
  grep -v -e '/fix_main\.c$' -e '/sl_lu\.c$')
compile() {
  local f=$1 o
  o="$OUT/obj/$(basename "$f" .c).o"
  if [ ! -f "$o" ] || [ "$f" -nt "$o" ]; then
    gcc $CFLAGS -c "$f" -o "$o"
  fi
}
export -f compile
export CFLAGS OUT
printf '%s\n' $SRCS | xargs -P "$(nproc)" -I{} bash -c 'compile {}'
objcopy --redefine-sym main=goma_ref_main "$OUT/obj/main.o" "$OUT/obj/main_renamed.o"
SHIMC="-std=gnu11 -O2 -g -Wall -Wno-alloc-size-larger-than"
gcc $SHIMC -c "$SHIM/exo_mem.c" -o "$OUT/exo_mem.o"
gcc $SHIMC -c "$SHIM/mpi_serial.c" -o "$OUT/mpi_serial.o"
gcc $SHIMC -c "$SHIM/band_lu.c" -o "$OUT/band_lu.o"
gcc $SHIMC -c "$SHIM/tpl_stubs.c" -o "$OUT/tpl_stubs.o"
gcc $SHIMC -c "$HERE/mesh_gen.c" -o "$OUT/mesh_gen.o"
gcc $CFLAGS -c "$SHIM/harness.c" -o "$OUT/harness.o"
gcc $CFLAGS -c "$SHIM/user_species.c" -o "$OUT/user_species.o"
gcc $CFLAGS -c "$SHIM/user_heat.c" -o "$OUT/user_heat.o"
gcc $SHIMC -c "$SHIM/ref_main.c" -o "$OUT/ref_main.o"
OBJS=$(ls "$OUT"/obj/*.o | grep -v '/main\.o$')
gcc -o "$OUT/goma_ref" "$OUT/ref_main.o" $OBJS "$OUT"/exo_mem.o "$OUT"/mpi_serial.o \
  "$OUT"/band_lu.o "$OUT"/tpl_stubs.o "$OUT"/mesh_gen.o "$OUT"/harness.o "$OUT"/user_species.o \
  "$OUT"/user_heat.o -Wl,--wrap=matrix_fill_full -Wl,--wrap=numerical_jacobian \
  -Wl,--wrap=usr_species_source -Wl,--wrap=usr_heat_source -lm
echo "build_ref: built $OUT/goma_ref"
