"""The C ABI as a C caller sees it: every header under include/ compiles as
C99 with warnings as errors, a C program links libgbnewton.so and calls the
entry points that need no device -- the option defaults, the struct sizes
(which must equal the program's own sizeof), the plugin-table factory of
the "gb300" matrix format and its host-side graph checks -- the way the
reference's C code would."""
import os
import subprocess

import pytest

from goma_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "gb_problem.h"
#include "gb_newton.h"
#include "gb_sparse_matrix.h"

int main(void) {
  gb_newton_opts o;
  gb_newton_opts_default(&o);
  if (o.max_newton != 20 || o.krylov_dim != 30 || o.factorization_reuse != GB_FACTOR_CALC ||
      o.linear_precision != GB_LINEAR_FP64)
    return 1;
  if (gb_abi_struct_size(0) != (long long)sizeof(gb_newton_opts)) return 2;
  if (gb_abi_struct_size(1) != (long long)sizeof(gb_newton_stats)) return 3;
  if (gb_abi_struct_size(2) != (long long)sizeof(gb_problem_desc)) return 4;
  if (gb_abi_struct_size(3) != (long long)sizeof(gb_material)) return 5;
  gb_sparse_matrix_i32 m;
  memset(&m, 0, sizeof(m));
  if (gb_sparse_matrix_create_i32(&m) != 0 || m.type != GB_SPARSE_MATRIX_TYPE_GB300) return 6;
  if (!m.create_graph || !m.sum_into_row_values || !m.row_sum_scaling || !m.destroy) return 7;
  /* a graph entry outside the row list is refused before any device work */
  int rows[2] = {0, 1}, cr[2] = {0, 5}, cc[2] = {0, 1};
  if (m.create_graph(&m, 2, rows, 2, rows, 2, 1, cr, cc) != -1) return 8;
  if (strstr(gb_last_error(), "not in row_list") == NULL) return 9;
  if (m.put_scalar(&m, 0.0) != -1) return 10;
  gb_sparse_matrix_i64 m64;
  if (gb_sparse_matrix_create_i64(&m64) != 0 || m64.data != NULL) return 11;
  printf("ok\n");
  return 0;
}
"""


def test_headers_compile_as_c_and_the_abi_links(tmp_path):
    if not os.path.exists(_lib.LIB_PATH):
        pytest.skip("libgbnewton.so is not built")
    src = os.path.join(tmp_path, "abi.c")
    exe = os.path.join(tmp_path, "abi")
    with open(src, "w") as f:
        f.write(PROGRAM)
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                    "-I", os.path.join(ROOT, "include"), src, "-o", exe,
                    "-L", libdir, "-lgbnewton", "-Wl,-rpath," + libdir],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.returncode, r.stdout, r.stderr)
