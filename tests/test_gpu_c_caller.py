"""The device entry points called from C, the way the reference's own C
code would call its replacements: a C99 program fills a gb_problem_desc
from plain arrays (a lid-driven cavity read from a file the test writes),
creates the context, sets the Dirichlet values (gb_dirichlet_init, for
find_and_set_Dirichlet), assembles the residual and the MSR Jacobian at a
given state (gb_matrix_fill_full, for matrix_fill_full) and runs the Newton
loop (gb_solve_nonlinear_problem, for solve_nonlinear_problem).  Its
outputs must equal the oracle's: the assembly within 1e-12 (row-scaled),
the converged solution within 1e-8."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from goma_gb300 import _lib
from goma_gb300 import problem as pb
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "gb_problem.h"
#include "gb_newton.h"

static void *slurp(FILE *f, size_t n) {
  void *p = malloc(n ? n : 1);
  if (!p || fread(p, 1, n, f) != n) { fprintf(stderr, "short read\n"); exit(20); }
  return p;
}

int main(int argc, char **argv) {
  if (argc != 3) return 1;
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 2;
  int hdr[7];   /* dim, nodes, elements, nodes per element, cards, card nodes, datum element */
  double mat[2], datum;  /* density, viscosity; datum value */
  if (fread(hdr, sizeof(int), 7, f) != 7 || fread(mat, sizeof(double), 2, f) != 2 ||
      fread(&datum, sizeof(double), 1, f) != 1) return 3;
  const int dim = hdr[0], nn = hdr[1], ne = hdr[2], npe = hdr[3], nbc = hdr[4], nbn = hdr[5];
  double *coords = slurp(f, sizeof(double) * (size_t)nn * dim);
  int *conn = slurp(f, sizeof(int) * (size_t)ne * npe);
  int *bc_var = slurp(f, sizeof(int) * nbc);
  double *bc_value = slurp(f, sizeof(double) * nbc);
  int *bc_ptr = slurp(f, sizeof(int) * (nbc + 1));
  int *bc_nodes = slurp(f, sizeof(int) * nbn);
  int N = 0;
  if (fread(&N, sizeof(int), 1, f) != 1) return 4;
  double *x_state = slurp(f, sizeof(double) * N);
  fclose(f);

  gb_problem_desc d;
  memset(&d, 0, sizeof(d));
  d.dim = dim;
  d.num_nodes = nn;
  d.num_elems = ne;
  d.coords = coords;
  d.conn = conn;
  d.mat.density = mat[0];
  d.mat.viscosity_model = GB_VISC_NEWTONIAN;
  d.mat.viscosity = mat[1];
  d.mat.momentum_source_model = GB_SOURCE_CONSTANT;
  d.num_bc = nbc;
  d.bc_var = bc_var;
  d.bc_value = bc_value;
  d.bc_ptr = bc_ptr;
  d.bc_nodes = bc_nodes;
  d.pressure_datum_elem = hdr[6];
  d.pressure_datum_value = datum;

  gb_ctx *ctx = NULL;
  if (gb_create(&d, &ctx) != 0) { fprintf(stderr, "%s\n", gb_last_error()); return 5; }
  if (gb_num_unknowns(ctx) != N) return 6;
  const long long L = gb_msr_length(ctx);
  double *R = calloc((size_t)N, sizeof(double));
  double *a = calloc((size_t)L, sizeof(double));
  int *ija = calloc((size_t)L, sizeof(int));
  if (gb_msr_pattern(ctx, ija) != 0) return 7;
  if (gb_matrix_fill_full(ctx, x_state, R, a) != 0) {
    fprintf(stderr, "%s\n", gb_last_error());
    return 8;
  }
  double *x = calloc((size_t)N, sizeof(double));
  if (gb_dirichlet_init(ctx, x) != 0) return 9;
  gb_newton_opts o;
  gb_newton_opts_default(&o);
  o.residual_tol = 1e-11;
  o.linear_tol = 1e-10;
  o.max_newton = 30;
  o.krylov_dim = 60;
  o.max_linear_its = 2000;
  int converged = 0;
  gb_newton_stats st;
  if (gb_solve_nonlinear_problem(ctx, x, &o, &converged, &st) != 0) {
    fprintf(stderr, "%s\n", gb_last_error());
    return 10;
  }
  FILE *g = fopen(argv[2], "wb");
  if (!g) return 11;
  const int out_hdr[3] = {N, (int)L, converged};
  fwrite(out_hdr, sizeof(int), 3, g);
  fwrite(&st.newton_its, sizeof(int), 1, g);
  fwrite(R, sizeof(double), (size_t)N, g);
  fwrite(a, sizeof(double), (size_t)L, g);
  fwrite(ija, sizeof(int), (size_t)L, g);
  fwrite(x, sizeof(double), (size_t)N, g);
  fclose(g);
  gb_destroy(ctx);
  printf("ok\n");
  return 0;
}
"""


def _write_case(path, prob, x_state):
    m = prob.mesh
    bcs = prob.bcs
    lists = [np.asarray(m.node_sets[b[1] - 1], np.int32) for b in bcs]
    bc_ptr = np.concatenate([[0], np.cumsum([len(l) for l in lists])]).astype(np.int32)
    with open(path, "wb") as f:
        np.array([m.dim, m.num_nodes, m.num_elems, np.asarray(m.conn).shape[1], len(bcs),
                  int(bc_ptr[-1]), prob.pressure_datum[0]], np.int32).tofile(f)
        np.array([prob.material.density, prob.material.viscosity, prob.pressure_datum[1]],
                 np.float64).tofile(f)
        np.ascontiguousarray(m.coords, np.float64).tofile(f)
        np.ascontiguousarray(m.conn, np.int32).tofile(f)
        np.array([b[0] for b in bcs], np.int32).tofile(f)
        np.array([b[2] for b in bcs], np.float64).tofile(f)
        bc_ptr.tofile(f)
        np.concatenate(lists).astype(np.int32).tofile(f)
        np.array([len(x_state)], np.int32).tofile(f)
        np.asarray(x_state, np.float64).tofile(f)


def test_c_program_assembles_and_solves_through_the_abi(tmp_path):
    prob = pb.lid_cavity_2d(6, 100.0, mesh=pb.box_mesh(2, 6, 6, amp=0.1, seed=3))
    o = oracle.Oracle(prob)
    x_state = o.dirichlet_init(np.random.default_rng(5).uniform(-1, 1, o.N))
    case = os.path.join(tmp_path, "case.bin")
    out = os.path.join(tmp_path, "out.bin")
    _write_case(case, prob, x_state)
    src = os.path.join(tmp_path, "caller.c")
    exe = os.path.join(tmp_path, "caller")
    with open(src, "w") as f:
        f.write(PROGRAM)
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-O1",
                    "-I", os.path.join(ROOT, "include"), src, "-o", exe,
                    "-L", libdir, "-lgbnewton", "-Wl,-rpath," + libdir],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([exe, case, out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.returncode, r.stdout, r.stderr)
    with open(out, "rb") as f:
        N, L, conv, its = np.fromfile(f, np.int32, 4)
        R = np.fromfile(f, np.float64, N)
        a = np.fromfile(f, np.float64, L)
        ija = np.fromfile(f, np.int32, L)
        x = np.fromfile(f, np.float64, N)
    assert N == o.N
    assert np.array_equal(ija, o.ija())
    Ro, ao, st = o.matrix_fill(x_state)
    assert st == 0
    assert np.abs(R - Ro).max() <= 1e-12 * np.abs(Ro).max()
    assert gc.msr_row_scaled_error(ija, a, ao) <= 1e-12
    assert conv == 1 and its > 0
    xo, ito, _ = o.newton(o.dirichlet_init(np.zeros(o.N)), 30, 1e-11)
    assert ito > 0
    assert np.abs(x - xo).max() <= 1e-8 * np.abs(xo).max()
