/* Structured QUAD9 / HEX27 box mesh generator for the CPU oracle.  See
 * mesh_gen.h for the numbering conventions. */
#include "mesh_gen.h"

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* grid offsets (0..2) of the QUAD9 local nodes, Goma order */
const int gb_quad9_local[9][2] = {{0, 0}, {2, 0}, {2, 2}, {0, 2}, {1, 0},
                                  {2, 1}, {1, 2}, {0, 1}, {1, 1}};
/* grid offsets (0..2) of the HEX27 local nodes, Goma order */
const int gb_hex27_local[27][3] = {
    {0, 0, 0}, {2, 0, 0}, {2, 2, 0}, {0, 2, 0}, {0, 0, 2}, {2, 0, 2}, {2, 2, 2},
    {0, 2, 2}, {1, 0, 0}, {2, 1, 0}, {1, 2, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 1},
    {2, 2, 1}, {0, 2, 1}, {1, 0, 2}, {2, 1, 2}, {1, 2, 2}, {0, 1, 2}, {1, 1, 1},
    {1, 1, 0}, {1, 1, 2}, {0, 1, 1}, {2, 1, 1}, {1, 0, 1}, {1, 2, 1}};

static int add_set(gb_mesh *m, int s, int *tmp, int n) {
  m->set_nodes[s] = (int *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int));
  if (!m->set_nodes[s]) return -1;
  memcpy(m->set_nodes[s], tmp, (size_t)n * sizeof(int));
  m->set_len[s] = n;
  return 0;
}

/* splitmix64 finaliser: a fixed integer hash, so the perturbation is the
 * same on every machine and in every implementation of the generator */
static uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

double gb_mesh_jitter(uint64_t seed, uint64_t node, int axis) {
  uint64_t h = mix64(seed * 0x100000001B3ull + node * 3ull + (uint64_t)axis);
  return (double)(h >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
}

int gb_mesh_build(gb_mesh *m, int dim, int nx, int ny, int nz, double lx, double ly, double lz) {
  return gb_mesh_build_perturbed(m, dim, nx, ny, nz, lx, ly, lz, 0.0, 0);
}

int gb_mesh_build_perturbed(gb_mesh *m, int dim, int nx, int ny, int nz, double lx, double ly,
                            double lz, double amp, uint64_t seed) {
  memset(m, 0, sizeof(*m));
  if (dim != 2 && dim != 3) return -1;
  if (nx < 1 || ny < 1 || (dim == 3 && nz < 1)) return -1;
  if (dim == 2) {
    nz = 1;
    lz = 0.0;
  }
  m->dim = dim;
  m->nx = nx;
  m->ny = ny;
  m->nz = nz;
  m->lx = lx;
  m->ly = ly;
  m->lz = lz;
  const int NX = 2 * nx + 1, NY = 2 * ny + 1, NZ = dim == 3 ? 2 * nz + 1 : 1;
  m->num_nodes = NX * NY * NZ;
  m->num_elems = nx * ny * (dim == 3 ? nz : 1);
  m->nodes_per_elem = dim == 3 ? 27 : 9;
  m->x = (double *)malloc((size_t)m->num_nodes * sizeof(double));
  m->y = (double *)malloc((size_t)m->num_nodes * sizeof(double));
  m->z = dim == 3 ? (double *)malloc((size_t)m->num_nodes * sizeof(double)) : NULL;
  m->conn = (int *)malloc((size_t)m->num_elems * m->nodes_per_elem * sizeof(int));
  if (!m->x || !m->y || (dim == 3 && !m->z) || !m->conn) return -1;
  for (int k = 0; k < NZ; k++)
    for (int j = 0; j < NY; j++)
      for (int i = 0; i < NX; i++) {
        int n = i + NX * (j + NY * k);
        m->x[n] = lx * (double)i / (double)(NX - 1);
        m->y[n] = ly * (double)j / (double)(NY - 1);
        if (dim == 3) m->z[n] = lz * (double)k / (double)(NZ - 1);
        int interior = i > 0 && i < NX - 1 && j > 0 && j < NY - 1 &&
                       (dim == 2 || (k > 0 && k < NZ - 1));
        if (amp != 0.0 && interior) {
          m->x[n] += amp * (lx / (double)(NX - 1)) * gb_mesh_jitter(seed, (uint64_t)n, 0);
          m->y[n] += amp * (ly / (double)(NY - 1)) * gb_mesh_jitter(seed, (uint64_t)n, 1);
          if (dim == 3)
            m->z[n] += amp * (lz / (double)(NZ - 1)) * gb_mesh_jitter(seed, (uint64_t)n, 2);
        }
      }
  if (dim == 2) {
    for (int ey = 0; ey < ny; ey++)
      for (int ex = 0; ex < nx; ex++) {
        int e = ex + nx * ey;
        for (int l = 0; l < 9; l++) {
          int i = 2 * ex + gb_quad9_local[l][0], j = 2 * ey + gb_quad9_local[l][1];
          m->conn[e * 9 + l] = i + NX * j;
        }
      }
  } else {
    for (int ez = 0; ez < nz; ez++)
      for (int ey = 0; ey < ny; ey++)
        for (int ex = 0; ex < nx; ex++) {
          int e = ex + nx * (ey + ny * ez);
          for (int l = 0; l < 27; l++) {
            int i = 2 * ex + gb_hex27_local[l][0], j = 2 * ey + gb_hex27_local[l][1],
                k = 2 * ez + gb_hex27_local[l][2];
            m->conn[e * 27 + l] = i + NX * (j + NY * k);
          }
        }
  }
  int *tmp = (int *)malloc((size_t)m->num_nodes * sizeof(int));
  if (!tmp) return -1;
  if (dim == 2) {
    m->num_sets = 6;
    for (int s = 0; s < 6; s++) {
      int n = 0;
      for (int j = 0; j < NY; j++)
        for (int i = 0; i < NX; i++) {
          int on = 0;
          switch (s) {
          case 0: on = (j == 0); break;
          case 1: on = (i == NX - 1); break;
          case 2: on = (j == NY - 1); break;
          case 3: on = (i == 0); break;
          case 4: on = (i == 0) && (2 * j <= NY - 1); break;
          case 5: on = (i == 0) && (2 * j >= NY - 1); break;
          }
          if (on) tmp[n++] = i + NX * j;
        }
      if (add_set(m, s, tmp, n)) return -1;
    }
  } else {
    m->num_sets = 6;
    for (int s = 0; s < 6; s++) {
      int n = 0;
      for (int k = 0; k < NZ; k++)
        for (int j = 0; j < NY; j++)
          for (int i = 0; i < NX; i++) {
            int on = 0;
            switch (s) {
            case 0: on = (i == 0); break;
            case 1: on = (i == NX - 1); break;
            case 2: on = (j == 0); break;
            case 3: on = (j == NY - 1); break;
            case 4: on = (k == 0); break;
            case 5: on = (k == NZ - 1); break;
            }
            if (on) tmp[n++] = i + NX * (j + NY * k);
          }
      if (add_set(m, s, tmp, n)) return -1;
    }
  }
  free(tmp);
  /* side sets */
  {
    const int ne = m->num_elems;
    int *te = (int *)malloc((size_t)ne * sizeof(int));
    if (!te) return -1;
    /* (selector, side): 2-D y=0, x=Lx, y=Ly, x=0; 3-D x=0, x=Lx, y=0, y=Ly, z=0, z=Lz */
    static const int side2[4] = {1, 2, 3, 4};
    static const int side3[6] = {4, 2, 1, 3, 5, 6};
    m->num_ssets = dim == 2 ? 4 : 6;
    for (int s = 0; s < m->num_ssets; s++) {
      int n = 0;
      for (int e = 0; e < ne; e++) {
        const int ex = e % nx, ey = (e / nx) % ny, ez = e / (nx * ny);
        int on = 0;
        if (dim == 2) {
          switch (s) {
          case 0: on = ey == 0; break;
          case 1: on = ex == nx - 1; break;
          case 2: on = ey == ny - 1; break;
          case 3: on = ex == 0; break;
          }
        } else {
          switch (s) {
          case 0: on = ex == 0; break;
          case 1: on = ex == nx - 1; break;
          case 2: on = ey == 0; break;
          case 3: on = ey == ny - 1; break;
          case 4: on = ez == 0; break;
          case 5: on = ez == nz - 1; break;
          }
        }
        if (on) te[n++] = e;
      }
      m->sset_len[s] = n;
      m->sset_elem[s] = (int *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int));
      m->sset_side[s] = (int *)malloc((size_t)(n > 0 ? n : 1) * sizeof(int));
      if (!m->sset_elem[s] || !m->sset_side[s]) return -1;
      for (int k = 0; k < n; k++) {
        m->sset_elem[s][k] = te[k];
        m->sset_side[s][k] = dim == 2 ? side2[s] : side3[s];
      }
    }
    free(te);
  }
  return 0;
}

int gb_mesh_side_nodes(int dim, int side, int *local) {
  /* Exodus side node orders, 1-based element node numbers */
  static const int q9[4][3] = {{1, 2, 5}, {2, 3, 6}, {3, 4, 7}, {4, 1, 8}};
  static const int h27[6][9] = {{1, 2, 6, 5, 9, 14, 17, 13, 26},
                                {2, 3, 7, 6, 10, 15, 18, 14, 25},
                                {3, 4, 8, 7, 11, 16, 19, 15, 27},
                                {1, 5, 8, 4, 13, 20, 16, 12, 24},
                                {1, 4, 3, 2, 12, 11, 10, 9, 22},
                                {5, 6, 7, 8, 17, 18, 19, 20, 23}};
  if (dim == 2) {
    if (side < 1 || side > 4) return 0;
    for (int k = 0; k < 3; k++) local[k] = q9[side - 1][k] - 1;
    return 3;
  }
  if (side < 1 || side > 6) return 0;
  for (int k = 0; k < 9; k++) local[k] = h27[side - 1][k] - 1;
  return 9;
}

int gb_mesh_build_from_spec(gb_mesh *m, const char *spec) {
  char kind[16];
  int nx = 0, ny = 0, nz = 0;
  double lx = 1, ly = 1, lz = 1, amp = 0.0;
  unsigned long long seed = 0;
  int got;
  if (!spec || sscanf(spec, "%15s", kind) != 1) return -1;
  if (strcmp(kind, "quad9") == 0) {
    got = sscanf(spec, "%15s %d %d %lf %lf %lf %llu", kind, &nx, &ny, &lx, &ly, &amp, &seed);
    if (got != 5 && got != 7) return -1;
    return gb_mesh_build_perturbed(m, 2, nx, ny, 1, lx, ly, 0.0, amp, (uint64_t)seed);
  }
  if (strcmp(kind, "hex27") == 0) {
    got = sscanf(spec, "%15s %d %d %d %lf %lf %lf %lf %llu", kind, &nx, &ny, &nz, &lx, &ly, &lz,
                 &amp, &seed);
    if (got != 7 && got != 9) return -1;
    return gb_mesh_build_perturbed(m, 3, nx, ny, nz, lx, ly, lz, amp, (uint64_t)seed);
  }
  return -1;
}

void gb_mesh_free(gb_mesh *m) {
  free(m->x);
  free(m->y);
  free(m->z);
  free(m->conn);
  for (int s = 0; s < m->num_sets; s++) free(m->set_nodes[s]);
  for (int s = 0; s < m->num_ssets; s++) {
    free(m->sset_elem[s]);
    free(m->sset_side[s]);
  }
  memset(m, 0, sizeof(*m));
}
