/* Structured QUAD9 / HEX27 box meshes for the CPU oracle (test
 * infrastructure only; the product has its own generator and a test checks
 * the two agree node for node).
 *
 * Node numbering is lexicographic over the (2nx+1) x (2ny+1) [x (2nz+1)]
 * grid of vertex + mid-edge + mid-face + centre nodes, x fastest.  Elements
 * are numbered x fastest as well.  Local node order inside an element is the
 * Exodus / Goma order used by the reference shape functions
 * (src/rf_shape.c:361 BIQUAD_QUAD, src/rf_shape.c:1105 TRIQUAD_HEX):
 *   QUAD9: 4 corners counter-clockwise from (-1,-1), 4 mid-edges starting at
 *          (0,-1), centre.
 *   HEX27: 8 corners (bottom face ccw, then top face), 12 mid-edges (bottom,
 *          vertical, top), centre (node 20), then the face centres
 *          -z, +z, -x, +x, -y, +y (nodes 21..26).
 *
 * Node sets (ids are 1-based as in Exodus):
 *   2-D: 1 y=0, 2 x=Lx, 3 y=Ly, 4 x=0, 5 x=0 & y<=Ly/2, 6 x=0 & y>=Ly/2
 *   3-D: 1 x=0, 2 x=Lx, 3 y=0, 4 y=Ly, 5 z=0, 6 z=Lz
 */
#ifndef GB_ORACLE_MESH_GEN_H
#define GB_ORACLE_MESH_GEN_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GB_MESH_MAX_SETS 6

typedef struct gb_mesh {
  int dim;            /* 2 or 3 */
  int nx, ny, nz;     /* elements per direction (nz = 1 in 2-D for convenience) */
  double lx, ly, lz;  /* box extents */
  int num_nodes;
  int num_elems;
  int nodes_per_elem; /* 9 or 27 */
  double *x, *y, *z;  /* coordinates, z NULL in 2-D */
  int *conn;          /* num_elems * nodes_per_elem, 0-based node ids */
  int num_sets;
  int set_len[GB_MESH_MAX_SETS];
  int *set_nodes[GB_MESH_MAX_SETS]; /* ascending 0-based node ids */
  /* side sets on the boundaries of node sets 1..4 (2-D) / 1..6 (3-D):
   * 0-based elements and Exodus side numbers (QUAD9 1 t=-1, 2 s=+1,
   * 3 t=+1, 4 s=-1; HEX27 the same and 5 u=-1, 6 u=+1) */
  int num_ssets;
  int sset_len[GB_MESH_MAX_SETS];
  int *sset_elem[GB_MESH_MAX_SETS];
  int *sset_side[GB_MESH_MAX_SETS];
} gb_mesh;

/* Local nodes (0-based, Goma order) of Exodus side `side` (1-based) of a
 * QUAD9 (3 nodes: corners then mid-edge) or HEX27 (9: corners, mid-edges,
 * face centre); returns the count. */
int gb_mesh_side_nodes(int dim, int side, int *local);

/* Reference-coordinate offsets (-1,0,1 mapped to grid steps 0,1,2) of each
 * local node. */
extern const int gb_quad9_local[9][2];
extern const int gb_hex27_local[27][3];

int gb_mesh_build(gb_mesh *m, int dim, int nx, int ny, int nz, double lx, double ly, double lz);
/* Same grid with every strictly interior node moved by amp * (node spacing)
 * * U(-1,1) per axis, U drawn from a fixed integer hash of (seed, node,
 * axis); amp <= 0.2 keeps every element valid. */
int gb_mesh_build_perturbed(gb_mesh *m, int dim, int nx, int ny, int nz, double lx, double ly,
                            double lz, double amp, uint64_t seed);
double gb_mesh_jitter(uint64_t seed, uint64_t node, int axis);
/* Parse "quad9 NX NY LX LY [AMP SEED]" or "hex27 NX NY NZ LX LY LZ [AMP SEED]". */
int gb_mesh_build_from_spec(gb_mesh *m, const char *spec);
void gb_mesh_free(gb_mesh *m);

#ifdef __cplusplus
}
#endif
#endif
