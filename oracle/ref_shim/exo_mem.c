/* In-memory Exodus II reader for the reference-as-oracle build (test
 * infrastructure).  The reference's rd_exo() (src/rd_exo.c:99) reads its
 * mesh through these calls; they serve the structured mesh named by the
 * environment variable GB_REF_MESH (see oracle/mesh_gen.h), whatever file
 * name the input deck gives.  Writer calls succeed and store nothing. */
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../mesh_gen.h"

#define EXM_NODE_SET 2
#define EXM_SIDE_SET 3
#define EXM_ELEM_BLOCK 1
#define EXM_GLOBAL 13
#define EXM_NODAL 14

int exerrval = 0;
static gb_mesh g_mesh;
static int g_loaded = 0;

static void load_mesh(void) {
  if (g_loaded) return;
  const char *spec = getenv("GB_REF_MESH");
  if (!spec || gb_mesh_build_from_spec(&g_mesh, spec) != 0) {
    fprintf(stderr, "exo_mem: GB_REF_MESH unset or invalid (\"%s\")\n", spec ? spec : "");
    abort();
  }
  g_loaded = 1;
}

int ex_open(const char *path, int mode, int *comp_ws, int *io_ws, float *version) {
  (void)path;
  (void)mode;
  load_mesh();
  if (comp_ws && *comp_ws == 0) *comp_ws = 8;
  if (io_ws) *io_ws = 8;
  if (version) *version = 8.0f;
  return 1;
}
int ex_create(const char *path, int mode, int *comp_ws, int *io_ws) {
  (void)path;
  (void)mode;
  (void)comp_ws;
  (void)io_ws;
  return 2;
}
int ex_close(int id) {
  (void)id;
  return 0;
}
int ex_opts(int o) {
  (void)o;
  return 0;
}
void ex_error(const char *a, const char *b, int c) {
  fprintf(stderr, "exo_mem: ex_error %s %s %d\n", a ? a : "", b ? b : "", c);
}

int ex_get_init(int id, char *title, int *num_dim, int *num_nodes, int *num_elem, int *num_blk,
                int *num_ns, int *num_ss) {
  (void)id;
  load_mesh();
  if (title) snprintf(title, 81, "structured %s mesh", g_mesh.dim == 2 ? "QUAD9" : "HEX27");
  *num_dim = g_mesh.dim;
  *num_nodes = g_mesh.num_nodes;
  *num_elem = g_mesh.num_elems;
  *num_blk = 1;
  *num_ns = g_mesh.num_sets;
  *num_ss = g_mesh.num_ssets;
  return 0;
}

int ex_inquire(int id, int req, int *ri, float *rf, char *rc) {
  (void)id;
  (void)rc;
  load_mesh();
  int v = 0;
  float f = 0.0f;
  switch (req) {
  case 2: /* API_VERS */
  case 3: /* DB_VERS */
    f = 8.0f;
    break;
  case 10: /* NS_NODE_LEN */
    for (int s = 0; s < g_mesh.num_sets; s++) v += g_mesh.set_len[s];
    break;
  case 11: /* SIDE_SETS */
    v = g_mesh.num_ssets;
    break;
  case 12: /* SS_NODE_LEN */
    for (int s = 0; s < g_mesh.num_ssets; s++)
      v += g_mesh.sset_len[s] * (g_mesh.dim == 2 ? 3 : 9);
    break;
  case 13: /* SS_ELEM_LEN */
    for (int s = 0; s < g_mesh.num_ssets; s++) v += g_mesh.sset_len[s];
    break;
  case 17: /* EB_PROP */
  case 18: /* NS_PROP */
  case 19: /* SS_PROP */
    v = 1;
    break;
  default:
    v = 0;
  }
  if (ri) *ri = v;
  if (rf) *rf = f;
  return 0;
}
int64_t ex_inquire_int(int id, int req) {
  int v = 0;
  float f;
  char c;
  ex_inquire(id, req, &v, &f, &c);
  return v;
}

int ex_get_qa(int id, void *qa) {
  (void)id;
  (void)qa;
  return 0;
}
int ex_get_info(int id, char **info) {
  (void)id;
  (void)info;
  return 0;
}
int ex_get_coord(int id, double *x, double *y, double *z) {
  (void)id;
  size_t n = (size_t)g_mesh.num_nodes * sizeof(double);
  if (x) memcpy(x, g_mesh.x, n);
  if (y) memcpy(y, g_mesh.y, n);
  if (z && g_mesh.dim == 3) memcpy(z, g_mesh.z, n);
  return 0;
}
int ex_get_coord_names(int id, char **names) {
  (void)id;
  static const char *nm[3] = {"x", "y", "z"};
  for (int i = 0; i < g_mesh.dim; i++) strcpy(names[i], nm[i]);
  return 0;
}
int ex_get_ids(int id, int type, int *ids) {
  (void)id;
  if (type == EXM_ELEM_BLOCK) {
    ids[0] = 1;
  } else if (type == EXM_NODE_SET) {
    for (int s = 0; s < g_mesh.num_sets; s++) ids[s] = s + 1;
  } else if (type == EXM_SIDE_SET) {
    for (int s = 0; s < g_mesh.num_ssets; s++) ids[s] = s + 1;
  }
  return 0;
}
int ex_get_block(int id, int type, int64_t blk, char *elem_type, int *num_entries,
                 int *nodes_per, int *edges_per, int *faces_per, int *num_attr) {
  (void)id;
  (void)type;
  (void)blk;
  if (elem_type) strcpy(elem_type, g_mesh.dim == 2 ? "QUAD9" : "HEX27");
  if (num_entries) *num_entries = g_mesh.num_elems;
  if (nodes_per) *nodes_per = g_mesh.nodes_per_elem;
  if (edges_per) *edges_per = 0;
  if (faces_per) *faces_per = 0;
  if (num_attr) *num_attr = 0;
  return 0;
}
int ex_get_conn(int id, int type, int64_t blk, int *conn, void *e, void *f) {
  (void)id;
  (void)type;
  (void)blk;
  (void)e;
  (void)f;
  size_t n = (size_t)g_mesh.num_elems * g_mesh.nodes_per_elem;
  for (size_t i = 0; i < n; i++) conn[i] = g_mesh.conn[i] + 1;
  return 0;
}
int ex_get_attr(int id, int type, int64_t blk, void *a) {
  (void)id;
  (void)type;
  (void)blk;
  (void)a;
  return 0;
}

typedef struct {
  int *sets_ids, *num_entries_per_set, *num_dist_per_set, *sets_entry_index, *sets_dist_index,
      *sets_entry_list, *sets_extra_list;
  void *sets_dist_fact;
} exm_set_specs;

int ex_get_concat_sets(int id, int type, exm_set_specs *sp) {
  (void)id;
  if (type == EXM_SIDE_SET) {
    int off = 0;
    for (int s = 0; s < g_mesh.num_ssets; s++) {
      sp->sets_ids[s] = s + 1;
      sp->num_entries_per_set[s] = g_mesh.sset_len[s];
      sp->num_dist_per_set[s] = 0;
      sp->sets_entry_index[s] = off;
      sp->sets_dist_index[s] = 0;
      for (int i = 0; i < g_mesh.sset_len[s]; i++) {
        sp->sets_entry_list[off + i] = g_mesh.sset_elem[s][i] + 1;
        if (sp->sets_extra_list) sp->sets_extra_list[off + i] = g_mesh.sset_side[s][i];
      }
      off += g_mesh.sset_len[s];
    }
    return 0;
  }
  if (type != EXM_NODE_SET) return 0;
  int off = 0;
  for (int s = 0; s < g_mesh.num_sets; s++) {
    sp->sets_ids[s] = s + 1;
    sp->num_entries_per_set[s] = g_mesh.set_len[s];
    sp->num_dist_per_set[s] = 0;
    sp->sets_entry_index[s] = off;
    sp->sets_dist_index[s] = 0;
    for (int i = 0; i < g_mesh.set_len[s]; i++) sp->sets_entry_list[off + i] = g_mesh.set_nodes[s][i] + 1;
    off += g_mesh.set_len[s];
  }
  return 0;
}
int ex_get_side_set_node_list_len(int id, int64_t ss, int *len) {
  (void)id;
  const int s = (int)ss - 1;
  *len = (s >= 0 && s < g_mesh.num_ssets) ? g_mesh.sset_len[s] * (g_mesh.dim == 2 ? 3 : 9) : 0;
  return 0;
}
/* per side its node count and the nodes (1-based), Exodus side order */
int ex_get_side_set_node_list(int id, int64_t ss, int *cnt, int *list) {
  (void)id;
  const int s = (int)ss - 1;
  if (s < 0 || s >= g_mesh.num_ssets) return 0;
  int off = 0, loc[9];
  for (int i = 0; i < g_mesh.sset_len[s]; i++) {
    const int e = g_mesh.sset_elem[s][i];
    const int n = gb_mesh_side_nodes(g_mesh.dim, g_mesh.sset_side[s][i], loc);
    cnt[i] = n;
    for (int k = 0; k < n; k++)
      list[off + k] = g_mesh.conn[(size_t)e * g_mesh.nodes_per_elem + loc[k]] + 1;
    off += n;
  }
  return 0;
}
int ex_get_prop_names(int id, int type, char **names) {
  (void)id;
  (void)type;
  strcpy(names[0], "ID");
  return 0;
}
int ex_get_prop_array(int id, int type, const char *name, int *vals) {
  (void)id;
  (void)name;
  if (type == EXM_ELEM_BLOCK) {
    vals[0] = 1;
  } else if (type == EXM_NODE_SET) {
    for (int s = 0; s < g_mesh.num_sets; s++) vals[s] = s + 1;
  } else if (type == EXM_SIDE_SET) {
    for (int s = 0; s < g_mesh.num_ssets; s++) vals[s] = s + 1;
  }
  return 0;
}
int ex_get_variable_param(int id, int type, int *n) {
  (void)id;
  (void)type;
  *n = 0;
  return 0;
}
int ex_get_var_param(int id, const char *t, int *n) {
  (void)id;
  (void)t;
  *n = 0;
  return 0;
}

/* Everything below is either never reached on the oracle's path (no
 * results are read back) or a writer whose output is not needed. */
#define EXM_NOOP(name)     \
  int name() { return 0; }
#define EXM_FAIL(name)                                                      \
  int name() {                                                              \
    fprintf(stderr, "exo_mem: %s is not served by the oracle shim\n", #name); \
    abort();                                                                \
    return -1;                                                              \
  }
EXM_FAIL(ex_get_variable_names)
EXM_FAIL(ex_get_all_times)
EXM_FAIL(ex_get_truth_table)
EXM_FAIL(ex_get_var)
EXM_FAIL(ex_get_time)
EXM_FAIL(ex_get_nodal_var)
EXM_FAIL(ex_get_elem_var)
EXM_FAIL(ex_get_map)
EXM_FAIL(ex_get_id_map)
EXM_FAIL(ex_get_init_info)
EXM_FAIL(ex_get_init_global)
EXM_FAIL(ex_get_cmap_params)
EXM_FAIL(ex_get_elem_cmap)
EXM_FAIL(ex_get_node_cmap)
EXM_FAIL(ex_get_loadbal_param)
EXM_FAIL(ex_get_processor_node_maps)
EXM_FAIL(ex_get_eb_info_global)
EXM_FAIL(ex_get_ns_param_global)
EXM_FAIL(ex_get_ss_param_global)
EXM_NOOP(ex_put_block)
EXM_NOOP(ex_put_blocks)
EXM_NOOP(ex_put_conn)
EXM_NOOP(ex_put_coord)
EXM_NOOP(ex_put_coord_names)
EXM_NOOP(ex_put_elem_block)
EXM_NOOP(ex_put_elem_num_map)
EXM_NOOP(ex_put_node_num_map)
EXM_NOOP(ex_put_id_map)
EXM_NOOP(ex_put_info)
EXM_NOOP(ex_put_init)
EXM_NOOP(ex_put_init_global)
EXM_NOOP(ex_put_init_info)
EXM_NOOP(ex_put_loadbal_param)
EXM_NOOP(ex_put_cmap_params)
EXM_NOOP(ex_put_node_cmap)
EXM_NOOP(ex_put_elem_cmap)
EXM_NOOP(ex_put_processor_node_maps)
EXM_NOOP(ex_put_eb_info_global)
EXM_NOOP(ex_put_ns_param_global)
EXM_NOOP(ex_put_ss_param_global)
EXM_NOOP(ex_put_prop_array)
EXM_NOOP(ex_put_prop_names)
EXM_NOOP(ex_put_qa)
EXM_NOOP(ex_put_set)
EXM_NOOP(ex_put_set_param)
EXM_NOOP(ex_put_concat_sets)
EXM_NOOP(ex_put_time)
EXM_NOOP(ex_put_times)
EXM_NOOP(ex_put_var)
EXM_NOOP(ex_put_variable_names)
EXM_NOOP(ex_put_variable_param)
EXM_NOOP(ex_put_truth_table)
EXM_NOOP(ex_put_elem_var_tab)
