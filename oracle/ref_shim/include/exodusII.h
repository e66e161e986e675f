/* Minimal Exodus II API surface used only to compile the reference Goma
 * sources into the CPU oracle (test infrastructure).  The functions are
 * served from an in-memory structured mesh by oracle/ref_shim/exo_mem.c;
 * writers are accepted and discarded. */
#ifndef GB_REF_SHIM_EXODUSII_H
#define GB_REF_SHIM_EXODUSII_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
#define MAX_STR_LENGTH 32
#define MAX_LINE_LENGTH 80
#define MAX_ERR_LENGTH 256
#define EX_NOERR 0
#define EX_WARN 1
#define EX_FATAL (-1)
#define EX_READ 0x0000
#define EX_WRITE 0x0001
#define EX_CLOBBER 0x0004
#define EX_VERBOSE 1
#define EX_DEBUG 2
#define EX_ABORT 4
typedef enum ex_entity_type {
  EX_NODAL = 14,
  EX_NODE_BLOCK = 14,
  EX_NODE_SET = 2,
  EX_EDGE_BLOCK = 6,
  EX_EDGE_SET = 7,
  EX_FACE_BLOCK = 8,
  EX_FACE_SET = 9,
  EX_ELEM_BLOCK = 1,
  EX_ELEM_SET = 10,
  EX_SIDE_SET = 3,
  EX_ELEM_MAP = 4,
  EX_NODE_MAP = 5,
  EX_EDGE_MAP = 11,
  EX_FACE_MAP = 12,
  EX_GLOBAL = 13,
  EX_COORDINATE = 15,
  EX_INVALID = -1
} ex_entity_type;
typedef enum ex_inquiry {
  EX_INQ_FILE_TYPE = 1,
  EX_INQ_API_VERS = 2,
  EX_INQ_DB_VERS = 3,
  EX_INQ_TITLE = 4,
  EX_INQ_DIM = 5,
  EX_INQ_NODES = 6,
  EX_INQ_ELEM = 7,
  EX_INQ_ELEM_BLK = 8,
  EX_INQ_NODE_SETS = 9,
  EX_INQ_NS_NODE_LEN = 10,
  EX_INQ_SIDE_SETS = 11,
  EX_INQ_SS_NODE_LEN = 12,
  EX_INQ_SS_ELEM_LEN = 13,
  EX_INQ_QA = 14,
  EX_INQ_INFO = 15,
  EX_INQ_TIME = 16,
  EX_INQ_EB_PROP = 17,
  EX_INQ_NS_PROP = 18,
  EX_INQ_SS_PROP = 19,
  EX_INQ_NS_DF_LEN = 20,
  EX_INQ_SS_DF_LEN = 21
} ex_inquiry;
typedef int64_t ex_entity_id;
typedef void void_int;
typedef struct ex_set_specs {
  void_int *sets_ids;
  void_int *num_entries_per_set;
  void_int *num_dist_per_set;
  void_int *sets_entry_index;
  void_int *sets_dist_index;
  void_int *sets_entry_list;
  void_int *sets_extra_list;
  void *sets_dist_fact;
} ex_set_specs;
typedef struct ex_init_params {
  char title[MAX_LINE_LENGTH + 1];
  int64_t num_dim, num_nodes, num_edge, num_edge_blk, num_face, num_face_blk, num_elem,
      num_elem_blk, num_node_sets, num_edge_sets, num_face_sets, num_side_sets, num_elem_sets,
      num_node_maps, num_edge_maps, num_face_maps, num_elem_maps;
} ex_init_params;
extern int exerrval;
/* Unprototyped on purpose: the reference calls these with a mix of the
 * old and new Exodus signatures; exo_mem.c implements the forms it uses. */
int ex_open();
int ex_create();
int ex_close();
int ex_opts();
void ex_error();
int ex_inquire();
int64_t ex_inquire_int();
int ex_get_init();
int ex_get_init_info();
int ex_get_init_global();
int ex_get_qa();
int ex_get_info();
int ex_get_coord();
int ex_get_coord_names();
int ex_get_ids();
int ex_get_block();
int ex_get_conn();
int ex_get_elem_conn();
int ex_get_attr();
int ex_get_concat_sets();
int ex_get_concat_node_sets();
int ex_get_concat_side_sets();
int ex_get_side_set_node_list();
int ex_get_side_set_node_list_len();
int ex_get_prop_names();
int ex_get_prop_array();
int ex_get_map();
int ex_get_id_map();
int ex_get_elem_num_map();
int ex_get_node_num_map();
int ex_get_all_times();
int ex_get_time();
int ex_get_var();
int ex_get_nodal_var();
int ex_get_elem_var();
int ex_get_glob_vars();
int ex_get_var_param();
int ex_get_variable_param();
int ex_get_variable_names();
int ex_get_truth_table();
int ex_get_cmap_params();
int ex_get_elem_cmap();
int ex_get_node_cmap();
int ex_get_loadbal_param();
int ex_get_processor_node_maps();
int ex_get_eb_info_global();
int ex_get_ns_param_global();
int ex_get_ss_param_global();
int ex_put_block();
int ex_put_blocks();
int ex_put_conn();
int ex_put_coord();
int ex_put_coord_names();
int ex_put_elem_block();
int ex_put_elem_num_map();
int ex_put_node_num_map();
int ex_put_id_map();
int ex_put_info();
int ex_put_init();
int ex_put_init_global();
int ex_put_init_info();
int ex_put_loadbal_param();
int ex_put_cmap_params();
int ex_put_node_cmap();
int ex_put_elem_cmap();
int ex_put_processor_node_maps();
int ex_put_eb_info_global();
int ex_put_ns_param_global();
int ex_put_ss_param_global();
int ex_put_prop_array();
int ex_put_prop_names();
int ex_put_qa();
int ex_put_set();
int ex_put_set_param();
int ex_put_concat_sets();
int ex_put_time();
int ex_put_times();
int ex_put_var();
int ex_put_variable_names();
int ex_put_variable_param();
int ex_put_truth_table();
int ex_put_elem_var_tab();
#ifdef __cplusplus
}
#endif
#endif
