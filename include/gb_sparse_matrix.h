/* GB300 backend of the reference's sparse-matrix plugin interface, part of
 * libgbnewton.so.
 *
 * The reference reaches its Epetra / Tpetra matrices through a table of
 * function pointers, struct g_GomaSparseMatrix
 * (include/linalg/sparse_matrix.h:35-88), filled by
 * GomaSparseMatrix_CreateFromFormat (src/linalg/sparse_matrix.cpp:31-40)
 * and used by GomaSparseMatrix_SetProblemGraph (create_graph, :242),
 * GomaSparseMatrix_LoadLec (sum_into_row_values, :361, :454), the Newton
 * loop (put_scalar, src/mm_sol_nonlinear.c:1114; matrix_vector_mult, :448),
 * row_sum_scaling_scale (row_sum_scaling, src/sl_matrix_util.c:447-449) and
 * the level-set code (zero_global_row_set_diag, src/mm_fill_ls.c:10778).
 * The structs below have that table's layout for the two GomaGlobalOrdinal
 * builds (int, and long long under GOMA_MATRIX_GO_LONG_LONG,
 * include/linalg/sparse_matrix.h:7-13), so a "gb300" matrix format is one
 * more case in GomaSparseMatrix_CreateFromFormat that calls
 * gb_sparse_matrix_create_i32 (or _i64) on the table the reference has
 * just allocated.
 *
 * Storage: CSR in device memory (64-bit row pointers, 32-bit local column
 * indices ascending in every row, FP64 values), with a pinned host copy of
 * the values.  The per-row calls (insert_row_values, sum_into_row_values,
 * zero_global_row*) edit the host copy; put_scalar sets both copies;
 * row_sum_scaling and matrix_vector_mult run on the GPU after uploading
 * pending host edits once.  Semantics follow the Tpetra backend
 * (src/linalg/sparse_matrix_tpetra.cpp): row_sum_scaling divides each row
 * and b by the sum of the row's absolute values (1 for an all-zero row) and
 * returns that sum in scale; insert_row_values replaces existing values and
 * sum_into_row_values adds to them; a column outside the graph is an error.
 * One rank: the rows are the local rows in row_list order and every column
 * id must be in col_list.
 *
 * Every function returns 0 (GOMA_SUCCESS) or -1 (GOMA_ERROR) with a message
 * for gb_last_error() (gb_newton.h).
 */
#ifndef GB_SPARSE_MATRIX_H
#define GB_SPARSE_MATRIX_H

#ifdef __cplusplus
extern "C" {
#endif

/* The value a "gb300" matrix puts in the table's type field: the next
 * enumerator after GOMA_SPARSE_MATRIX_TYPE_PETSC
 * (include/linalg/sparse_matrix.h:28-33). */
#define GB_SPARSE_MATRIX_TYPE_GB300 4

#define GB_SPARSE_MATRIX_TABLE(NAME, GO)                                                      \
  typedef struct NAME {                                                                      \
    int type;                                                                                \
    void *data;                                                                              \
    GO *global_ids;                                                                          \
    GO n_rows;                                                                               \
    GO n_cols;                                                                               \
    GO nnz;                                                                                  \
    int (*create_graph)(struct NAME *m, GO n_rows, GO *row_list, GO n_cols, GO *col_list,    \
                        GO local_nnz, GO max_nz_per_row, GO *coo_rows, GO *coo_cols);        \
    int (*complete_graph)(struct NAME *m);                                                   \
    int (*insert_row_values)(struct NAME *m, GO global_row, GO num_entries, double *values,  \
                             GO *indices);                                                   \
    int (*sum_into_row_values)(struct NAME *m, GO global_row, GO num_entries, double *values, \
                               GO *indices);                                                 \
    int (*put_scalar)(struct NAME *m, double scalar);                                        \
    int (*row_sum_scaling)(struct NAME *m, double *b, double *scale);                        \
    int (*zero_global_row)(struct NAME *m, GO global_row);                                   \
    int (*zero_global_row_set_diag)(struct NAME *m, GO global_row);                          \
    int (*matrix_vector_mult)(struct NAME *m, double *vector_in, double *vector_out);        \
    int (*destroy)(struct NAME *m);                                                          \
  } NAME;

GB_SPARSE_MATRIX_TABLE(gb_sparse_matrix_i32, int)
GB_SPARSE_MATRIX_TABLE(gb_sparse_matrix_i64, long long)
#undef GB_SPARSE_MATRIX_TABLE

/* GomaSparseMatrix_Create for the "gb300" format (the Epetra case is
 * GomaSparseMatrix_Epetra_Create, src/linalg/sparse_matrix_epetra.cpp:29):
 * sets type and every function pointer, data = NULL.  No device work:
 * create_graph allocates the device storage. */
int gb_sparse_matrix_create_i32(gb_sparse_matrix_i32 *m);
int gb_sparse_matrix_create_i64(gb_sparse_matrix_i64 *m);

/* The assembled matrix on the device, after uploading pending host edits:
 * rowptr (n_rows + 1, int64), colidx (nnz, local column indices),
 * values (nnz).  The pointers stay valid until destroy. */
int gb_sparse_matrix_device_csr_i32(gb_sparse_matrix_i32 *m, const long long **rowptr,
                                    const int **colidx, double **values);
int gb_sparse_matrix_device_csr_i64(gb_sparse_matrix_i64 *m, const long long **rowptr,
                                    const int **colidx, double **values);

#ifdef __cplusplus
}
#endif
#endif
