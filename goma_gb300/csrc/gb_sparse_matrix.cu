// GB300 backend of the reference's sparse-matrix plugin table (struct
// g_GomaSparseMatrix, include/linalg/sparse_matrix.h:35-88): the functions
// behind include/gb_sparse_matrix.h.  Semantics follow the Tpetra backend
// (src/linalg/sparse_matrix_tpetra.cpp): create_graph builds the pattern
// from the graph's COO lists (:42-95), insert_row_values replaces and
// sum_into_row_values adds values of existing entries, put_scalar sets every
// value, row_sum_scaling divides rows and b by the row's sum of absolute
// values (:160-198), zero_global_row[_set_diag] clear one row (and put 1 on
// its diagonal), matrix_vector_mult computes A x (:133-158).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/gb_sparse_matrix.h"
#include "gb_context.h"

namespace gb {
namespace {

__global__ void spm_fill_kernel(int64_t n, double *v, double s) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    v[i] = s;
}

// one warp per row: s = sum |a_ij| (1 for an all-zero row); the row and b
// are multiplied by 1/s and scale = 1/(1/s), as the Tpetra backend does
// (left scaling by the reciprocal row sums)
__global__ void spm_row_sum_scale_kernel(int64_t n_rows, const int64_t *__restrict__ rowptr,
                                         double *__restrict__ vals, double *__restrict__ b,
                                         double *__restrict__ scale) {
  const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n_rows) return;
  const int64_t r0 = rowptr[i], r1 = rowptr[i + 1];
  double s = 0.0;
  for (int64_t k = r0 + lane; k < r1; k += 32) s += fabs(vals[k]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (s == 0.0) s = 1.0;
  const double inv = 1.0 / s;
  for (int64_t k = r0 + lane; k < r1; k += 32) vals[k] *= inv;
  if (lane == 0) {
    b[i] *= inv;
    scale[i] = 1.0 / inv;
  }
}

// y = A x, one warp per row
__global__ void spm_matvec_kernel(int64_t n_rows, const int64_t *__restrict__ rowptr,
                                  const int *__restrict__ colidx, const double *__restrict__ vals,
                                  const double *__restrict__ x, double *__restrict__ y) {
  const int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n_rows) return;
  double s = 0.0;
  for (int64_t k = rowptr[i] + lane; k < rowptr[i + 1]; k += 32) s += vals[k] * x[colidx[k]];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[i] = s;
}

inline int grid_rows(int64_t n_rows) { return (int)((n_rows * 32 + 255) / 256); }

// The matrix behind the table's data pointer.
struct SparseMatrix {
  int64_t n_rows = 0, n_cols = 0, nnz = 0;
  std::vector<int64_t> rowptr;  // host copy of the pattern
  std::vector<int> colidx;
  std::unordered_map<long long, int64_t> row_of, col_of;  // global id -> local index
  bool rows_identity = true, cols_identity = true;
  double *h_vals = nullptr;  // pinned
  int64_t *d_rowptr = nullptr;
  int *d_colidx = nullptr;
  double *d_vals = nullptr;
  double *d_x = nullptr;  // n_cols
  double *d_y = nullptr;  // n_rows (matvec output, the b of row_sum_scaling)
  double *d_s = nullptr;  // n_rows (scale)
  cudaStream_t st = nullptr;
  bool host_current = true, dev_current = true;

  ~SparseMatrix() {
    if (st) cudaStreamSynchronize(st);
    for (void *p : {(void *)d_rowptr, (void *)d_colidx, (void *)d_vals, (void *)d_x, (void *)d_y,
                    (void *)d_s})
      if (p) cudaFree(p);
    if (h_vals) cudaFreeHost(h_vals);
    if (st) cudaStreamDestroy(st);
  }

  int64_t local_row(long long g) const {
    if (rows_identity) return (g >= 0 && g < n_rows) ? g : -1;
    auto it = row_of.find(g);
    return it == row_of.end() ? -1 : it->second;
  }
  int64_t local_col(long long g) const {
    if (cols_identity) return (g >= 0 && g < n_cols) ? g : -1;
    auto it = col_of.find(g);
    return it == col_of.end() ? -1 : it->second;
  }
  // position of local column c in local row r, -1 if outside the pattern
  int64_t find(int64_t r, int64_t c) const {
    const int *b = colidx.data() + rowptr[r], *e = colidx.data() + rowptr[r + 1];
    const int *p = std::lower_bound(b, e, (int)c);
    return (p != e && *p == c) ? rowptr[r] + (p - b) : -1;
  }
  int to_host() {
    if (host_current) return 0;
    cudaError_t e = cudaMemcpyAsync(h_vals, d_vals, sizeof(double) * nnz, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "gb300 matrix: values to host");
    host_current = true;
    return 0;
  }
  int to_device() {
    if (dev_current) return 0;
    cudaError_t e = cudaMemcpyAsync(d_vals, h_vals, sizeof(double) * nnz, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "gb300 matrix: values to device");
    dev_current = true;
    return 0;
  }
};

template <class M>
SparseMatrix *mat(M *m) {
  return static_cast<SparseMatrix *>(m->data);
}

template <class M>
int check(M *m, const char *what) {
  if (!m || !m->data) return fail(std::string("gb300 matrix: ") + what + " before create_graph");
  return 0;
}

#define SPM_CU(call, what)                           \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

template <class M, class GO>
int create_graph(M *m, GO n_rows, GO *row_list, GO n_cols, GO *col_list, GO local_nnz,
                 GO /*max_nz_per_row*/, GO *coo_rows, GO *coo_cols) {
  if (!m) return fail("gb300 matrix: null table");
  if (m->data) return fail("gb300 matrix: create_graph called twice");
  if (n_rows < 0 || n_cols < 0 || local_nnz < 0 || (n_rows > 0 && !row_list) ||
      (n_cols > 0 && !col_list) || (local_nnz > 0 && (!coo_rows || !coo_cols)))
    return fail("gb300 matrix: bad graph arguments");
  if ((long long)n_cols > 0x7fffffffLL) return fail("gb300 matrix: more than 2^31 - 1 columns");
  auto *A = new SparseMatrix();
  std::unique_ptr<SparseMatrix> guard(A);
  A->n_rows = n_rows;
  A->n_cols = n_cols;
  for (GO i = 0; i < n_rows; i++) A->rows_identity &= (long long)row_list[i] == (long long)i;
  for (GO i = 0; i < n_cols; i++) A->cols_identity &= (long long)col_list[i] == (long long)i;
  if (!A->rows_identity)
    for (GO i = 0; i < n_rows; i++)
      if (!A->row_of.emplace((long long)row_list[i], (int64_t)i).second)
        return fail("gb300 matrix: repeated row id");
  if (!A->cols_identity)
    for (GO i = 0; i < n_cols; i++)
      if (!A->col_of.emplace((long long)col_list[i], (int64_t)i).second)
        return fail("gb300 matrix: repeated column id");
  // COO -> CSR with ascending, unique columns per row
  std::vector<int64_t> cnt((size_t)n_rows + 1, 0);
  std::vector<int64_t> lr((size_t)local_nnz);
  std::vector<int> lc((size_t)local_nnz);
  for (GO k = 0; k < local_nnz; k++) {
    const int64_t r = A->local_row(coo_rows[k]), c = A->local_col(coo_cols[k]);
    if (r < 0) return fail("gb300 matrix: graph entry in a row not in row_list");
    if (c < 0) return fail("gb300 matrix: graph entry in a column not in col_list");
    lr[(size_t)k] = r;
    lc[(size_t)k] = (int)c;
    cnt[(size_t)r + 1]++;
  }
  for (int64_t i = 0; i < A->n_rows; i++) cnt[(size_t)i + 1] += cnt[(size_t)i];
  std::vector<int> cols((size_t)local_nnz);
  {
    std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
    for (GO k = 0; k < local_nnz; k++) cols[(size_t)pos[(size_t)lr[(size_t)k]]++] = lc[(size_t)k];
  }
  A->rowptr.assign((size_t)n_rows + 1, 0);
  A->colidx.reserve((size_t)local_nnz);
  for (int64_t i = 0; i < A->n_rows; i++) {
    auto b = cols.begin() + cnt[(size_t)i], e = cols.begin() + cnt[(size_t)i + 1];
    std::sort(b, e);
    e = std::unique(b, e);
    A->colidx.insert(A->colidx.end(), b, e);
    A->rowptr[(size_t)i + 1] = (int64_t)A->colidx.size();
  }
  A->nnz = (int64_t)A->colidx.size();
  // device copies, values zero (as the Tpetra backend's PutScalar(0))
  SPM_CU(cudaStreamCreateWithFlags(&A->st, cudaStreamNonBlocking), "gb300 matrix: stream");
  const size_t nz = (size_t)std::max<int64_t>(A->nnz, 1);
  SPM_CU(cudaMallocHost(&A->h_vals, sizeof(double) * nz), "gb300 matrix: host values");
  SPM_CU(cudaMalloc(&A->d_rowptr, sizeof(int64_t) * ((size_t)n_rows + 1)), "gb300 matrix: rowptr");
  SPM_CU(cudaMalloc(&A->d_colidx, sizeof(int) * nz), "gb300 matrix: colidx");
  SPM_CU(cudaMalloc(&A->d_vals, sizeof(double) * nz), "gb300 matrix: values");
  SPM_CU(cudaMalloc(&A->d_x, sizeof(double) * (size_t)std::max<GO>(n_cols, 1)), "gb300 matrix: x");
  SPM_CU(cudaMalloc(&A->d_y, sizeof(double) * (size_t)std::max<GO>(n_rows, 1)), "gb300 matrix: y");
  SPM_CU(cudaMalloc(&A->d_s, sizeof(double) * (size_t)std::max<GO>(n_rows, 1)), "gb300 matrix: s");
  SPM_CU(cudaMemcpyAsync(A->d_rowptr, A->rowptr.data(), sizeof(int64_t) * ((size_t)n_rows + 1),
                         cudaMemcpyHostToDevice, A->st), "gb300 matrix: rowptr");
  if (A->nnz)
    SPM_CU(cudaMemcpyAsync(A->d_colidx, A->colidx.data(), sizeof(int) * (size_t)A->nnz,
                           cudaMemcpyHostToDevice, A->st), "gb300 matrix: colidx");
  SPM_CU(cudaMemsetAsync(A->d_vals, 0, sizeof(double) * nz, A->st), "gb300 matrix: values");
  std::memset(A->h_vals, 0, sizeof(double) * nz);
  SPM_CU(cudaStreamSynchronize(A->st), "gb300 matrix: create_graph");
  m->data = guard.release();
  m->nnz = (GO)A->nnz;
  return 0;
}

template <class M>
int complete_graph(M *m) {
  return check(m, "complete_graph");
}

template <class M, class GO>
int row_values(M *m, GO global_row, GO num_entries, double *values, GO *indices, bool add) {
  if (check(m, add ? "sum_into_row_values" : "insert_row_values")) return -1;
  SparseMatrix *A = mat(m);
  const int64_t r = A->local_row(global_row);
  if (r < 0) return fail("gb300 matrix: row " + std::to_string((long long)global_row) + " not local");
  if (num_entries > 0 && (!values || !indices)) return fail("gb300 matrix: null row values");
  if (A->to_host()) return -1;
  for (GO k = 0; k < num_entries; k++) {
    const int64_t c = A->local_col(indices[k]);
    const int64_t p = c < 0 ? -1 : A->find(r, c);
    if (p < 0)
      return fail("gb300 matrix: entry (" + std::to_string((long long)global_row) + ", " +
                  std::to_string((long long)indices[k]) + ") is not in the graph");
    if (add) A->h_vals[p] += values[k];
    else A->h_vals[p] = values[k];
  }
  A->dev_current = false;
  return 0;
}

template <class M, class GO>
int insert_row_values(M *m, GO global_row, GO num_entries, double *values, GO *indices) {
  return row_values<M, GO>(m, global_row, num_entries, values, indices, false);
}
template <class M, class GO>
int sum_into_row_values(M *m, GO global_row, GO num_entries, double *values, GO *indices) {
  return row_values<M, GO>(m, global_row, num_entries, values, indices, true);
}

template <class M>
int put_scalar(M *m, double s) {
  if (check(m, "put_scalar")) return -1;
  SparseMatrix *A = mat(m);
  if (A->nnz) {
    spm_fill_kernel<<<304, 256, 0, A->st>>>(A->nnz, A->d_vals, s);
    SPM_CU(cudaGetLastError(), "gb300 matrix: put_scalar");
  }
  std::fill(A->h_vals, A->h_vals + A->nnz, s);
  SPM_CU(cudaStreamSynchronize(A->st), "gb300 matrix: put_scalar");
  A->host_current = A->dev_current = true;
  return 0;
}

template <class M>
int row_sum_scaling(M *m, double *b, double *scale) {
  if (check(m, "row_sum_scaling")) return -1;
  SparseMatrix *A = mat(m);
  if (A->n_rows && (!b || !scale)) return fail("gb300 matrix: null b or scale");
  if (A->to_device()) return -1;
  if (A->n_rows) {
    SPM_CU(cudaMemcpyAsync(A->d_y, b, sizeof(double) * A->n_rows, cudaMemcpyHostToDevice, A->st),
           "gb300 matrix: b to device");
    spm_row_sum_scale_kernel<<<grid_rows(A->n_rows), 256, 0, A->st>>>(A->n_rows, A->d_rowptr,
                                                                      A->d_vals, A->d_y, A->d_s);
    SPM_CU(cudaGetLastError(), "gb300 matrix: row_sum_scaling");
    SPM_CU(cudaMemcpyAsync(b, A->d_y, sizeof(double) * A->n_rows, cudaMemcpyDeviceToHost, A->st),
           "gb300 matrix: b to host");
    SPM_CU(cudaMemcpyAsync(scale, A->d_s, sizeof(double) * A->n_rows, cudaMemcpyDeviceToHost, A->st),
           "gb300 matrix: scale to host");
  }
  SPM_CU(cudaStreamSynchronize(A->st), "gb300 matrix: row_sum_scaling");
  A->host_current = false;
  return 0;
}

template <class M, class GO>
int zero_row(M *m, GO global_row, bool set_diag) {
  if (check(m, "zero_global_row")) return -1;
  SparseMatrix *A = mat(m);
  const int64_t r = A->local_row(global_row);
  if (r < 0) return fail("gb300 matrix: row " + std::to_string((long long)global_row) + " not local");
  if (A->to_host()) return -1;
  const int64_t dc = set_diag ? A->local_col(global_row) : -1;
  for (int64_t p = A->rowptr[(size_t)r]; p < A->rowptr[(size_t)r + 1]; p++)
    A->h_vals[p] = (set_diag && A->colidx[(size_t)p] == dc) ? 1.0 : 0.0;
  A->dev_current = false;
  return 0;
}

template <class M, class GO>
int zero_global_row(M *m, GO global_row) {
  return zero_row<M, GO>(m, global_row, false);
}
template <class M, class GO>
int zero_global_row_set_diag(M *m, GO global_row) {
  return zero_row<M, GO>(m, global_row, true);
}

template <class M>
int matrix_vector_mult(M *m, double *x, double *y) {
  if (check(m, "matrix_vector_mult")) return -1;
  SparseMatrix *A = mat(m);
  if ((A->n_cols && !x) || (A->n_rows && !y)) return fail("gb300 matrix: null vector");
  if (A->to_device()) return -1;
  if (A->n_cols)
    SPM_CU(cudaMemcpyAsync(A->d_x, x, sizeof(double) * A->n_cols, cudaMemcpyHostToDevice, A->st),
           "gb300 matrix: x to device");
  if (A->n_rows) {
    spm_matvec_kernel<<<grid_rows(A->n_rows), 256, 0, A->st>>>(A->n_rows, A->d_rowptr,
                                                               A->d_colidx, A->d_vals, A->d_x,
                                                               A->d_y);
    SPM_CU(cudaGetLastError(), "gb300 matrix: matrix_vector_mult");
    SPM_CU(cudaMemcpyAsync(y, A->d_y, sizeof(double) * A->n_rows, cudaMemcpyDeviceToHost, A->st),
           "gb300 matrix: y to host");
  }
  SPM_CU(cudaStreamSynchronize(A->st), "gb300 matrix: matrix_vector_mult");
  return 0;
}

template <class M>
int destroy(M *m) {
  if (!m) return 0;
  delete mat(m);
  m->data = nullptr;
  return 0;
}

template <class M, class GO>
int create(M *m) {
  if (!m) return fail("gb300 matrix: null table");
  m->type = GB_SPARSE_MATRIX_TYPE_GB300;
  m->data = nullptr;
  m->create_graph = create_graph<M, GO>;
  m->complete_graph = complete_graph<M>;
  m->insert_row_values = insert_row_values<M, GO>;
  m->sum_into_row_values = sum_into_row_values<M, GO>;
  m->put_scalar = put_scalar<M>;
  m->row_sum_scaling = row_sum_scaling<M>;
  m->zero_global_row = zero_global_row<M, GO>;
  m->zero_global_row_set_diag = zero_global_row_set_diag<M, GO>;
  m->matrix_vector_mult = matrix_vector_mult<M>;
  m->destroy = destroy<M>;
  return 0;
}

template <class M>
int device_csr(M *m, const long long **rowptr, const int **colidx, double **values) {
  if (check(m, "device_csr")) return -1;
  SparseMatrix *A = mat(m);
  if (A->to_device()) return -1;
  SPM_CU(cudaStreamSynchronize(A->st), "gb300 matrix: device_csr");
  if (rowptr) *rowptr = reinterpret_cast<const long long *>(A->d_rowptr);
  if (colidx) *colidx = A->d_colidx;
  if (values) *values = A->d_vals;
  // the caller may change the values on the device
  A->host_current = false;
  return 0;
}

}  // namespace
}  // namespace gb

extern "C" {
int gb_sparse_matrix_create_i32(gb_sparse_matrix_i32 *m) {
  return gb::create<gb_sparse_matrix_i32, int>(m);
}
int gb_sparse_matrix_create_i64(gb_sparse_matrix_i64 *m) {
  return gb::create<gb_sparse_matrix_i64, long long>(m);
}
int gb_sparse_matrix_device_csr_i32(gb_sparse_matrix_i32 *m, const long long **rowptr,
                                    const int **colidx, double **values) {
  return gb::device_csr(m, rowptr, colidx, values);
}
int gb_sparse_matrix_device_csr_i64(gb_sparse_matrix_i64 *m, const long long **rowptr,
                                    const int **colidx, double **values) {
  return gb::device_csr(m, rowptr, colidx, values);
}
}
