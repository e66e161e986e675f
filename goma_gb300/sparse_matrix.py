"""Python mirror of the reference's sparse-matrix plugin table
(struct g_GomaSparseMatrix, include/linalg/sparse_matrix.h:35-88) for the
"gb300" format of include/gb_sparse_matrix.h.

`table_type(ordinal)` gives a ctypes Structure with the table's layout
(GomaGlobalOrdinal int or long long); `GpuSparseMatrix` fills one through
gb_sparse_matrix_create_* and calls its function pointers exactly as the
reference's code does (create_graph from GomaSparseMatrix_SetProblemGraph,
sum_into_row_values from GomaSparseMatrix_LoadLec, ...), raising GbError
on a -1 return.
"""
import ctypes

import numpy as np

from goma_gb300 import _lib

_TABLES = {}


def table_type(ordinal=32):
    """ctypes Structure with the layout of struct g_GomaSparseMatrix for a
    32-bit (int) or 64-bit (long long) GomaGlobalOrdinal."""
    if ordinal in _TABLES:
        return _TABLES[ordinal]
    GO = ctypes.c_int if ordinal == 32 else ctypes.c_longlong
    GOP = ctypes.POINTER(GO)
    DP = ctypes.POINTER(ctypes.c_double)

    class Table(ctypes.Structure):
        pass

    TP = ctypes.POINTER(Table)
    F = ctypes.CFUNCTYPE
    i = ctypes.c_int
    Table._fields_ = [
        ("type", ctypes.c_int),
        ("data", ctypes.c_void_p),
        ("global_ids", GOP),
        ("n_rows", GO),
        ("n_cols", GO),
        ("nnz", GO),
        ("create_graph", F(i, TP, GO, GOP, GO, GOP, GO, GO, GOP, GOP)),
        ("complete_graph", F(i, TP)),
        ("insert_row_values", F(i, TP, GO, GO, DP, GOP)),
        ("sum_into_row_values", F(i, TP, GO, GO, DP, GOP)),
        ("put_scalar", F(i, TP, ctypes.c_double)),
        ("row_sum_scaling", F(i, TP, DP, DP)),
        ("zero_global_row", F(i, TP, GO)),
        ("zero_global_row_set_diag", F(i, TP, GO)),
        ("matrix_vector_mult", F(i, TP, DP, DP)),
        ("destroy", F(i, TP)),
    ]
    Table.go = GO
    Table.np_go = np.int32 if ordinal == 32 else np.int64
    _TABLES[ordinal] = Table
    return Table


class GpuSparseMatrix:
    """A "gb300"-format matrix behind the plugin table."""

    def __init__(self, ordinal=32):
        self._L = _lib.load()
        self.T = table_type(ordinal)
        self.t = self.T()
        self._ref = ctypes.byref(self.t)
        suffix = "i32" if ordinal == 32 else "i64"
        fn = getattr(self._L, "gb_sparse_matrix_create_" + suffix)
        fn.argtypes = [ctypes.POINTER(self.T)]
        fn.restype = ctypes.c_int
        _lib.check(fn(self._ref))

    def _arr(self, a):
        a = np.ascontiguousarray(a, self.T.np_go)
        return a, a.ctypes.data_as(ctypes.POINTER(self.T.go))

    @staticmethod
    def _dp(a):
        return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))

    def create_graph(self, row_list, col_list, coo_rows, coo_cols):
        """Pattern from COO lists (ordered by row, as SetProblemGraph gives
        them); the values start at zero."""
        rl, rlp = self._arr(row_list)
        cl, clp = self._arr(col_list)
        cr, crp = self._arr(coo_rows)
        cc, ccp = self._arr(coo_cols)
        max_per_row = int(np.unique(cr, return_counts=True)[1].max()) if len(cr) else 0
        self.t.n_rows, self.t.n_cols = len(rl), len(cl)
        _lib.check(self.t.create_graph(self._ref, len(rl), rlp, len(cl), clp, len(cr),
                                       max_per_row, crp, ccp))
        self.n_rows, self.n_cols = len(rl), len(cl)

    def complete_graph(self):
        _lib.check(self.t.complete_graph(self._ref))

    def insert_row_values(self, row, values, indices):
        v = np.ascontiguousarray(values, np.float64)
        ix, ixp = self._arr(indices)
        _lib.check(self.t.insert_row_values(self._ref, row, len(v), self._dp(v), ixp))

    def sum_into_row_values(self, row, values, indices):
        v = np.ascontiguousarray(values, np.float64)
        ix, ixp = self._arr(indices)
        _lib.check(self.t.sum_into_row_values(self._ref, row, len(v), self._dp(v), ixp))

    def put_scalar(self, s):
        _lib.check(self.t.put_scalar(self._ref, float(s)))

    def row_sum_scaling(self, b):
        """Scales the rows and b by 1 / sum |a_ij|: returns (scaled b, scale)."""
        b = np.ascontiguousarray(b, np.float64).copy()
        s = np.empty(self.n_rows)
        _lib.check(self.t.row_sum_scaling(self._ref, self._dp(b), self._dp(s)))
        return b, s

    def zero_global_row(self, row):
        _lib.check(self.t.zero_global_row(self._ref, row))

    def zero_global_row_set_diag(self, row):
        _lib.check(self.t.zero_global_row_set_diag(self._ref, row))

    def matrix_vector_mult(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.empty(self.n_rows)
        _lib.check(self.t.matrix_vector_mult(self._ref, self._dp(x), self._dp(y)))
        return y

    def close(self):
        if getattr(self, "t", None) is not None and self.t.data:
            _lib.check(self.t.destroy(self._ref))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
