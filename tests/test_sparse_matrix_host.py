"""The "gb300" backend of the reference's sparse-matrix plugin table, the
parts that need no GPU: gb_sparse_matrix_create_* fills the table's type
and every function pointer without touching a device, calls before
create_graph fail cleanly, and create_graph checks its graph on the host
before any device work."""
import ctypes

import numpy as np
import pytest

from goma_gb300 import _lib
from goma_gb300.sparse_matrix import GpuSparseMatrix, table_type

FUNCS = ["create_graph", "complete_graph", "insert_row_values", "sum_into_row_values",
         "put_scalar", "row_sum_scaling", "zero_global_row", "zero_global_row_set_diag",
         "matrix_vector_mult", "destroy"]


@pytest.mark.parametrize("ordinal", [32, 64])
def test_create_fills_the_table(ordinal):
    m = GpuSparseMatrix(ordinal)
    assert m.t.type == 4 and not m.t.data
    for f in FUNCS:
        assert ctypes.cast(getattr(m.t, f), ctypes.c_void_p).value, f
    T = table_type(ordinal)
    go = 4 if ordinal == 32 else 8
    # the reference's layout: enum, data, global_ids, three ordinals, ten pointers
    assert T.n_rows.offset == 24 and T.create_graph.offset == 24 + ((3 * go + 7) // 8) * 8
    assert ctypes.sizeof(T) == T.create_graph.offset + 10 * 8


@pytest.mark.parametrize("ordinal", [32, 64])
def test_calls_before_the_graph_and_bad_graphs_fail_cleanly(ordinal):
    m = GpuSparseMatrix(ordinal)
    m.n_rows = 2
    with pytest.raises(_lib.GbError, match="before create_graph"):
        m.put_scalar(0.0)
    with pytest.raises(_lib.GbError, match="before create_graph"):
        m.matrix_vector_mult(np.zeros(2))
    rows = np.arange(3)
    with pytest.raises(_lib.GbError, match="not in row_list"):
        m.create_graph(rows, rows, [0, 1, 5], [0, 1, 2])
    with pytest.raises(_lib.GbError, match="not in col_list"):
        m.create_graph(rows, rows, [0, 1, 2], [0, 1, 7])
    with pytest.raises(_lib.GbError, match="repeated row id"):
        m.create_graph([0, 0, 1], rows, [0], [0])
    assert not m.t.data
