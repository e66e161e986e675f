"""The "gb300" backend of the reference's sparse-matrix plugin table on the
GPU, against numpy on the reference's own golden matrices: the graph of the
reference's MSR pattern, values summed in row by row (as LoadLec does),
A x, row-sum scaling (Tpetra semantics: divide by the sum of absolute
values), row replacement and zeroing, put_scalar, and errors for entries
outside the graph."""
import numpy as np
import pytest

from goma_gb300 import _lib
from goma_gb300.sparse_matrix import GpuSparseMatrix
from tests import golden_cases as gc

pytestmark = pytest.mark.gpu


def _dense_from_msr(ija, a):
    N = int(ija[0]) - 1
    D = np.zeros((N, N))
    D[np.arange(N), np.arange(N)] = a[:N]
    for i in range(N):
        for k in range(ija[i], ija[i + 1]):
            D[i, ija[k]] += a[k]
    return D


@pytest.mark.parametrize("ordinal", [32, 64])
@pytest.mark.parametrize("name,offset", [("cav2d_3x2_pert", 0), ("box3d_2x2x2_bouss", 0),
                                         ("cav2d_3x2_pert", 1000)])
def test_gb300_matrix_format(name, offset, ordinal):
    g, case = gc.load(name)
    ija, a = g["ija"], g["a"]
    D = _dense_from_msr(ija, a)
    N = D.shape[0]
    pattern = [sorted([i] + list(ija[ija[i]:ija[i + 1]])) for i in range(N)]
    coo_r = np.concatenate([[i] * len(p) for i, p in enumerate(pattern)]) + offset
    coo_c = np.concatenate(pattern) + offset
    ids = np.arange(N) + offset
    m = GpuSparseMatrix(ordinal)
    m.create_graph(ids, ids, coo_r, coo_c)
    assert m.t.nnz == len(coo_c)
    m.complete_graph()
    m.put_scalar(0.0)
    # values summed in two halves, row by row
    for i, p in enumerate(pattern):
        v = D[i, p]
        m.sum_into_row_values(i + offset, 0.25 * v, np.array(p) + offset)
        m.sum_into_row_values(i + offset, 0.75 * v, np.array(p) + offset)
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, N)
    scale_ref = np.abs(D @ x).max()
    assert np.abs(m.matrix_vector_mult(x) - D @ x).max() <= 1e-13 * scale_ref
    # replace one row, then restore it
    r = N // 2
    m.insert_row_values(r + offset, np.arange(len(pattern[r])) + 1.0, np.array(pattern[r]) + offset)
    y = m.matrix_vector_mult(x)
    w = np.arange(len(pattern[r])) + 1.0
    assert abs(y[r] - w @ x[pattern[r]]) <= 1e-14 * (np.abs(w) @ np.abs(x[pattern[r]]))
    m.insert_row_values(r + offset, D[r, pattern[r]], np.array(pattern[r]) + offset)
    # row-sum scaling: divide by sum |a_ij|
    b = rng.uniform(-1, 1, N)
    bs, s = m.row_sum_scaling(b)
    s_ref = np.abs(D).sum(axis=1)
    s_ref[s_ref == 0] = 1.0
    assert np.abs(s - s_ref).max() <= 1e-14 * s_ref.max()
    assert np.abs(bs - b / s_ref).max() <= 1e-14 * np.abs(b / s_ref).max()
    Ds = D / s_ref[:, None]
    assert np.abs(m.matrix_vector_mult(x) - Ds @ x).max() <= 1e-13 * np.abs(Ds @ x).max()
    # zero a row with and without a unit diagonal (after device-side changes)
    m.zero_global_row_set_diag(r + offset)
    m.zero_global_row(r + 1 + offset)
    y = m.matrix_vector_mult(x)
    assert y[r] == x[r] and y[r + 1] == 0.0
    others = np.setdiff1d(np.arange(N), [r, r + 1])
    assert np.abs(y[others] - (Ds @ x)[others]).max() <= 1e-13 * np.abs(Ds @ x).max()
    # entries outside the graph are errors and change nothing
    outside = [j for j in range(N) if j not in set(pattern[0])]
    if outside:
        with pytest.raises(_lib.GbError, match="not in the graph"):
            m.sum_into_row_values(offset, [1.0], [outside[0] + offset])
    m.put_scalar(0.0)
    assert not np.any(m.matrix_vector_mult(x))
    m.close()
    assert not m.t.data
