"""Matrix converters (sucemfem/Utilities/Converters.py:27-51)."""
import numpy as np


def dolfin_ublassparse_to_scipy_csr(A, dtype=None, imagify=False):
    """(row, col, data) = A.data() -> scipy.sparse.csr_matrix, int32 indices."""
    import scipy.sparse
    (row, col, data) = A.data()
    col = np.intc(col)
    row = np.intc(row)
    n = A.size(0)
    if imagify:
        data = data * 1j
    return scipy.sparse.csr_matrix((data, col, row), shape=(n, n), dtype=dtype)


def as_dolfin_vector(a):
    assert len(a.shape) == 1
    return np.require(a, requirements=["C"]).copy()
