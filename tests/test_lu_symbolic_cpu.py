"""Symbolic multifrontal analysis on the CPU (no GPU needed): the
elimination order is a permutation, the assembly tree partitions the
unknowns into fronts, the dense fronts hold every fill entry of an exact
sparse LU in the same order (scipy's SuperLU without pivoting), with
bounded extra storage from the amalgamated leaves, and the nested
dissection order fills less than SuperLU's own COLAMD order."""
import numpy as np
import pytest
import scipy.sparse.linalg as spla

from oracle import fem


def _analyse(n, order):
    from sucemfem.mesh import Mesh
    from sucemfem.solvers import lu_for_space
    from sucemfem.space import FunctionSpace
    c, t = fem.unit_cube(n, n, n)
    V = FunctionSpace(Mesh(c, t), order=order)
    lu = lu_for_space(V)
    A = fem.assemble(c, t, order)
    M = (A.S - 20.0 * A.T + 1j * A.B).tocsc()    # the driven pencil's pattern and values
    return V, lu, M


@pytest.mark.parametrize("n,order", [(4, 2), (6, 1), (3, 3)])
def test_fronts_hold_the_exact_fill(n, order):
    V, lu, M = _analyse(n, order)
    p = lu.perm()
    assert np.array_equal(np.sort(p), np.arange(V.n))
    fr = lu.fronts()                      # (level, pivots k, front size f)
    assert fr[:, 1].sum() == V.n
    assert np.all(fr[:, 1] >= 1) and np.all(fr[:, 2] >= fr[:, 1])
    assert lu.info["nodes"] == len(fr) and lu.info["levels"] == fr[:, 0].max() + 1
    assert lu.info["max_front"] == fr[:, 2].max()
    # storage of the dense fronts: k x k pivot block, k x (f-k) of U and
    # (f-k) x k of L per front
    front_entries = int((fr[:, 1] * (2 * fr[:, 2] - fr[:, 1])).sum())
    Ap = M[p][:, p].tocsc()
    f = spla.splu(Ap, permc_spec="NATURAL", diag_pivot_thresh=0.0,
                  options=dict(SymmetricMode=True))
    exact = f.L.nnz + f.U.nnz - V.n
    assert exact <= front_entries <= 2 * exact
    # the reported factor work (multiply-adds, the unit of bench.py's
    # TFLOP/s figures) is that of the dense fronts: sum over the k pivots of
    # each front of its (f - i - 1)^2 rank-one update
    madds = sum(sum((int(f) - i - 1) ** 2 for i in range(int(k))) for _, k, f in fr)
    assert lu.info["flops"] == madds


def test_nested_dissection_fills_less_than_colamd():
    V, lu, M = _analyse(4, 2)
    p = lu.perm()
    Ap = M[p][:, p].tocsc()
    ours = spla.splu(Ap, permc_spec="NATURAL", diag_pivot_thresh=0.0,
                     options=dict(SymmetricMode=True))
    colamd = spla.splu(M, permc_spec="COLAMD")
    assert ours.L.nnz + ours.U.nnz < colamd.L.nnz + colamd.U.nnz
