"""LinalgSolvers drop-in (sucemfem/Utilities/tests/test_LinalgSolvers.py:35-95
and the solver classes of LinalgSolvers.py:239-322)."""
import numpy as np
import pytest
import scipy.sparse
import scipy.sparse.linalg as spl

from oracle import fem


def _ls():
    from sucemfem.Utilities import LinalgSolvers
    return LinalgSolvers


@pytest.mark.parametrize("bshape,xshape", [((1000,), None), ((1, 1000), None), ((1000, 1), None),
                                           ((1000,), (1000, 1)), ((1, 1000), (1000, 1)),
                                           ((1000, 1), (1000, 1))])
def test_calculate_residual_shapes(bshape, xshape):
    # TestOther: residual of x == b against the identity is exactly zero
    A = scipy.sparse.eye(1000, 1000)
    b = np.random.default_rng(0).random(bshape)
    x = b.copy().reshape(xshape if xshape else (1000,))
    assert _ls().calculate_residual(A, x, b) == 0


@pytest.mark.gpu
def test_sparse_identity_exact():
    A = scipy.sparse.eye(1000, 1000).tocsr()
    b = np.random.default_rng(1).random(1000)
    x = _ls().solve_sparse_system(A, b)
    np.testing.assert_array_equal(b, x)


def _driven(order=1):
    coords, cells = fem.box_mesh(1.0, 1.0, 1.0, 4, 4, 4)
    eps = np.random.default_rng(2).uniform(1, 4, len(cells))
    f = 299792458 / 0.4
    A = fem.assemble(coords, cells, order, eps_r=eps)
    L = fem.lhs_matrix(A.S, A.T, A.B, f)
    d, v = fem.point_source_contrib(coords, cells, order, A.topo, A.dofmap,
                                    np.array([0.5, 0.5, 0.5]), np.array([0, 0, 1.0]))
    return L.tocsr(), fem.rhs_vector(A.n, f, d, v)


@pytest.mark.gpu
@pytest.mark.parametrize("cls", ["BiCGStabSolver", "HostBiCGStabSolver", "GMRESSolver", "UMFPACKSolver"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_solvers_on_driven_system(cls, precision):
    LS = _ls()
    old = LS.FACTOR_PRECISION
    LS.FACTOR_PRECISION = precision
    try:
        L, b = _driven()
        s = getattr(LS, cls)(L, "ilu")
        s.tol = 1e-10
        x = s.solve(b)
        xr = spl.spsolve(L.tocsc(), b)
        assert np.linalg.norm(L @ x - b) / np.linalg.norm(b) < 1e-9
        assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-7
        log = s.get_logging_data()
        assert log["id"][0] == "init" and "solve::end" in log["id"]
    finally:
        LS.FACTOR_PRECISION = old


@pytest.mark.gpu
def test_diagonal_preconditioner_converges_on_dominant_system():
    LS = _ls()
    rng = np.random.default_rng(3)
    n = 500
    A = (scipy.sparse.random(n, n, 0.01, random_state=4) + scipy.sparse.eye(n) * 5).tocsr()
    A = A + A.T
    b = rng.standard_normal(n)
    s = LS.BiCGStabSolver(A, "diagonal")
    s.tol = 1e-10
    x = s.solve(b)
    assert np.linalg.norm(A @ x - b) / np.linalg.norm(b) < 1e-9
    assert len(s.get_logging_data()["res"]) > 3
