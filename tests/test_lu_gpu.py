"""GPU multifrontal LU against scipy's sparse direct solve (the oracle side
of the reference's UMFPACK/LUSolver calls).  Tolerances: relative residual
of the single-precision factor solve < 1e-4 (one solve) and < 1e-12 after
double-precision refinement; double-precision factor < 1e-11."""
import numpy as np
import pytest
import scipy.sparse.linalg as spl

from oracle import fem

pytestmark = pytest.mark.gpu


def _problem(order, n=(4, 3, 3), driven=True):
    coords, cells = fem.box_mesh(1.0, 0.8, 0.6, *n)
    rng = np.random.default_rng(1)
    eps = rng.uniform(1, 4, len(cells))
    A = fem.assemble(coords, cells, order, eps_r=eps)
    if driven:
        L = fem.lhs_matrix(A.S, A.T, A.B, 299792458 / 0.7)
    else:
        L = (A.S - 1.0 * A.T)
    return coords, cells, L.tocsr(), A


def _space(coords, cells, order):
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    return FunctionSpace(Mesh(coords, cells), order=order)


def _values_on_pattern(V, M):
    """Values of scipy matrix M on the space's CSR pattern."""
    M = M.tocsr()
    out = np.zeros(V.nnz, dtype=M.dtype)
    rows = np.repeat(np.arange(V.n), np.diff(V.indptr))
    out[:] = np.asarray(M[rows, V.indices]).ravel()
    return out


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("dtype", ["c64", "c128"])
@pytest.mark.parametrize("ordering", ["cells", "dofs"])
def test_lu_driven(order, dtype, ordering):
    import torch
    from sucemfem import _device
    from sucemfem.lu import SparseLU
    coords, cells, L, _ = _problem(order)
    V = _space(coords, cells, order)
    vals = _values_on_pattern(V, L)
    if ordering == "cells":
        lu = SparseLU(V.indptr, V.indices, leaf_size=32,
                      cells=(V.cell_dofs, coords[V.cells].mean(1)))
    else:
        lu = SparseLU(V.indptr, V.indices, V.dof_xyz, leaf_size=32)
    assert sorted(lu.perm()) == list(range(V.n))
    tdt = torch.complex64 if dtype == "c64" else torch.complex128
    dv = torch.as_tensor(vals, device=_device.device()).to(tdt)
    lu.factor(dv, dtype)
    b = np.random.default_rng(0).standard_normal(V.n) + 1j * np.random.default_rng(1).standard_normal(V.n)
    db = torch.as_tensor(b, device=_device.device())
    x = lu.solve(db if dtype == "c128" else db).cpu().numpy()
    res = np.linalg.norm(L @ x - b) / np.linalg.norm(b)
    assert res < (1e-4 if dtype == "c64" else 1e-11), res
    xr = spl.spsolve(L.tocsc(), b)
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < (1e-3 if dtype == "c64" else 1e-9)
    assert lu.perturbed() == 0


@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_lu_real_indefinite(dtype):
    import torch
    from sucemfem import _device
    from sucemfem.lu import SparseLU
    coords, cells = fem.box_mesh(1.0, 0.5, 0.75, 4, 2, 3)
    A = fem.assemble(coords, cells, 1, with_abc=False)
    V = _space(coords, cells, 1)
    M = (A.S - 1.3 * A.T).tocsr()
    vals = M.data.copy()  # oracle pattern == space pattern (bit-exact)
    lu = SparseLU(V.indptr, V.indices, leaf_size=16, cells=(V.cell_dofs, coords[V.cells].mean(1)))
    tdt = torch.float32 if dtype == "f32" else torch.float64
    lu.factor(torch.as_tensor(vals, device=_device.device()).to(tdt), dtype)
    b = np.random.default_rng(0).standard_normal(V.n)
    x = lu.solve(torch.as_tensor(b, device=_device.device())).cpu().numpy()
    res = np.linalg.norm(M @ x - b) / np.linalg.norm(b)
    assert res < (1e-3 if dtype == "f32" else 1e-11), res


def test_bounded_wait_gives_up_and_the_context_stays_usable():
    """Failure detection without a fault: a device wait on a barrier phase
    that nothing completes (the tensor-core kernel's own bounded wait, here
    limited to 2000 polls) gives up and its kernel returns; afterwards the
    same process factorises and solves as usual."""
    from sucemfem.lu import SparseLU
    assert SparseLU.selftest_bounded_wait(2000)
    test_lu_driven(2, "c64", "cells")


def test_timed_out_factor_is_refused_until_refactored():
    """A factorisation whose tensor-core update gave up waiting must not be
    used: the failure is injected on the host (the device flag is written,
    no kernel is made to fail); the status check and every later solve then
    raise, and a fresh factorisation clears it."""
    import torch
    from sucemfem import _device
    from sucemfem.lu import SparseLU
    coords, cells, L, _ = _problem(1)
    V = _space(coords, cells, 1)
    vals = torch.as_tensor(_values_on_pattern(V, L), device=_device.device()).to(torch.complex64)
    lu = SparseLU(V.indptr, V.indices, leaf_size=32, cells=(V.cell_dofs, coords[V.cells].mean(1)))
    b = torch.ones(V.n, dtype=torch.complex128, device=_device.device())
    lu.factor(vals, "c64").check()
    lu._inject_timeout()
    with pytest.raises(RuntimeError, match="gave up"):
        lu.check()
    with pytest.raises(RuntimeError, match="gave up"):
        lu.solve(b)
    with pytest.raises(RuntimeError, match="gave up"):
        lu.perturbed()
    lu.factor(vals, "c64")
    x = lu.solve(b).cpu().numpy()
    res = np.linalg.norm(L @ x - b.cpu().numpy()) / np.linalg.norm(b.cpu().numpy())
    assert res < 1e-4


@pytest.mark.parametrize("dtype", ["c64", "f32", "c128"])
def test_lookahead_solve_matches_the_sequential_schedule(dtype, monkeypatch):
    """Levels of three or more 128-column sub-steps solve with a look-ahead
    schedule on two streams (each sub-step's products split into the part
    the next triangular solve needs and the rest, run beside it, adding
    atomically).  On a mesh whose top fronts span several sub-steps the
    solution matches the one-stream schedule to the rounding of the
    changed summation order (1e-5 relative in single, 1e-12 in double
    precision) and solves the system."""
    import torch
    from sucemfem import _device
    from sucemfem.lu import SparseLU
    coords, cells = fem.box_mesh(1.0, 0.8, 0.6, 8, 6, 6)
    rng = np.random.default_rng(3)
    if dtype == "f32":
        A = fem.assemble(coords, cells, 2, with_abc=False)
        M = (A.S - 1.3 * A.T).tocsr()
        b = rng.standard_normal(M.shape[0])
        tdt = torch.float32
    else:
        A = fem.assemble(coords, cells, 2, eps_r=rng.uniform(1, 4, len(cells)))
        M = fem.lhs_matrix(A.S, A.T, A.B, 299792458 / 0.7).tocsr()
        b = rng.standard_normal(M.shape[0]) + 1j * rng.standard_normal(M.shape[0])
        tdt = torch.complex64 if dtype == "c64" else torch.complex128
    V = _space(coords, cells, 2)
    vals = torch.as_tensor(_values_on_pattern(V, M), device=_device.device()).to(tdt)
    db = torch.as_tensor(b, device=_device.device())
    xs = []
    for sequential in (False, True):
        if sequential:
            monkeypatch.setenv("SUCEM_LU_SOLVE_SEQUENTIAL", "1")
        # a new handle: the solve's launch graph is built at its first solve
        lu = SparseLU(V.indptr, V.indices, leaf_size=32,
                      cells=(V.cell_dofs, coords[V.cells].mean(1)))
        top = lu.fronts()
        assert top[:, 1].max() > 2 * 128  # a level of three or more sub-steps
        lu.factor(vals, dtype)
        xs.append(lu.solve(db).cpu().numpy())
    tol = 1e-12 if dtype == "c128" else 1e-5
    assert np.linalg.norm(xs[0] - xs[1]) / np.linalg.norm(xs[1]) < tol
    res = np.linalg.norm(M @ xs[0] - b) / np.linalg.norm(b)
    assert res < {"c64": 1e-4, "f32": 1e-3, "c128": 1e-11}[dtype], res


@pytest.mark.parametrize("dtype", ["c128", "f64"])
def test_block_gram_schmidt_matches_two_pass_projection(dtype):
    """sucem_vec_gs (FGMRES's orthogonalisation on the device): against a
    numpy two-pass classical Gram-Schmidt of the same vectors, the
    coefficients, the orthogonalised vector and its norm agree to 1e-12."""
    import torch
    from sucemfem import _device
    from sucemfem.solvers import Vec
    rng = np.random.default_rng(7)
    n, k = 5000, 6
    cplx = dtype == "c128"
    A = rng.standard_normal((k + 1, n)) + (1j * rng.standard_normal((k + 1, n)) if cplx else 0)
    Q, _ = np.linalg.qr(A[:k].T)
    Vh = np.zeros((k + 1, n), dtype=A.dtype)
    Vh[:k] = Q.T
    wh = A[k].copy()
    tdt = torch.complex128 if cplx else torch.float64
    V = torch.as_tensor(Vh, device=_device.device()).to(tdt)
    w = torch.as_tensor(wh, device=_device.device()).to(tdt)
    c, nrm = Vec().gs(V, k, w)
    c1 = Vh[:k].conj() @ wh
    w1 = wh - Vh[:k].T @ c1
    c2 = Vh[:k].conj() @ w1
    w2 = w1 - Vh[:k].T @ c2
    assert np.allclose(c, c1 + c2, rtol=1e-12, atol=1e-12)
    assert np.allclose(w.cpu().numpy(), w2, rtol=1e-12, atol=1e-12)
    assert abs(nrm - np.linalg.norm(w2)) < 1e-12 * np.linalg.norm(w2)
