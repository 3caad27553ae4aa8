"""Shift-invert eigen solves on the GPU against the FP64 oracle (dense
generalized eigenproblem of the PEC-free oracle matrices) and against the
analytic cavity wavenumbers (functional_tests/test_EigenProblems.py:42-65).

Bars: k^2 within 1e-9 relative of the oracle (FP32 LU + FP64 Lanczos/RR);
analytic agreement only up to the discretisation error (order 1 on the
8x4x6 mesh: a few per cent; order 2: < 1 %)."""
import numpy as np
import pytest
import scipy.linalg as sla

from oracle import fem

pytestmark = pytest.mark.gpu


def analytic_k2(a, b, d, count):
    vals = []
    for m in range(6):
        for n in range(6):
            for l in range(6):
                idx = (m, n, l)
                if idx.count(0) >= 2:
                    continue
                k2 = np.pi ** 2 * ((m / a) ** 2 + (n / b) ** 2 + (l / d) ** 2)
                vals += [k2] * (2 if idx.count(0) == 0 else 1)
    return np.sort(vals)[:count]


def oracle_k2(coords, cells, order, nev, sigma, eps=None):
    A = fem.assemble(coords, cells, order, eps_r=eps, with_abc=False)
    pec = fem.pec_dofs(A.topo, order)
    free = np.setdiff1d(np.arange(A.n), pec)
    S = A.S.toarray()[np.ix_(free, free)]
    T = A.T.toarray()[np.ix_(free, free)]
    w = sla.eigh(S, T, eigvals_only=True)
    return np.sort(w[w > sigma])[:nev]


def _cavity_problem(a, b, d, nx, ny, nz, order):
    from sucemfem.BoundaryConditions import PECWallsBoundaryCondition
    from sucemfem.ProblemConfigurations.EMVectorWaveEigenproblem import EigenProblem
    from sucemfem.mesh import BoxMesh
    mesh = BoxMesh(a, b, d, nx, ny, nz)
    pec = PECWallsBoundaryCondition()
    pec.init_with_mesh(mesh)
    ep = EigenProblem()
    ep.set_mesh(mesh)
    ep.set_basis_order(order)
    ep.set_boundary_conditions(pec)
    ep.init_problem()
    return ep, mesh


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_config1_cavity_order1(precision):
    from sucemfem.ProblemConfigurations.EMVectorWaveEigenproblem import DefaultEigenSolver
    ep, mesh = _cavity_problem(1.0, 0.5, 0.75, 8, 4, 6, 1)
    es = DefaultEigenSolver()
    es.precision = precision
    es.set_eigenproblem(ep)
    es.set_sigma(1.0)
    w, v = es.solve_problem(10)
    assert w.shape == (10,) and v.shape == (10, ep.get_global_dimension())
    k2 = np.sort(1.0 / w.real + 1.0)
    ref = oracle_k2(*fem.box_mesh(1.0, 0.5, 0.75, 8, 4, 6), 1, 10, 1.0)
    assert np.max(np.abs(k2 - ref) / ref) < 1e-9
    ana = analytic_k2(1.0, 0.5, 0.75, 10)
    assert np.max(np.abs(k2 - ana) / ana) < 0.08
    # eigenvectors: unit norm, zero on PEC DOFs, satisfy S x = k^2 T x
    A = fem.assemble(*fem.box_mesh(1.0, 0.5, 0.75, 8, 4, 6), 1, with_abc=False)
    pec = fem.pec_dofs(A.topo, 1)
    assert np.allclose(np.linalg.norm(v, axis=1), 1.0)
    assert np.all(v[:, pec] == 0)
    free = np.setdiff1d(np.arange(A.n), pec)
    kk = 1.0 / w.real + 1.0
    for i in range(10):
        x = v[i, free].real
        r = A.S[free][:, free] @ x - kk[i] * (A.T[free][:, free] @ x)
        assert np.linalg.norm(r) <= 1e-7 * kk[i] * np.linalg.norm(A.T[free][:, free] @ x)


def test_order2_cavity():
    from sucemfem.ProblemConfigurations.EMVectorWaveEigenproblem import DefaultEigenSolver
    ep, mesh = _cavity_problem(1.0, 1.0, 1.0, 3, 3, 3, 2)
    es = DefaultEigenSolver()
    es.set_eigenproblem(ep)
    es.set_sigma(1.1)
    w, v = es.solve_problem(6)
    k2 = np.sort(1.0 / w.real + 1.1)
    ref = oracle_k2(*fem.box_mesh(1.0, 1.0, 1.0, 3, 3, 3), 2, 6, 1.1)
    assert np.max(np.abs(k2 - ref) / ref) < 1e-9
    ana = analytic_k2(1.0, 1.0, 1.0, 6)
    assert np.max(np.abs(k2 - ana) / ana) < 0.03


def test_batched_cavities_match_individual_oracles():
    """Three cavities of different sizes stacked in one space: one assembly
    launch, one LU, one batched Lanczos; each matches its own oracle."""
    import torch
    from sucemfem import _device
    from sucemfem._native import call, ptr
    from sucemfem.eigen import BatchedShiftInvertLanczos
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    boxes = [((1.0, 0.5, 0.75), (6, 3, 4)), ((0.6, 0.6, 0.9), (4, 4, 5)), ((1.2, 0.4, 0.5), (7, 3, 3))]
    rng = np.random.default_rng(4)
    coords, cells, seg_cells, eps, off = [], [], [], [], 0
    for k, ((a, b, d), n) in enumerate(boxes):
        c, t = fem.box_mesh(a, b, d, *n, origin=(3.0 * k, 0, 0))
        coords.append(c)
        cells.append(t + off)
        off += len(c)
        seg_cells.append(np.full(len(t), k))
        eps.append(rng.uniform(1, 4, len(t)))
    V = FunctionSpace(Mesh(np.concatenate(coords), np.concatenate(cells)), order=1)
    seg_cells = np.concatenate(seg_cells)
    dof_seg = np.zeros(V.n, dtype=np.int64)
    dof_seg[V.cell_dofs.ravel()] = np.repeat(seg_cells, 6)
    dev = _device.device()
    S = torch.empty(V.nnz, dtype=torch.float64, device=dev)
    T = torch.empty_like(S)
    d_eps = torch.as_tensor(np.concatenate(eps), device=dev)
    call("sucem_assemble", V.upload(), 8, ptr(d_eps), None, ptr(S), ptr(T), None, _device.stream_ptr())
    sol = BatchedShiftInvertLanczos(V, S, T, V.boundary_dofs, 1.0, dof_segment=dof_seg)
    k2, Z = sol.solve(6)
    for k, ((a, b, d), n) in enumerate(boxes):
        c, t = fem.box_mesh(a, b, d, *n)
        ref = oracle_k2(c, t, 1, 6, 1.0, eps=eps[k])
        assert np.max(np.abs(np.sort(k2[k]) - ref) / ref) < 1e-9, k
