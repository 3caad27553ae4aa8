"""N1curl orders 3 and 4 on the GPU (cell-based assembly through the C-ABI)
against the FP64 oracle, and the reference's higher-order functional tests
(functional_tests/test_EigenProblems.py:86-150) through the product's
EigenProblem / DefaultEigenSolver.

Tolerances: per-entry error over the largest |entry| of its row, as in
test_assembly_gpu.py: FP64 <= 1e-12; FP32 <= 5e-6 (sums of up to ~20 cell
contributions per entry, in ascending cell order); driven solve to the
FGMRES tolerance 1e-10 against scipy's direct solve of the oracle matrix;
cavity wavenumbers within the reference test's decimal=4 bound and the
oracle's eigenvalues within 1e-8."""
import numpy as np
import pytest

from oracle import fem
from test_assembly_gpu import _assemble, _row_err
from test_high_order_cpu import analytic_k, oracle_cavity_k, prism_mesh

pytestmark = pytest.mark.gpu

TOL = {8: 1e-12, 4: 5e-6}


def _jitter_box():
    coords, cells = fem.box_mesh(1.0, 0.5, 0.75, 3, 2, 2)
    return fem.jitter_interior(coords, cells, 0.25, 0.2, seed=1), cells


@pytest.mark.parametrize("rb", [8, 4])
@pytest.mark.parametrize("order", [3, 4])
@pytest.mark.parametrize("mesh", ["inscribed", "jitter"])
def test_high_order_assembly_matches_oracle(rb, order, mesh):
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    coords, cells = fem.inscribed_tet() if mesh == "inscribed" else _jitter_box()
    rng = np.random.default_rng(5)
    eps = rng.uniform(1, 4, len(cells))
    mu = rng.uniform(1, 2, len(cells))
    ref = fem.assemble(coords, cells, order, eps_r=eps, mu_r=mu)
    V = FunctionSpace(Mesh(coords, cells), order=order)
    got = _assemble(V, rb, eps, 1 / mu)
    for k, R in (("S", ref.S), ("T", ref.T), ("B", ref.B)):
        assert _row_err(got[k], R, 1.0 if k == "B" else 1e-6) <= TOL[rb], k
    # every entry is summed in a fixed order: a second assembly gives the
    # same bits
    again = _assemble(V, rb, eps, 1 / mu, which="T")
    assert np.array_equal(again["T"], got["T"])


@pytest.mark.parametrize("order", [3, 4])
def test_high_order_helmholtz_and_driven_solve(order):
    """Fused complex A = S - k0^2 T + j k0 B, then the FP32-LU + FP64-FGMRES
    driven solve against scipy's direct solve of the oracle matrix."""
    import scipy.sparse.linalg as spla
    import torch
    from sucemfem.mesh import Mesh
    from sucemfem.solvers import DrivenSolver
    from sucemfem.space import FunctionSpace
    coords, cells = _jitter_box()
    eps = np.random.default_rng(6).uniform(1, 4, len(cells))
    k0 = 2 * np.pi / 0.6
    import scipy.sparse as sps
    ref = fem.assemble(coords, cells, order, eps_r=eps)
    a_ref = ref.S.data - k0 ** 2 * ref.T.data + 1j * k0 * ref.B.data   # one pattern
    A_ref = sps.csr_matrix((a_ref, ref.S.indices, ref.S.indptr), shape=ref.S.shape)
    V = FunctionSpace(Mesh(coords, cells), order=order)
    ds = DrivenSolver(V, eps_r=eps)
    A = ds.assemble(k0, 8).cpu().numpy()
    assert np.abs(A - a_ref).max() <= 1e-12 * np.abs(a_ref).max()
    b = np.random.default_rng(7).standard_normal(V.n) + 0j
    x, info = ds.solve(k0, b, precision="fp32-ir", tol=1e-10)
    assert info["converged"], info
    x_ref = spla.spsolve(A_ref.tocsc(), b)
    x = x.cpu().numpy()
    assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
    torch.cuda.synchronize()


def _solve_cavity(mesh, pec, order, nev=10, sigma=1.1):
    from sucemfem.ProblemConfigurations.EMVectorWaveEigenproblem import DefaultEigenSolver, EigenProblem
    ep = EigenProblem()
    ep.set_mesh(mesh)
    ep.set_basis_order(order)
    ep.set_boundary_conditions(pec)
    ep.init_problem()
    es = DefaultEigenSolver()
    es.set_eigenproblem(ep)
    es.set_sigma(sigma)
    w, v = es.solve_problem(nev)
    assert w.shape == (nev,) and v.shape == (nev, ep.get_global_dimension())
    k2 = np.sort(1.0 / w.real + sigma)
    return np.sqrt(k2) / np.pi


def test_reference_cube_cavity_order3():
    """test_cube_resonant_cavity (test_EigenProblems.py:124-178):
    UnitCube(4,4,4), PEC walls from the mesh, order 3, sigma 1.1."""
    from sucemfem.BoundaryConditions import PECWallsBoundaryCondition
    from sucemfem.mesh import BoxMesh
    mesh = BoxMesh(1.0, 1.0, 1.0, 4, 4, 4)
    pec = PECWallsBoundaryCondition()
    pec.init_with_mesh(mesh)
    res = _solve_cavity(mesh, pec, 3)
    ref = analytic_k((1.0, 1.0, 1.0), 3)[:10]
    np.testing.assert_array_almost_equal(np.abs(res - ref) / ref, np.zeros(10), 4)
    c, t = fem.unit_cube(4, 4, 4)
    assert np.max(np.abs(res - oracle_cavity_k(c, t, 3)) / res) < 1e-8


def test_reference_prism_cavity_order4(tmp_path):
    """test_gmsh_resonant_cavity (test_EigenProblems.py:68-122): the
    rectangular prism XML mesh, PEC on facet region 1, order 4, sigma 1.1."""
    from sucemfem.BoundaryConditions import PECWallsBoundaryCondition
    m, f = prism_mesh(tmp_path)
    pec = PECWallsBoundaryCondition()
    pec.init_with_meshfunction(f, 1)
    res = _solve_cavity(m, pec, 4)
    ref = analytic_k((1.0, 0.5, 0.25), 5)[:10]
    np.testing.assert_array_almost_equal(np.abs(res - ref) / ref, np.zeros(10), 4)
    assert np.max(np.abs(res - oracle_cavity_k(m.coordinates(), m.cells(), 4)) / res) < 1e-8


def test_high_order_rejects_order_1_2_only_features():
    """Point sources and the post-processing kernels are provided for orders
    1 and 2; on order 3-4 spaces they fail loudly instead of misreading the
    element."""
    from sucemfem._native import call, ptr
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    coords, cells = fem.unit_cube(2, 2, 2)
    V = FunctionSpace(Mesh(coords, cells), order=3)
    h = V.upload()
    pts = np.array([[0.3, 0.3, 0.3]])
    vals = np.array([[0.0, 0.0, 1.0]])
    cells_out = np.zeros(1, dtype=np.int32)
    contrib = np.zeros(45 * 2)
    with pytest.raises(ValueError, match="orders 1 and 2"):
        call("sucem_point_sources", h, ptr(pts), ptr(vals), 1, ptr(cells_out), ptr(contrib), None)
