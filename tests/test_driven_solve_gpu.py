"""Driven solves on the GPU (multifrontal LU + double-precision refinement)
against the oracle (scipy direct solve of the oracle's LHS/RHS) and against
the reference's own order-2 solution golden.  Bar: relative residual of the
FP64-assembled system <= 1e-10 and the solution within 1e-8 of the oracle's."""
import numpy as np
import pytest
import scipy.sparse.linalg as spl

from conftest import golden
from oracle import fem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("precision", ["fp32-ir", "fp64"])
@pytest.mark.parametrize("method", ["gmres", "ir"])
def test_driven_solve_matches_oracle(order, precision, method):
    from sucemfem.mesh import Mesh
    from sucemfem.solvers import DrivenSolver
    from sucemfem.space import FunctionSpace
    coords, cells = fem.box_mesh(1.0, 1.0, 1.0, 4, 4, 4)
    eps = np.random.default_rng(2).uniform(1, 4, len(cells))
    f = 299792458 / 0.4
    k0 = 2 * np.pi * f / 299792458
    A = fem.assemble(coords, cells, order, eps_r=eps)
    L = fem.lhs_matrix(A.S, A.T, A.B, f)
    d, v = fem.point_source_contrib(coords, cells, order, A.topo, A.dofmap,
                                    np.array([0.5, 0.5, 0.5]), np.array([0, 0, 1.0]))
    b = fem.rhs_vector(A.n, f, d, v)
    xr = spl.spsolve(L.tocsc(), b)
    V = FunctionSpace(Mesh(coords, cells), order=order)
    ds = DrivenSolver(V, eps_r=eps)
    x, info = ds.solve(k0, b, precision=precision, tol=1e-10, method=method)
    x = x.cpu().numpy()
    assert info["converged"], info
    assert np.linalg.norm(L @ x - b) / np.linalg.norm(b) <= 1.5e-10
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) <= 1e-8


def test_power_flux_golden_through_gpu_solver():
    """Order-2 driven solution of the reference (power_flux_generate_dofs.py)."""
    from sucemfem.BoundaryConditions import ABCBoundaryCondition, BoundaryConditions
    from sucemfem.ProblemConfigurations.EMDrivenProblem import DrivenProblemABC
    from sucemfem.Sources import current_source
    from sucemfem.Sources.fillament_current_source import FillamentCurrentSource
    from sucemfem.mesh import Mesh, MeshFunction
    from sucemfem.solvers import DrivenSolver
    g = golden("power_flux_solution_o2.npz")
    lam = 299792458 / float(g["freq"])
    mesh = Mesh(*fem.centred_cube(np.array([lam] * 3) * 0.25, lam / 6))
    abc = ABCBoundaryCondition()
    abc.set_region_number(1)
    bcs = BoundaryConditions()
    bcs.add_boundary_condition(abc)
    dp = DrivenProblemABC()
    dp.set_mesh(mesh)
    dp.set_basis_order(2)
    mf = MeshFunction("uint", mesh, 3)
    mf.set_all(0)
    dp.set_material_regions({0: dict(eps_r=1, mu_r=1)})
    dp.set_region_meshfunction(mf)
    dp.set_boundary_conditions(bcs)
    cs = current_source.CurrentSources()
    fs = FillamentCurrentSource()
    fs.set_source_endpoints(g["source_endpoints"])
    fs.set_value(float(g["I"]))
    cs.add_source(fs)
    dp.set_sources(cs)
    dp.init_problem()
    dp.set_frequency(float(g["freq"]))
    b = dp.get_RHS()
    ds = DrivenSolver(dp.function_space)
    x, info = ds.solve(dp.get_k0(), b, precision="fp32-ir", tol=1e-12)
    x = x.cpu().numpy()
    assert np.linalg.norm(x - g["x"]) / np.linalg.norm(g["x"]) < 1e-9
