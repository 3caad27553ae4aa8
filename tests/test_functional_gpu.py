"""functional_tests/test_current_fillament.py:41-161 through the product's
drop-in API: get_centred_cube, DrivenProblemABC with a 1000-point
FillamentCurrentSource, get_LHS_matrix / get_RHS, UMFPACKSolver, and the
surface NTFF's calc_pt per direction; the far-field errors against the
analytic filament field below the reference's 4.7 % and equal to the FP64
oracle's (test_functional_cpu.py) to 1e-6."""
import numpy as np
import pytest

from test_functional_cpu import filament_far_field_errors, oracle_solve_and_ntff

pytestmark = pytest.mark.gpu


def product_solve_and_ntff():
    from sucemfem.BoundaryConditions import ABCBoundaryCondition, BoundaryConditions
    from sucemfem.mesh import MeshFunction
    from sucemfem.PostProcessing import surface_ntff
    from sucemfem.ProblemConfigurations.EMDrivenProblem import DrivenProblemABC
    from sucemfem.Sources import current_source
    from sucemfem.Sources.fillament_current_source import FillamentCurrentSource
    from sucemfem.Utilities import LinalgSolvers
    from sucemfem.Utilities.MeshGenerators import get_centred_cube
    cache = {}

    def run(freq, lam, ends, I, theta, phi):
        if "dp" not in cache:
            mesh = get_centred_cube(np.array([lam] * 3), lam / 6)
            materials = MeshFunction("uint", mesh, 3)
            materials.set_all(0)
            abc = ABCBoundaryCondition()
            abc.set_region_number(1)
            bcs = BoundaryConditions()
            bcs.add_boundary_condition(abc)
            dp = DrivenProblemABC()
            dp.set_mesh(mesh)
            dp.set_basis_order(2)
            dp.set_material_regions({0: dict(eps_r=1, mu_r=1)})
            dp.set_region_meshfunction(materials)
            dp.set_boundary_conditions(bcs)
            sources = current_source.CurrentSources()
            fil = FillamentCurrentSource()
            fil.no_integration_points = 1000
            fil.set_source_endpoints(ends)
            fil.set_value(I)
            sources.add_source(fil)
            dp.set_sources(sources)
            dp.init_problem()
            dp.set_frequency(freq)
            cache.update(dp=dp, fil=fil, solver=LinalgSolvers.UMFPACKSolver(dp.get_LHS_matrix()))
        dp, fil = cache["dp"], cache["fil"]
        fil.set_source_endpoints(ends)
        x = cache["solver"].solve(dp.get_RHS())
        ntff = surface_ntff.NTFF(dp.function_space)
        ntff.set_dofs(x)
        ntff.set_frequency(freq)
        E = np.array([ntff.calc_pt(th, ph) for th, ph in zip(theta, phi)])
        return E[:, 0], E[:, 1]
    return run


def test_current_filament_far_field():
    got = filament_far_field_errors(product_solve_and_ntff())
    ref = filament_far_field_errors(oracle_solve_and_ntff())
    for g, r in zip(got, ref):
        assert g < 4.7
        assert abs(g - r) <= 1e-6 * r
