"""Essential (Dirichlet) conditions; PEC walls.

Same behaviour as dolfin.DirichletBC(...).apply with the topological
method used by sucemfem/BoundaryConditions/essential.py:65-99: every DOF on
the closure of a marked facet gets its matrix row zeroed and a unit
diagonal (columns untouched); a RHS vector gets the boundary value (0 for
PEC).  The row treatment runs on the GPU (sucem_apply_essential)."""
import numpy as np

from ..mesh import DomainBoundary, MeshFunction
from .base_boundary_condition import BoundaryCondition


class EssentialBoundaryCondition(BoundaryCondition):
    def init_with_meshfunction(self, mesh_function, region_number):
        self.set_region_number(region_number)
        self.set_mesh_function(mesh_function)

    def set_PEC_expression(self):
        self.set_boundary_value_expression(0.0)

    def constrained_dofs(self, function_space=None):
        V = function_space if function_space is not None else self.function_space
        mf = self.mesh_function
        if getattr(mf, "mark_all_exterior", False) and mf.boundary_value == self.region_number:
            return V.boundary_dofs
        faces = np.nonzero(np.asarray(mf.array()) == self.region_number)[0]
        return V.facet_closure_dofs(faces)

    def get_essential_application_func(self, function_space=None):
        if function_space is not None:
            self.set_function_space(function_space)
        if self.boundary_value_expression is None:
            self.set_PEC_expression()
        if self.boundary_value_expression != 0.0:
            raise NotImplementedError("only homogeneous (PEC) essential values are supported")
        dofs = self.constrained_dofs()

        def apply(A, b=None):
            A.ident_rows(dofs)
            if b is not None:
                b[dofs] = 0.0
        return apply


class PECWallsBoundaryCondition(EssentialBoundaryCondition):
    def init_with_mesh(self, mesh):
        mesh_function = MeshFunction("uint", mesh, 2)
        mesh_function.set_all(0)
        DomainBoundary().mark(mesh_function, 999)
        self.init_with_meshfunction(mesh_function, 999)
