"""BoundaryConditions container (sucemfem/BoundaryConditions/container.py:25-68)."""
from .. import Forms


class BoundaryConditions:
    def __init__(self):
        self.boundary_conditions = {}

    def add_boundary_condition(self, boundary_condition):
        bc_num = boundary_condition.region_number
        # boundary condition numbers have to be unique
        assert bc_num not in self.boundary_conditions
        self.boundary_conditions[bc_num] = boundary_condition

    def apply_essential(self, A, b=None):
        for bc_num, bc in self.boundary_conditions.items():
            apply_fn = bc.get_essential_application_func()
            if b is not None:
                apply_fn(A, b)
            else:
                apply_fn(A)

    def get_linear_form(self):
        lin = Forms.NullForm()
        for bc in self.boundary_conditions.values():
            lin = lin + bc.get_linear_form()
        return lin

    def get_bilinear_form(self):
        bilin = Forms.NullForm()
        for bc in self.boundary_conditions.values():
            bilin = bilin + bc.get_bilinear_form()
        return bilin

    def set_function_space(self, function_space):
        self.function_space = function_space
        for bc in self.boundary_conditions.values():
            bc.set_function_space(function_space)
