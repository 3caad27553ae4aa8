"""Boundary-condition base class (sucemfem/BoundaryConditions/
base_boundary_condition.py:24-112): no essential part, null forms."""
from .. import Forms


class BoundaryCondition:
    mesh_function = None
    function_space = None
    boundary_value_expression = None
    region_number = None

    def set_boundary_value_expression(self, boundary_value_expression):
        self.boundary_value_expression = boundary_value_expression

    def set_mesh_function(self, mesh_function):
        self.mesh_function = mesh_function

    def set_region_number(self, region_number):
        self.region_number = region_number

    def set_function_space(self, function_space):
        self.function_space = function_space

    def get_essential_application_func(self, function_space=None):
        return lambda *args: None

    def get_linear_form(self, test_function=None):
        return Forms.NullForm()

    def get_bilinear_form(self, test_function=None, trial_function=None):
        return Forms.NullForm()
