"""Bilinear-form descriptors (the reference builds UFL forms here,
sucemfem/Forms.py:25-116).  A form is a recipe the GPU assembler evaluates:
which reference tensor, which per-cell coefficient."""


class NullForm:
    """Zero contribution; adding it to a form returns the other form."""
    _integrals = []

    def __add__(self, other):
        return other

    def __radd__(self, other):
        return other


class BilinearForm:
    """Sum of terms (kind, coefficient) with kind in {'mass','stiffness','abc'}."""

    def __init__(self, terms):
        self.terms = list(terms)

    def __add__(self, other):
        if isinstance(other, NullForm):
            return self
        return BilinearForm(self.terms + other.terms)

    __radd__ = __add__

    def kinds(self):
        return [k for k, _ in self.terms]


class GalerkinInteriorForms:
    def set_material_functions(self, material_functions):
        self.material_functions = material_functions

    def set_function_space(self, function_space):
        self.function_space = function_space

    def get_mass_form(self):
        raise NotImplementedError()

    def get_stiffness_form(self):
        raise NotImplementedError()


class EMGalerkinInteriorForms(GalerkinInteriorForms):
    """mass eps_r*inner(v,u)*dx and stiffness dot(curl v, curl u)/mu_r*dx
    (sucemfem/Forms.py:71-85)."""

    def get_mass_form(self):
        return BilinearForm([("mass", self.material_functions["eps_r"])])

    def get_stiffness_form(self):
        return BilinearForm([("stiffness", self.material_functions["mu_r"])])


class CombineGalerkinForms:
    def set_interior_forms(self, interior_forms):
        self.interior_forms = interior_forms

    def set_boundary_conditions(self, boundary_conditions):
        self.boundary_conditions = boundary_conditions

    def get_combined_forms(self):
        raise NotImplementedError("Use a concrete class")
