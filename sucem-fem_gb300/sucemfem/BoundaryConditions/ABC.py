"""First-order ABC: bilinear form inner(cross(n,v), cross(n,u))*ds over
every exterior facet; the region number is ignored, as in the reference
(sucemfem/BoundaryConditions/ABC.py:26-57)."""
from .. import Forms
from .base_boundary_condition import BoundaryCondition


class ABCBoundaryCondition(BoundaryCondition):
    def get_bilinear_form(self, test_function=None, trial_function=None):
        return Forms.BilinearForm([("abc", None)])
