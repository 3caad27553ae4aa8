"""Eigen problem and its default solver
(sucemfem/ProblemConfigurations/EMVectorWaveEigenproblem.py:38-105).

DefaultEigenSolver.solve_problem(nev, ncv) returns (eigs_w, eigs_v) as the
reference does: eigs_w are eigenvalues mu of (S - sigma M)^-1 M, i.e.
mu = 1/(k^2 - sigma) (user code recovers k^2 = 1/mu + sigma), eigs_v has
shape (nev, n).  The computation is the GPU shift-invert Lanczos of
sucemfem.eigen with the essential-BC DOFs eliminated (see that module).
Selection: the nev largest mu, i.e. the nev smallest k^2 above sigma; the
reference asks ARPACK for the mu nearest sigma, which selects the same modes
whenever every selected mu lies below 2*sigma (sigma below the first
nonzero k^2, as in its examples).  Eigenvalues come sorted by k^2."""
import numpy as np

from .. import Forms
from ..eigen import BatchedShiftInvertLanczos
from .EMProblem import EMProblem


class CombineForms(Forms.CombineGalerkinForms):
    def get_forms(self):
        m = self.interior_forms.get_mass_form()
        s = self.interior_forms.get_stiffness_form()
        BC_bilin_forms = self.boundary_conditions.get_bilinear_form()
        return dict(M=m, S=s, BC=BC_bilin_forms)


class EigenProblem(EMProblem):
    FormCombiner = CombineForms

    def constrained_dofs(self):
        out = [np.zeros(0, dtype=np.int64)]
        for bc in self.boundary_conditions.boundary_conditions.values():
            if hasattr(bc, "constrained_dofs"):
                out.append(np.asarray(bc.constrained_dofs(self.function_space), dtype=np.int64))
        return np.unique(np.concatenate(out))


class DefaultEigenSolver:
    precision = "fp32"   # LU precision; "fp64" for the plain double path

    def set_eigenproblem(self, eigenproblem):
        self.eigenproblem = eigenproblem

    def set_sigma(self, sigma):
        self.sigma = sigma

    def solve_problem(self, nev, ncv=None):
        ep = self.eigenproblem
        M = ep.system_matrices["M"]
        S = ep.system_matrices["S"]
        if M.values.dtype != S.values.dtype or M.values.element_size() != 8:
            raise ValueError("eigen solve needs double-precision system matrices")
        self.solver = BatchedShiftInvertLanczos(ep.function_space, S.values, M.values,
                                                ep.constrained_dofs(), self.sigma)
        k2, Z = self.solver.solve(nev, ncv=ncv, precision=self.precision)
        self.k2 = k2[0]
        eigs_w = (1.0 / (k2[0] - self.sigma)).astype(np.complex128)
        eigs_v = self.solver.full_vectors(Z, 0)
        return eigs_w, eigs_v

    def get_k2(self):
        """k^2 of the last solve (ascending)."""
        return self.k2
