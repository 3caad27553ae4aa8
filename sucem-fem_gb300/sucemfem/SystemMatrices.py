"""SystemMatrices: assemble named bilinear forms on the GPU.

Same interface as sucemfem/SystemMatrices.py:26-58: set_matrix_class,
set_matrix_forms, set_boundary_conditions, calc_system_matrices -> dict of
matrices (None for a NullForm), essential conditions applied to every
assembled matrix.  All matrices of one call come out of a single fused
assembly launch on the shared cell pattern."""
import numpy as np
import torch

from . import Forms, _device, config
from ._native import call, ptr
from .matrix import GPUMatrix


class SystemMatrices:
    MatrixClass = GPUMatrix

    def set_matrix_class(self, matrix_class):
        # kept for interface parity; every matrix is a device CSR
        self.MatrixClass = matrix_class

    def set_matrix_forms(self, matrix_forms):
        self.matrix_forms = matrix_forms

    def set_boundary_conditions(self, boundary_conditions):
        self.boundary_conditions = boundary_conditions

    def set_function_space(self, function_space):
        self.function_space = function_space

    def _space(self):
        V = getattr(self, "function_space", None)
        if V is None:
            V = self.boundary_conditions.function_space
        return V

    def calc_system_matrices(self, real_bytes=None):
        V = self._space()
        rb = real_bytes or config.ASSEMBLY_REAL_BYTES
        rdt = _device.REAL[rb]
        out = {}
        plan = {}
        eps = mu_inv = None
        for name, form in self.matrix_forms.items():
            if isinstance(form, Forms.NullForm) or form is None:
                out[name] = None
                continue
            kinds = form.kinds()
            if len(set(kinds)) != 1:
                raise NotImplementedError("mixed-kind forms are not supported: %r" % kinds)
            kind = kinds[0]
            plan[name] = (kind, len(kinds))
            if kind == "mass":
                eps = form.terms[0][1]
            elif kind == "stiffness":
                mu_inv = 1.0 / np.asarray(form.terms[0][1], dtype=np.float64)
        bufs = {}
        for kind in set(k for k, _ in plan.values()):
            bufs[kind] = torch.empty(V.nnz, dtype=rdt, device=_device.device())
        d_eps = None if eps is None else _device.to_dev(np.asarray(eps, np.float64), rdt)
        d_mu = None if mu_inv is None else _device.to_dev(mu_inv, rdt)
        call("sucem_assemble", V.upload(), rb, ptr(d_eps), ptr(d_mu), ptr(bufs.get("stiffness")),
             ptr(bufs.get("mass")), ptr(bufs.get("abc")), _device.stream_ptr())
        used = set()
        for name, (kind, count) in plan.items():
            vals = bufs[kind] if kind not in used else bufs[kind].clone()
            used.add(kind)
            if count != 1:
                vals = vals * count
            mat = GPUMatrix(V, vals)
            self.boundary_conditions.apply_essential(mat)
            out[name] = mat
        return out


class SystemVectors:
    """Interface placeholder of sucemfem/SystemMatrices.py:61-80 (unused by
    the reference's drivers)."""

    def set_vector_forms(self, vector_forms):
        self.vector_forms = vector_forms

    def set_boundary_conditions(self, boundary_conditions):
        self.boundary_conditions = boundary_conditions

    def calc_system_vectors(self):
        raise NotImplementedError("linear-form assembly is provided by the Sources package")
