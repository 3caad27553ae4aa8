"""Driven problem with ABC (sucemfem/ProblemConfigurations/EMDrivenProblem.py:33-92).

get_LHS_matrix returns A = S - k0**2*M + 1j*k0*S_0 as a complex128 scipy
CSR exactly as the reference's scipy arithmetic would (exact complex zeros
dropped); the combination and the compaction run on the GPU."""
import numpy as N
import torch

from .. import Forms, _device
from .._native import call, ptr
from ..Consts import c0, Z0
from ..matrix import GPUMatrix
from .EMProblem import EMProblem


class CombineForms(Forms.CombineGalerkinForms):
    def get_forms(self):
        m = self.interior_forms.get_mass_form()
        s = self.interior_forms.get_stiffness_form()
        ABC_form = self.boundary_conditions.get_bilinear_form()
        return dict(M=m, S=s, S_0=ABC_form)


def k0_of(frequency):
    return 2 * N.pi * frequency / c0


def lhs_device(S, M, S_0, k0):
    """Full-pattern complex128 values of S - k0^2 M + 1j k0 S_0 (device)."""
    V = S.space
    out = torch.empty(V.nnz, dtype=torch.complex128, device=_device.device())
    call("sucem_combine", V.nnz, 8, 1.0, ptr(S.values), -(k0 ** 2), ptr(M.values),
         float(k0), ptr(S_0.values) if S_0 is not None else None, ptr(out), 1,
         _device.stream_ptr())
    return out


def compact_to_scipy(V, vals):
    """Drop exact zeros on the GPU and return a host scipy CSR."""
    import scipy.sparse as sps
    dev = _device.device()
    dt = 3 if vals.dtype == torch.complex128 else 2
    indptr = torch.empty(V.n + 1, dtype=torch.int32, device=dev)
    work = torch.empty(max(V.n, 1), dtype=torch.int32, device=dev)
    call("sucem_compact_count", V.upload(), dt, ptr(vals), ptr(indptr), ptr(work),
         _device.stream_ptr())
    nnz = int(indptr[-1].item())
    indices = torch.empty(max(nnz, 1), dtype=torch.int32, device=dev)
    out = torch.empty(max(nnz, 1), dtype=vals.dtype, device=dev)
    call("sucem_compact_fill", V.upload(), dt, ptr(vals), ptr(indptr), ptr(indices), ptr(out),
         _device.stream_ptr())
    return sps.csr_matrix((out[:nnz].cpu().numpy(), indices[:nnz].cpu().numpy(),
                           indptr.cpu().numpy()), shape=(V.n, V.n))


class DrivenProblemABC(EMProblem):
    FormCombiner = CombineForms

    def set_sources(self, sources):
        self.sources = sources

    def set_frequency(self, frequency):
        self.frequency = frequency

    def get_k0(self):
        return k0_of(self.frequency)

    def get_LHS_matrix(self):
        k0 = self.get_k0()
        m = self.system_matrices
        vals = lhs_device(m["S"], m["M"], m["S_0"], k0)
        return compact_to_scipy(self.function_space, vals)

    def get_LHS_device(self):
        """GPUMatrix of the full-pattern complex LHS (no compaction)."""
        k0 = self.get_k0()
        m = self.system_matrices
        return GPUMatrix(self.function_space, lhs_device(m["S"], m["M"], m["S_0"], k0))

    def get_RHS(self):
        RHS = N.zeros(self.get_global_dimension(), N.complex128)
        dofnos, contribs = self._get_RHS_contributions()
        k0 = self.get_k0()
        contribs = -1j * k0 * Z0 * contribs
        RHS[dofnos.astype(N.int64)] += contribs
        return RHS

    def _init_system_matrices(self):
        EMProblem._init_system_matrices(self, matrix_class=GPUMatrix)

    def _get_RHS_contributions(self):
        self.sources.set_function_space(self.function_space)
        self.sources.init_sources()
        return self.sources.get_source_contributions()
