"""Device-resident CSR matrix on a FunctionSpace's pattern.

Stands in for the dolfin matrix classes the reference passes around
(PETScMatrix / uBLASSparseMatrix, sucemfem/SystemMatrices.py:27,
EMDrivenProblem.py:86-87) and offers exactly the methods its callers use:
``data()`` and ``size(i)`` (sucemfem/Utilities/Converters.py:37-40),
``S - sigma*M`` (EMVectorWaveEigenproblem.py:76) and ``M*x``
(EMVectorWaveEigenproblem.py:86,98).  Values live on the GPU; every
operation is a libsucem_gb300 kernel."""
import numpy as np
import torch

from . import _device, _native
from ._native import call, ptr

_DT = {torch.float32: _native.F32, torch.float64: _native.F64,
       torch.complex64: _native.C64, torch.complex128: _native.C128}


class GPUMatrix:
    def __init__(self, space, values):
        self.space = space
        self.values = values          # torch tensor (nnz,) on the device

    # -- dolfin-matrix surface -------------------------------------------
    def size(self, dim):
        return self.space.n

    @property
    def shape(self):
        return (self.space.n, self.space.n)

    def data(self):
        """(row pointer, column indices, values) as host numpy arrays."""
        return (self.space.indptr, self.space.indices, self.values.cpu().numpy())

    def ident_rows(self, rows):
        rows = np.ascontiguousarray(rows, dtype=np.int32)
        if rows.size == 0:
            return
        d_rows = _device.to_dev(rows)
        call("sucem_apply_essential", self.space.upload(), _DT[self.values.dtype],
             ptr(self.values), ptr(d_rows), len(rows), _device.stream_ptr())

    def _combine(self, a, other, b):
        rb = self.values.element_size()
        if self.values.is_complex() or (other is not None and other.values.is_complex()):
            raise TypeError("linear combination of complex matrices is not supported")
        out = torch.empty_like(self.values)
        call("sucem_combine", self.space.nnz, rb, float(a), ptr(self.values), float(b),
             ptr(other.values) if other is not None else None, 0.0, None, ptr(out), 0,
             _device.stream_ptr())
        return GPUMatrix(self.space, out)

    def __sub__(self, other):
        return self._combine(1.0, other, -1.0)

    def __add__(self, other):
        return self._combine(1.0, other, 1.0)

    def __mul__(self, other):
        if np.isscalar(other):
            return self._combine(float(other), None, 0.0)
        return self.matvec(other)

    __rmul__ = lambda self, other: self.__mul__(other)

    def matvec(self, x):
        """A*x with x a numpy vector or device tensor (returns the same kind)."""
        is_np = not torch.is_tensor(x)
        xd = _device.to_dev(x) if is_np else x
        vals = self.values
        if xd.is_complex() and not vals.is_complex():
            cdt = torch.complex64 if vals.dtype == torch.float32 else torch.complex128
            vals = vals.to(cdt)
        elif vals.is_complex() and not xd.is_complex():
            xd = xd.to(vals.dtype)
        xd = xd.to(vals.dtype).contiguous()
        y = torch.empty(self.space.n, dtype=vals.dtype, device=vals.device)
        call("sucem_spmv", self.space.upload(), _DT[vals.dtype], ptr(vals), ptr(xd), ptr(y),
             _device.stream_ptr())
        return y.cpu().numpy() if is_np else y

    def to_scipy(self, dtype=None):
        import scipy.sparse as sps
        indptr, indices, data = self.data()
        return sps.csr_matrix((data, indices.astype(np.intc), indptr.astype(np.intc)),
                              shape=self.shape, dtype=dtype)

    def array(self):
        return self.to_scipy().toarray()
