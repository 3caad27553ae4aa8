"""Field reconstruction at points (sucemfem/PostProcessing/PostProcessing.py:
27-60 ``Reconstruct``), evaluated on the GPU by sucem_reconstruct_points."""
import ctypes

import numpy as np

from .. import _device, _native
from .._native import call, ptr

c_vp = ctypes.c_void_p
_native.declare("sucem_reconstruct_points", ctypes.c_int,
                [c_vp, ctypes.c_int, c_vp, c_vp, ctypes.c_int, c_vp, c_vp, c_vp])


def device_dofs(dofs):
    """DOF vector on the device as complex128 (a device complex64/complex128
    tensor is used as is)."""
    import torch
    if isinstance(dofs, torch.Tensor) and dofs.is_cuda:
        if dofs.dtype not in (torch.complex64, torch.complex128):
            dofs = dofs.to(torch.complex128)
        return dofs.contiguous()
    return torch.as_tensor(np.asarray(dofs, dtype=np.complex128), device=_device.device())


def dtype_code(t):
    import torch
    return _native.C64 if t.dtype == torch.complex64 else _native.C128


class Reconstruct:
    """``Reconstruct(function_space)``: ``set_dof_values(x)`` then
    ``reconstruct_points(points)`` -> complex array (npts, 3) of E; a point
    outside the mesh gives NaN (the reference raises from dolfin)."""

    def __init__(self, function_space):
        self.function_space = function_space
        self.x = None

    def set_dof_values(self, x):
        self.x = device_dofs(x)

    def reconstruct_points(self, points):
        import torch
        if self.x is None:
            raise ValueError("set_dof_values() first")
        V = self.function_space
        pts = np.ascontiguousarray(np.atleast_2d(points), dtype=np.float64)
        npts = len(pts)
        dev = _device.device()
        d_pts = torch.as_tensor(pts, device=dev)
        cells = torch.empty(npts, dtype=torch.int32, device=dev)
        E = torch.empty(npts * 3, dtype=torch.complex128, device=dev)
        call("sucem_reconstruct_points", V.upload(), dtype_code(self.x), ptr(self.x), ptr(d_pts),
             npts, ptr(cells), ptr(E), _device.stream_ptr())
        return E.cpu().numpy().reshape(npts, 3)
