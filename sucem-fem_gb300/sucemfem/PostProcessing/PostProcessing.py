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


_native.declare("sucem_em_functional", ctypes.c_int,
                [c_vp, c_vp, c_vp, ctypes.c_double, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp])
_native.declare("sucem_boundary_edge_cells", ctypes.c_int, [c_vp, c_vp])


def boundary_edge_cells(function_space):
    """Cells with an edge on the boundary (Geometry.BoundaryEdgeCells), as a
    uint8 array per cell."""
    mask = np.zeros(function_space.nt, dtype=np.uint8)
    call("sucem_boundary_edge_cells", function_space._h, ptr(mask))
    return mask


class CalcEMFunctional:
    """Evaluate the EM functional <curl E, curl g>/mu_r - k0^2 eps_r <E, g>
    (bilinear) over the whole mesh or the cells of a marked region, E the
    field solution and g an H(curl) testing function, both DOF vectors of
    the function space; evaluated on the GPU element by element."""

    def __init__(self, function_space, testing_space=None):
        if testing_space is not None and testing_space is not function_space:
            raise ValueError("the testing space must be the function space")
        self.function_space = function_space
        self.testing_space = function_space
        self.k0 = None
        self.E = None
        self.g = None
        self.mask = None
        self.eps = None
        self.mu_inv = None

    def set_k0(self, k0):
        self.k0 = float(k0)

    def set_cell_domains(self, cell_domains, cell_mark_value):
        """Restrict the integral to the cells where cell_domains (a cell
        MeshFunction or an array per cell) equals cell_mark_value."""
        import torch
        a = cell_domains.array() if hasattr(cell_domains, "array") else np.asarray(cell_domains)
        m = (np.asarray(a) == cell_mark_value).astype(np.uint8)
        self.set_cell_mask(m)

    def set_cell_mask(self, mask):
        import torch
        self.mask = torch.as_tensor(np.asarray(mask, dtype=np.uint8), device=_device.device())

    def _per_cell(self, values, invert=False):
        import torch
        if values is None:
            return None
        v = np.broadcast_to(np.asarray(values, dtype=np.float64), (self.function_space.nt,))
        return torch.as_tensor(1.0 / v if invert else v.copy(), device=_device.device())

    def set_epsr_function(self, epsr_function):
        """Relative permittivity: a number or one value per cell."""
        self.eps = self._per_cell(epsr_function)

    def set_mur_function(self, mur_function):
        """Relative permeability: a number or one value per cell."""
        self.mu_inv = self._per_cell(mur_function, invert=True)

    def set_quadrature_degree(self, quadrature_degree):
        """Accepted for interface parity: the element tensors are exact."""
        self.quadrature_degree = quadrature_degree

    def set_E_dofs(self, E_dofs):
        self.E = _c128(E_dofs)

    def set_g_dofs(self, g_dofs):
        self.g = _c128(g_dofs)

    def calc_functional(self):
        """Calculate functional using given E, g and k0 values"""
        import torch
        if self.E is None or self.g is None or self.k0 is None:
            raise ValueError("set_E_dofs(), set_g_dofs() and set_k0() first")
        V = self.function_space
        dev = _device.device()
        part = torch.empty(2 * V.nt, dtype=torch.float64, device=dev)
        out = torch.empty(2, dtype=torch.float64, device=dev)
        call("sucem_em_functional", V.upload(), ptr(self.E), ptr(self.g), self.k0,
             ptr(self.eps), ptr(self.mu_inv), ptr(self.mask), ptr(part), ptr(out),
             _device.stream_ptr())
        o = out.cpu().numpy()
        return complex(o[0], o[1])


def _c128(dofs):
    import torch
    x = device_dofs(dofs)
    return x if x.dtype == torch.complex128 else x.to(torch.complex128)
