"""Power flux through the mesh boundary (sucemfem/PostProcessing/
power_flux.py:11-60 ``SurfaceFlux``), integrated on the GPU by
sucem_surface_flux."""
import ctypes

import numpy as np

from .. import _device, _native
from .._native import call, ptr
from .PostProcessing import device_dofs, dtype_code

c_vp = ctypes.c_void_p
_native.declare("sucem_surface_flux", ctypes.c_int,
                [c_vp, ctypes.c_int, c_vp, ctypes.c_double, c_vp, c_vp, c_vp, c_vp])


class SurfaceFlux:
    """Real part of the power flux (integral of the Poynting vector E x H*
    over the bounding surface, outward normal); RMS power is half of it
    (peak-value phasors).  Only the problem's bounding surface is used, as in
    the reference."""

    def __init__(self, function_space):
        self.function_space = function_space
        self.x = None
        self.k0 = None
        self.mur = None

    def set_dofs(self, dofs):
        self.x = device_dofs(dofs)

    def set_k0(self, k0):
        self.k0 = float(k0)

    def set_mur_function(self, mur_function):
        """Relative permeability per cell: an array of nt values (the
        reference takes a dolfin Function; None restores 1)."""
        import torch
        if mur_function is None:
            self.mur = None
            return
        mu = np.asarray(mur_function, dtype=np.float64).reshape(-1)
        if len(mu) != self.function_space.nt:
            raise ValueError("mur_function needs one value per cell")
        self.mur = torch.as_tensor(mu, device=_device.device())

    def calc_flux(self):
        """Calculate the power flux"""
        import torch
        if self.x is None or self.k0 is None:
            raise ValueError("set_dofs() and set_k0() first")
        V = self.function_space
        dev = _device.device()
        part = torch.empty(V.nt, dtype=torch.float64, device=dev)
        out = torch.empty(1, dtype=torch.float64, device=dev)
        call("sucem_surface_flux", V.upload(), dtype_code(self.x), ptr(self.x), self.k0,
             ptr(self.mur) if self.mur is not None else None, ptr(part), ptr(out),
             _device.stream_ptr())
        return float(out.item())


class VariationalSurfaceFlux:
    """Power flux by the variational functional (power_flux.py:62-133): the
    EM functional over the cells with an edge on the boundary, with the
    testing function g = j conj(x_D) / (k0 Z0), x_D the DOF vector kept on
    the boundary DOFs only; the flux is its conjugate."""

    def __init__(self, function_space):
        from .PostProcessing import CalcEMFunctional, boundary_edge_cells
        self.function_space = V = function_space
        self.functional = CalcEMFunctional(V)
        self.functional.set_cell_mask(boundary_edge_cells(V))
        self.k0_dirty = True

    def set_dofs(self, dofs):
        import torch
        V = self.function_space
        x = device_dofs(dofs).to(torch.complex128)
        b = torch.as_tensor(V.boundary_dofs.astype(np.int64), device=x.device)
        xd = torch.zeros_like(x)
        xd[b] = x[b]
        self.dirich_dofs = xd
        self.functional.set_E_dofs(x)
        self.k0_dirty = True

    def set_k0(self, k0):
        self.k0 = float(k0)
        self.functional.set_k0(k0)
        self.k0_dirty = True

    def set_epsr_function(self, epsr_function):
        self.functional.set_epsr_function(epsr_function)

    def set_mur_function(self, mur_function):
        self.functional.set_mur_function(mur_function)

    def calc_flux(self):
        from ..Consts import Z0
        if self.k0_dirty:
            self.functional.set_g_dofs(1j * self.dirich_dofs.conj() / self.k0 / Z0)
            self.k0_dirty = False
        return self.functional.calc_functional().conjugate()
