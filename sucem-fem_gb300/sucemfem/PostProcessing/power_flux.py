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
