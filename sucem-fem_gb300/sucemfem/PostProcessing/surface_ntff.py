"""Surface near-to-far-field transform (sucemfem/PostProcessing/
surface_ntff.py:29-155 ``NTFF``), evaluated on the GPU by sucem_ntff."""
import ctypes

import numpy as np

from .. import _device, _native
from .._native import call, ptr
from ..Consts import c0
from .PostProcessing import device_dofs, dtype_code

c_vp = ctypes.c_void_p
_native.declare("sucem_ntff", ctypes.c_int,
                [c_vp, ctypes.c_int, c_vp, ctypes.c_double, ctypes.c_int, c_vp, c_vp, c_vp, c_vp])


class NTFF:
    """``set_dofs(x)``, ``set_frequency(f)``, then ``calc_pt(theta_deg,
    phi_deg)`` -> (E_theta, E_phi) of the far field normalised to radius 1;
    ``calc_pts`` evaluates many directions in one launch."""

    def __init__(self, function_space):
        self.function_space = function_space
        self.x = None
        self._L = []
        self._N = []
        self._r_fac = []

    def set_dofs(self, dofs):
        self.x = device_dofs(dofs)

    def set_frequency(self, frequency):
        self.frequency = frequency
        self.k0 = self.frequency * 2 * np.pi / c0

    def calc_pts(self, theta_deg, phi_deg):
        """Arrays of directions (degrees) -> (E_theta, E_phi) arrays."""
        import torch
        if self.x is None:
            raise ValueError("set_dofs() first")
        th = np.deg2rad(np.atleast_1d(np.asarray(theta_deg, dtype=np.float64)))
        ph = np.deg2rad(np.atleast_1d(np.asarray(phi_deg, dtype=np.float64)))
        if th.shape != ph.shape:
            raise ValueError("theta and phi need the same length")
        dev = _device.device()
        d_th = torch.as_tensor(th, device=dev)
        d_ph = torch.as_tensor(ph, device=dev)
        out = torch.empty(len(th) * 12, dtype=torch.float64, device=dev)
        call("sucem_ntff", self.function_space.upload(), dtype_code(self.x), ptr(self.x),
             float(self.k0), len(th), ptr(d_th), ptr(d_ph), ptr(out), _device.stream_ptr())
        o = out.cpu().numpy().reshape(len(th), 6, 2)
        z = o[..., 0] + 1j * o[..., 1]
        self._last = z
        return z[:, 0], z[:, 1]

    def calc_pt(self, theta_deg, phi_deg):
        E_theta, E_phi = self.calc_pts([theta_deg], [phi_deg])
        z = self._last[0]
        self._L.append([z[2], z[3]])
        self._N.append([z[4], z[5]])
        self._r_fac.append(1j * self.k0 * np.exp(-1j * self.k0) / (4 * np.pi))
        return (E_theta[0], E_phi[0])
