"""Variational near-to-far-field transform (sucemfem/PostProcessing/
variational_ntff.py:31-131): the H-field part by the EM functional over
the cells with an edge on the boundary, tested with plane waves
interpolated onto the boundary DOFs (GPU kernels sucem_plane_wave_dofs and
sucem_em_functional), the E-field part L from the surface transform
(sucem_ntff)."""
import ctypes

import numpy as np

from .. import _device, _native
from .._native import call, ptr
from ..Consts import c0
from .PostProcessing import CalcEMFunctional, _c128, boundary_edge_cells
from .surface_ntff import NTFF as SurfaceNTFF

c_vp = ctypes.c_void_p
_native.declare("sucem_plane_wave_dofs", ctypes.c_int,
                [c_vp, ctypes.c_int, c_vp, c_vp, ctypes.c_double, c_vp, c_vp])


class TransformTestingExpression:
    """1j/k0 rhat x (ahat x rhat) e^{j k0 rhat . r}, as real and imaginary
    expression objects with eval(value, x)."""

    class _Part:
        def __init__(self, owner, imag):
            self.owner, self.imag = owner, imag

        def eval(self, value, x):
            o = self.owner
            ph = o.k0 * np.dot(o.rhat, x)
            value[:] = o.cf * (np.cos(ph) if self.imag else -np.sin(ph))

    def set_parms(self, rhat, ahat, k0):
        self.rhat = np.asarray(rhat, dtype=np.float64)
        self.k0 = float(k0)
        self.cf = np.cross(self.rhat, np.cross(ahat, self.rhat)) / self.k0

    def get_expression(self):
        return self._Part(self, False), self._Part(self, True)


def _unit_vectors(theta_deg, phi_deg):
    th, ph = np.deg2rad(theta_deg), np.deg2rad(phi_deg)
    rhat = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], -1)
    thh = np.stack([np.cos(th) * np.cos(ph), np.cos(th) * np.sin(ph), -np.sin(th)], -1)
    phh = np.stack([-np.sin(ph), np.cos(ph), np.zeros_like(ph)], -1)
    return rhat, thh, phh


class NTFF:
    def __init__(self, function_space, testing_space=None):
        self.function_space = V = function_space
        self.testing_space = V if testing_space is None else testing_space
        self.functional = CalcEMFunctional(V, self.testing_space)
        self.functional.set_cell_mask(boundary_edge_cells(V))
        self.surface = SurfaceNTFF(V)

    def set_k0(self, k0):
        self.k0 = float(k0)
        self.functional.set_k0(k0)

    def set_frequency(self, frequency):
        self.frequency = frequency
        self.surface.set_frequency(frequency)
        self.set_k0(self.frequency * 2 * np.pi / c0)

    def set_dofs(self, dofs):
        self.functional.set_E_dofs(dofs)
        self.surface.set_dofs(dofs)

    def _testing_dofs(self, rhat, ahat):
        """Plane-wave testing DOF vectors, one row per (rhat, ahat) pair."""
        import torch
        V = self.function_space
        dev = _device.device()
        cf = np.cross(rhat, np.cross(ahat, rhat)) / self.k0
        d_r = torch.as_tensor(np.ascontiguousarray(rhat), device=dev)
        d_c = torch.as_tensor(np.ascontiguousarray(cf), device=dev)
        g = torch.zeros(len(rhat) * V.n, dtype=torch.complex128, device=dev)
        call("sucem_plane_wave_dofs", V.upload(), len(rhat), ptr(d_r), ptr(d_c), self.k0, ptr(g),
             _device.stream_ptr())
        return g.view(len(rhat), V.n)

    def calc_pts(self, theta_deg, phi_deg):
        theta_deg = np.atleast_1d(np.asarray(theta_deg, dtype=np.float64))
        phi_deg = np.atleast_1d(np.asarray(phi_deg, dtype=np.float64))
        rhat, thh, phh = _unit_vectors(theta_deg, phi_deg)
        gt = self._testing_dofs(rhat, thh)
        gp = self._testing_dofs(rhat, phh)
        EH = np.zeros((len(rhat), 2), dtype=np.complex128)
        for i in range(len(rhat)):
            for j, g in enumerate((gt, gp)):
                self.functional.set_g_dofs(g[i])
                EH[i, j] = self.functional.calc_functional()
        self.surface.calc_pts(theta_deg, phi_deg)
        L = self.surface._last[:, 2:4]
        r_fac = 1j * self.k0 * np.exp(-1j * self.k0) / (4 * np.pi)
        E_theta = r_fac * (-L[:, 1] + EH[:, 0])
        E_phi = r_fac * (L[:, 0] + EH[:, 1])
        return E_theta, E_phi

    def calc_pt(self, theta_deg, phi_deg):
        Et, Ep = self.calc_pts([theta_deg], [phi_deg])
        return (Et[0], Ep[0])

    def calc_pt_E_H(self, theta_deg, phi_deg):
        rhat, thh, phh = _unit_vectors(np.atleast_1d(theta_deg), np.atleast_1d(phi_deg))
        out = []
        for g in (self._testing_dofs(rhat, thh), self._testing_dofs(rhat, phh)):
            self.functional.set_g_dofs(g[0])
            out.append(self.functional.calc_functional())
        return tuple(out)
