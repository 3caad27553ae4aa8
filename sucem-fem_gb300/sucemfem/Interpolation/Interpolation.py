"""Surface interpolation (sucemfem/Interpolation/Interpolation.py:26-82):
an expression's DOFs on the boundary DOFs of a function space (the
DirichletBC the reference applies), zero elsewhere.  A general Python
interpolant is evaluated on the host at the boundary DOFs' dual-functional
points; plane waves (the NTFF testing functions) have a GPU kernel
(sucem_plane_wave_dofs)."""
import numpy as np

from .. import _native
from .._native import call, ptr

def boundary_dual(function_space):
    """(boundary DOFs, points (nb, 3), tangents (nb, 3)): DOF(u) = u(p) . t."""
    V = function_space
    b = V.boundary_dofs
    pt = np.zeros((len(b), 6), dtype=np.float64)
    call("sucem_space_copy", V._h, _native.COPY["boundary_dual"], ptr(pt))
    return b, pt[:, :3], pt[:, 3:]


class SurfaceInterpolant:
    """Calculate a complex surface interpolant on a 3D domain"""

    def __init__(self, function_space):
        self.function_space = function_space
        self.interpolant = None

    def set_interpolant(self, interpolant):
        """Set interpolant f([x,y,z]) -> [f_x, f_y, f_z] (complex)."""
        self.interpolant = interpolant

    def set_interpolant_expression(self, expr_r, expr_i):
        """Real and imaginary parts as expression objects with
        eval(value, x) (the dolfin.Expression interface)."""
        def f(x):
            vr, vi = np.zeros(3), np.zeros(3)
            expr_r.eval(vr, x)
            expr_i.eval(vi, x)
            return vr + 1j * vi
        self.interpolant = f

    def calculate_interpolation(self):
        V = self.function_space
        b, pts, tans = boundary_dual(V)
        vals = np.array([np.asarray(self.interpolant(p), dtype=np.complex128) for p in pts])
        x = np.zeros(V.n, dtype=np.complex128)
        if len(b):
            x[b] = np.sum(tans * vals.reshape(len(b), 3), axis=1)
        return x
