"""Point current source (sucemfem/Sources/point_source.py:28-94) with the
point location and basis evaluation done on the GPU (sucem_point_sources).
Cell rule for points on shared faces/edges/vertices: lowest cell index."""
import numpy as N
import torch

from .. import _device
from .._native import call, ptr
from .current_source import CurrentSource

NOT_FOUND = 0x7F7F7F7F


def evaluate_point_sources(V, points, values):
    """For each point p_k with current vector J_k: (cell_k, dofnos (k, ndof),
    contributions (k, ndof) complex128) with contribution N_i(p_k) . J_k."""
    pts = N.ascontiguousarray(N.atleast_2d(points), dtype=N.float64)
    vals = N.ascontiguousarray(N.atleast_2d(values), dtype=N.complex128)
    npts = len(pts)
    if vals.shape != (npts, 3):
        raise ValueError("values must have shape (npts, 3)")
    d_pts = _device.to_dev(pts)
    d_vals = _device.to_dev(vals.view(N.float64).reshape(-1))
    d_cells = torch.empty(npts, dtype=torch.int32, device=_device.device())
    d_con = torch.empty(npts * V.ndof_cell * 2, dtype=torch.float64, device=_device.device())
    call("sucem_point_sources", V.upload(), ptr(d_pts), ptr(d_vals), npts, ptr(d_cells),
         ptr(d_con), _device.stream_ptr())
    cells = d_cells.cpu().numpy()
    if N.any(cells == NOT_FOUND):
        bad = pts[cells == NOT_FOUND][0]
        raise ValueError("source point %r is outside the mesh" % (bad.tolist(),))
    con = d_con.cpu().numpy().view(N.complex128).reshape(npts, V.ndof_cell)
    return cells, V.cell_dofs[cells], con


def calc_pointsource_contrib(V, source_coords, source_value):
    """(dofnos, rhs_contribs): RHS[dofnos] += rhs_contribs adds the source."""
    source_value = N.asarray(source_value)
    _, dofs, con = evaluate_point_sources(V, N.asarray(source_coords, N.float64)[None],
                                          N.asarray(source_value)[None])
    contribs = con[0]
    if not N.any(N.iscomplex(source_value)):
        contribs = contribs.real.copy()
    return dofs[0].astype(N.uintc), contribs


class PointCurrentSource(CurrentSource):
    def set_position(self, position):
        self.position = N.array(position, dtype=N.float64)

    def set_value(self, value):
        iscomplex = N.any(N.iscomplex(value))
        self.value = N.array(value, dtype=N.complex128 if iscomplex else N.float64)

    def get_contribution(self):
        return calc_pointsource_contrib(self.function_space, self.position, self.value)
