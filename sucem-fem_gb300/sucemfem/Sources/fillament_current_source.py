"""Line-current filament as N equally spaced point sources
(sucemfem/Sources/fillament_current_source.py:29-82); all N points are
located and evaluated in one GPU call."""
import numpy as np

from .current_source import CurrentSource
from .point_source import evaluate_point_sources


def unit_vector(v):
    v = np.asarray(v, dtype=np.float64)
    return v / np.sqrt(np.sum(v ** 2))


def vector_length(v):
    return np.sqrt(np.sum(np.asarray(v, dtype=np.float64) ** 2))


class FillamentCurrentSource(CurrentSource):
    no_integration_points = 100

    def __init__(self, *names, **kwargs):
        self._dirty = True

    def set_no_integration_points(self, no_integration_points):
        self.no_integration_points = no_integration_points

    def set_source_endpoints(self, source_endpoints):
        self.source_endpoints = np.asarray(source_endpoints, dtype=np.float64)
        self._dirty = True

    def set_value(self, value):
        self.value = value
        self._dirty = True

    def _update(self):
        if self._dirty:
            self.source_start, self.source_end = self.source_endpoints
            self.source_delta = self.source_end - self.source_start
            self.vector_value = unit_vector(self.source_delta) * self.value
            self._dirty = False

    def get_contribution(self):
        self._update()
        source_len = vector_length(self.source_delta)
        no_pts = self.no_integration_points
        if no_pts == 1:
            pts = (self.source_start + self.source_delta * 0.5)[None]
        else:
            pts = self.source_start + self.source_delta * np.linspace(0, 1, no_pts)[:, None]
        mag = self.vector_value * source_len / no_pts
        _, dofs, con = evaluate_point_sources(self.function_space, pts,
                                              np.broadcast_to(mag, (len(pts), 3)))
        contribs = {}
        for dk, ck in zip(dofs, con):
            for dn, v in zip(dk, ck):
                contribs[int(dn)] = contribs.get(int(dn), 0.0) + v
        dofnos = np.array(list(contribs.keys()), dtype=np.uint)
        vals = np.array(list(contribs.values()))
        if not np.iscomplexobj(self.value):
            vals = vals.real.copy()
        return dofnos, vals
