"""Mesh generators (sucemfem/Utilities/MeshGenerators.py:26-53)."""
import numpy as np

from ..mesh import Mesh, UnitCube


def get_centred_cube(domain_size, max_edge_len, centred_element_coordinate=None):
    """Cube mesh centred around the origin: ceil(sqrt(2) * domain_size /
    max_edge_len) subdivisions per axis of the six-tet unit cube, scaled to
    domain_size (a number or one value per axis).

    With ``centred_element_coordinate`` the mesh is translated so that this
    point is the centroid of a cell: among the cells whose closure contains
    the point, the one whose centroid is nearest (lowest index on ties)."""
    ds = np.broadcast_to(np.asarray(domain_size, dtype=np.float64), (3,))
    n = np.array(np.ceil(np.sqrt(2) * ds / max_edge_len), dtype=np.int64)
    m = UnitCube(*[int(v) for v in n])
    x = m.coordinates() * ds - ds / 2
    cells = m.cells()
    if centred_element_coordinate is not None:
        p = np.asarray(centred_element_coordinate, dtype=np.float64)
        v = x[cells]                                  # (nt, 4, 3)
        T = np.stack([v[:, 1] - v[:, 0], v[:, 2] - v[:, 0], v[:, 3] - v[:, 0]], axis=2)
        lam = np.linalg.solve(T, (p - v[:, 0])[..., None])[..., 0]
        bary = np.concatenate([1 - lam.sum(1, keepdims=True), lam], axis=1)
        cand = np.nonzero(np.all(bary >= -1e-12, axis=1))[0]
        if len(cand) == 0:
            raise ValueError("centred_element_coordinate lies outside the mesh")
        mid = v[cand].mean(1)
        best = cand[int(np.argmin(np.linalg.norm(mid - p, axis=1)))]
        x = x - v[best].mean(0)
    return Mesh(x, cells)
