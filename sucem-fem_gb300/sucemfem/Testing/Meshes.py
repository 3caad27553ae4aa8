"""Test meshes of sucemfem/Testing/Meshes.py:25-61: ``InscribedTet``, a
tetrahedron inscribed in the cube [-1/2, 1/2]^3 with an inner tetrahedron,
split into 11 cells (every cell but the last touches the boundary through
an edge).  The vertex and cell tables are those of the reference."""
import numpy as np

from ..mesh import Mesh


class InscribedTet(object):
    def __init__(self):
        h, s = 0.5, 1.0 / 6
        self.coordinates = np.array(
            [[-h, h, -h], [h, h, h], [h, -h, -h], [-h, -h, h],
             [s, s, -s], [-s, s, s], [-s, -s, -s], [s, -s, s]], dtype=np.float64)
        self.element_nodes = np.array(
            [[1, 4, 6, 7], [1, 3, 5, 7], [3, 4, 7, 8], [1, 2, 5, 6], [2, 3, 5, 8],
             [2, 4, 6, 8], [4, 6, 7, 8], [1, 5, 6, 7], [3, 5, 7, 8], [2, 5, 6, 8],
             [5, 6, 7, 8]], dtype=np.uint32) - 1

    def get_dolfin_mesh(self):
        return Mesh(self.coordinates, self.element_nodes.astype(np.int64))
