"""Boundary edges and the cells attached to them (sucemfem/Geometry.py:
24-106) on the package's mesh objects.  Edge and facet numbers are those of
the mesh's order-1 function space (DOLFIN's numbering); the connectivity is
computed on demand, so ``EnsureInitialised`` has nothing to do."""
import numpy as np

from .mesh import DomainBoundary, EdgeFunction, FaceFunction

# UFC local edges of a tetrahedron (vertex pairs)
_EDGE_VERTS = np.array([(2, 3), (1, 3), (1, 2), (0, 3), (0, 2), (0, 1)])


def _mesh_of(meshfun):
    m = meshfun.mesh
    return m() if callable(m) else m


def _marked_faces(space, facefun, value):
    """Facet numbers whose facet-function value is ``value``."""
    if getattr(facefun, "mark_all_exterior", False) and facefun.boundary_value == value:
        c, lf = np.nonzero(space.ext_mask[:, None] >> np.arange(4)[None, :] & 1)
        return np.unique(space.cell_faces[c, lf])
    facefun._ensure(space.nf)
    return np.nonzero(np.asarray(facefun.array()) == value)[0]


class EnsureInitialised(object):
    """Kept for the reference's call sites: connectivity is always there."""

    def __init__(self, dolfin_mesh):
        self.dolfin_mesh = dolfin_mesh

    def __call__(self, dim0, dim1):
        return None


class BoundaryEdges(object):
    """Marks the edges of a set of faces: those where ``boundary_facefun``
    equals ``boundary_value`` (default: every exterior facet)."""

    def __init__(self, mesh, boundary_facefun=None, boundary_value=1):
        self.mesh = mesh
        if boundary_facefun is None:
            boundary_facefun = FaceFunction("uint", mesh)
            boundary_facefun.set_all(0)
            DomainBoundary().mark(boundary_facefun, boundary_value)
        self.boundary_facefun = boundary_facefun
        self.boundary_value = boundary_value
        self.ensure_initialised = EnsureInitialised(mesh)

    def mark(self, edge_meshfun, value):
        V = self.mesh.topology_space()
        mark = np.zeros(V.nf, dtype=bool)
        mark[_marked_faces(V, self.boundary_facefun, self.boundary_value)] = True
        c, lf = np.nonzero(mark[V.cell_faces])
        # the edges of local face lf are the local edges not touching vertex lf
        on = (_EDGE_VERTS[None, :, 0] != lf[:, None]) & (_EDGE_VERTS[None, :, 1] != lf[:, None])
        edge_meshfun.array()[np.unique(V.cell_edges[c][on])] = value


class CellsConnected2Edges(object):
    """Marks the cells that hold an edge where ``boundary_edgefun`` equals
    ``boundary_value``."""

    def __init__(self, boundary_edgefun, boundary_value):
        self.boundary_edgefun = boundary_edgefun
        self.boundary_value = boundary_value
        self.mesh = _mesh_of(boundary_edgefun)
        self.ensure_initialised = EnsureInitialised(self.mesh)

    def mark(self, cell_meshfun, value):
        V = self.mesh.topology_space()
        hit = np.asarray(self.boundary_edgefun.array()) == self.boundary_value
        cells = np.nonzero(hit[V.cell_edges].any(axis=1))[0]
        cell_meshfun.array()[cells] = value


class BoundaryEdgeCells(object):
    """Marks the cells connected to the domain boundary through an edge."""

    def __init__(self, mesh):
        self.edge_boundary_value = 1
        edgefun = EdgeFunction("uint", mesh)
        edgefun.set_all(0)
        BoundaryEdges(mesh).mark(edgefun, self.edge_boundary_value)
        self.boundary_edgefun = edgefun

    def mark(self, cell_meshfun, value):
        CellsConnected2Edges(self.boundary_edgefun, self.edge_boundary_value).mark(cell_meshfun,
                                                                                 value)
