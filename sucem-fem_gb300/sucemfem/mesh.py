"""Tetrahedral mesh objects standing in for the dolfin ones the reference's
drivers receive (dolfin.Mesh, dolfin.MeshFunction, dolfin.UnitCube,
dolfin.DomainBoundary).  Plain numpy arrays underneath.  ``Mesh(filename)``
and ``MeshFunction(type, mesh, filename)`` read DOLFIN XML files (the
format of the reference's meshes and facet/physical-region functions)."""
import xml.etree.ElementTree as ET

import numpy as np


def _tag(e):
    return e.tag.rsplit("}", 1)[-1]


def _child(e, name):
    for c in e:
        if _tag(c) == name:
            return c
    return None


def read_dolfin_xml_mesh(filename):
    """(coordinates (nv, 3), cells (nt, 4)) of a DOLFIN XML tetrahedral mesh
    (``<dolfin><mesh celltype="tetrahedron" dim="3"><vertices>...
    <cells><tetrahedron index v0 v1 v2 v3/>``)."""
    root = ET.parse(filename).getroot()
    mesh = root if _tag(root) == "mesh" else _child(root, "mesh")
    if mesh is None:
        raise ValueError("%s: no <mesh> element" % filename)
    if mesh.get("celltype", "tetrahedron") != "tetrahedron" or int(mesh.get("dim", 3)) != 3:
        raise ValueError("%s: only 3-D tetrahedral meshes are supported" % filename)
    verts, cells = _child(mesh, "vertices"), _child(mesh, "cells")
    if verts is None or cells is None:
        raise ValueError("%s: <vertices> and <cells> are required" % filename)
    nv = int(verts.get("size", len(verts)))
    x = np.full((nv, 3), np.nan)
    for v in verts:
        i = int(v.get("index"))
        x[i] = [float(v.get("x")), float(v.get("y", 0.0)), float(v.get("z", 0.0))]
    nt = int(cells.get("size", len(cells)))
    c = np.full((nt, 4), -1, dtype=np.int64)
    for t in cells:
        if _tag(t) != "tetrahedron":
            raise ValueError("%s: cell type %s is not a tetrahedron" % (filename, _tag(t)))
        c[int(t.get("index"))] = [int(t.get("v%d" % k)) for k in range(4)]
    if np.isnan(x).any() or (c < 0).any() or c.max() >= nv:
        raise ValueError("%s: incomplete vertex or cell list" % filename)
    return x, c


def read_dolfin_xml_meshfunction(filename):
    """(dim, values) of a DOLFIN XML mesh function (``<meshfunction
    type="uint" dim=".." size=".."><entity index value/>``)."""
    root = ET.parse(filename).getroot()
    if _tag(root) in ("meshfunction", "mesh_function"):
        mf = root
    else:
        mf = _child(root, "meshfunction")
        if mf is None:
            mf = _child(root, "mesh_function")
    if mf is None:
        raise ValueError("%s: no <meshfunction> element" % filename)
    size = int(mf.get("size"))
    vals = np.zeros(size, dtype=np.int64)
    seen = np.zeros(size, dtype=bool)
    for e in mf:
        i = int(e.get("index"))
        vals[i] = int(e.get("value"))
        seen[i] = True
    if not seen.all():
        raise ValueError("%s: %d entities without a value" % (filename, int((~seen).sum())))
    return int(mf.get("dim")), vals


class Mesh:
    def __init__(self, coordinates, cells=None):
        if cells is None:
            if not isinstance(coordinates, str):
                raise ValueError("Mesh(filename) or Mesh(coordinates, cells)")
            coordinates, cells = read_dolfin_xml_mesh(coordinates)
        self._x = np.ascontiguousarray(coordinates, dtype=np.float64)
        c = np.asarray(cells, dtype=np.int64)
        if c.ndim != 2 or c.shape[1] != 4 or self._x.ndim != 2 or self._x.shape[1] != 3:
            raise ValueError("expected coordinates (nv,3) and tetrahedra (nt,4)")
        # DOLFIN orders every cell's vertices by global index
        self._c = np.ascontiguousarray(np.sort(c, axis=1))

    def coordinates(self):
        return self._x

    def cells(self):
        return self._c

    def num_cells(self):
        return len(self._c)

    def num_vertices(self):
        return len(self._x)

    def topology_space(self):
        """The order-1 function space of this mesh, built once: its edges
        and faces carry DOLFIN's edge and facet numbering."""
        if getattr(self, "_space1", None) is None:
            from .space import FunctionSpace
            self._space1 = FunctionSpace(self, order=1)
        return self._space1

    def num_edges(self):
        return self.topology_space().ne

    def num_faces(self):
        return self.topology_space().nf

    num_facets = num_faces

    class _Topology:
        def __init__(self, mesh):
            self._m = mesh

        def dim(self):
            return 3

    def topology(self):
        return Mesh._Topology(self)


class MeshFunction:
    """MeshFunction('uint', mesh, dim): an integer per cell (dim 3), per
    facet (dim 2, facets in the space's face numbering), per edge (dim 1,
    the space's edge numbering) or per vertex (dim 0)."""

    def __init__(self, value_type, mesh, dim, value=0):
        self.mesh = mesh
        if isinstance(dim, str):
            # MeshFunction(type, mesh, filename): DOLFIN XML; facet (dim 2)
            # indices follow DOLFIN's facet numbering, which the space's
            # face numbering reproduces
            fdim, vals = read_dolfin_xml_meshfunction(dim)
            self.dim = fdim
            if fdim == 3 and len(vals) != mesh.num_cells():
                raise ValueError("cell function size %d != %d cells" % (len(vals), mesh.num_cells()))
            if fdim not in (2, 3):
                raise ValueError("only cell (3) and facet (2) mesh functions are supported")
            self._a = vals
            self._fill = value
            return
        self.dim = int(dim)
        if self.dim == 3:
            size = mesh.num_cells()
        elif self.dim == 2:
            size = None  # sized lazily from the facet numbering
        elif self.dim == 1:
            size = mesh.num_edges()
        elif self.dim == 0:
            size = mesh.num_vertices()
        else:
            raise ValueError("mesh function dimension must be 0, 1, 2 or 3")
        self._a = None if size is None else np.full(size, value, dtype=np.int64)
        self._fill = value

    def _ensure(self, size):
        if self._a is None:
            self._a = np.full(size, self._fill, dtype=np.int64)

    def set_all(self, value):
        self._fill = value
        if self._a is not None:
            self._a[:] = value

    def array(self):
        return self._a

    def __getitem__(self, i):
        return self._a[i]

    def __setitem__(self, i, v):
        self._a[i] = v


def VertexFunction(value_type, mesh, value=0):
    return MeshFunction(value_type, mesh, 0, value)


def EdgeFunction(value_type, mesh, value=0):
    return MeshFunction(value_type, mesh, 1, value)


def FaceFunction(value_type, mesh, value=0):
    return MeshFunction(value_type, mesh, 2, value)


FacetFunction = FaceFunction


def CellFunction(value_type, mesh, value=0):
    return MeshFunction(value_type, mesh, 3, value)


class DomainBoundary:
    """Marks every exterior facet (dolfin.DomainBoundary().mark)."""

    def mark(self, facet_function, value):
        facet_function.boundary_value = value
        facet_function.mark_all_exterior = True


def UnitCube(nx, ny, nz):
    """dolfin.UnitCube(nx, ny, nz): x-fastest vertex numbering, six tets per
    cube sharing the cube's v0-v7 diagonal."""
    nx, ny, nz = int(nx), int(ny), int(nz)
    i = np.arange(nx + 1) / float(nx)
    j = np.arange(ny + 1) / float(ny)
    k = np.arange(nz + 1) / float(nz)
    Z, Y, X = np.meshgrid(k, j, i, indexing="ij")
    coords = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    ii, jj, kk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    v0 = (kk * (nx + 1) * (ny + 1) + jj * (nx + 1) + ii).transpose(2, 1, 0).ravel()
    sx, sy = 1, nx + 1
    sz = (nx + 1) * (ny + 1)
    v1, v2 = v0 + sx, v0 + sy
    v3, v4 = v1 + sy, v0 + sz
    v5, v6, v7 = v1 + sz, v2 + sz, v3 + sz
    cells = np.stack([np.stack(t, axis=1) for t in
                      [(v0, v1, v3, v7), (v0, v1, v7, v5), (v0, v5, v7, v4),
                       (v0, v3, v2, v7), (v0, v6, v4, v7), (v0, v2, v6, v7)]], axis=1)
    return Mesh(coords, cells.reshape(-1, 4))


def BoxMesh(lx, ly, lz, nx, ny, nz, origin=(0.0, 0.0, 0.0)):
    m = UnitCube(nx, ny, nz)
    x = m.coordinates() * np.array([lx, ly, lz], dtype=np.float64) + np.asarray(origin, dtype=np.float64)
    return Mesh(x, m.cells())
