"""Tetrahedral mesh objects standing in for the dolfin ones the reference's
drivers receive (dolfin.Mesh, dolfin.MeshFunction, dolfin.UnitCube,
dolfin.DomainBoundary).  Plain numpy arrays underneath."""
import numpy as np


class Mesh:
    def __init__(self, coordinates, cells):
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

    class _Topology:
        def __init__(self, mesh):
            self._m = mesh

        def dim(self):
            return 3

    def topology(self):
        return Mesh._Topology(self)


class MeshFunction:
    """MeshFunction('uint', mesh, dim): an integer per cell (dim 3) or per
    facet (dim 2, facets in the space's face numbering)."""

    def __init__(self, value_type, mesh, dim, value=0):
        self.mesh = mesh
        self.dim = int(dim)
        if self.dim == 3:
            size = mesh.num_cells()
        elif self.dim == 2:
            size = None  # sized lazily from the facet numbering
        else:
            raise ValueError("only cell (3) and facet (2) mesh functions are supported")
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
