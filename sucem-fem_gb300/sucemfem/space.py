"""N1curl function space backed by the native builder.

Mirrors what the reference takes from ``dolfin.FunctionSpace(mesh,
"Nedelec 1st kind H(curl)", order)`` (sucemfem/ProblemConfigurations/
EMProblem.py:100-105): the DOF map with DOLFIN's numbering, the global
dimension and the sparsity pattern of dolfin.assemble.
"""
import ctypes

import numpy as np

from . import _native
from ._native import call, ptr

ELEMENT_FAMILY = "Nedelec 1st kind H(curl)"


class DofMap:
    def __init__(self, space):
        self._space = space

    def global_dimension(self):
        return self._space.n

    def max_cell_dimension(self):
        return self._space.ndof_cell

    def cell_dofs(self, cell_index):
        return self._space.cell_dofs[cell_index].copy()

    def tabulate_dofs(self, dofnos, cell):
        dofnos[:] = self._space.cell_dofs[int(cell)]


class FunctionSpace:
    """``FunctionSpace(mesh, family, order)`` for the N1curl family."""

    def __init__(self, mesh, family=ELEMENT_FAMILY, order=1):
        if family not in (ELEMENT_FAMILY, "N1curl"):
            raise ValueError("only the %r family is provided" % ELEMENT_FAMILY)
        if order not in (1, 2, 3, 4):
            raise ValueError("basis order must be 1, 2, 3 or 4")
        self._mesh = mesh
        self.order = k = int(order)
        self.ndof_cell = k * (k + 2) * (k + 3) // 2
        # DOFs per edge, per face and per cell interior
        self.dofs_edge, self.dofs_face, self.dofs_cell = k, k * (k - 1), k * (k - 1) * (k - 2) // 2
        coords = np.ascontiguousarray(mesh.coordinates(), dtype=np.float64)
        cells = np.ascontiguousarray(mesh.cells(), dtype=np.int64)
        h = ctypes.c_void_p()
        call("sucem_space_create", ptr(coords), len(coords), ptr(cells), len(cells), self.order,
             ctypes.byref(h))
        self._h = h
        sizes = np.zeros(10, dtype=np.int64)
        call("sucem_space_sizes", self._h, sizes.ctypes.data_as(_native.c_i64p))
        (self.n, self.nnz, self.nv, self.nt, self.ne, self.nf, self.n_ext_facets,
         self.n_boundary, self.max_row, self.n_incidences) = [int(x) for x in sizes]
        self._cache = {}
        self._uploaded = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _native._lib is not None:
            _native._lib.sucem_space_destroy(h)
            self._h = None

    # -- host copies -------------------------------------------------------
    def _copy(self, what, shape, dtype):
        key = ("h", what)
        if key not in self._cache:
            a = np.empty(shape, dtype=dtype)
            if a.size:
                call("sucem_space_copy", self._h, _native.COPY[what], ptr(a))
            self._cache[key] = a
        return self._cache[key]

    @property
    def indptr(self):
        return self._copy("indptr", self.n + 1, np.int64)

    @property
    def indices(self):
        return self._copy("indices", self.nnz, np.int32)

    @property
    def cell_dofs(self):
        return self._copy("cell_dofs", (self.nt, self.ndof_cell), np.int32)

    @property
    def boundary_dofs(self):
        return self._copy("boundary_dofs", self.n_boundary, np.int32)

    @property
    def cells(self):
        return self._copy("cells", (self.nt, 4), np.int32)

    @property
    def ext_mask(self):
        return self._copy("ext_mask", self.nt, np.uint8)

    @property
    def dof_xyz(self):
        return self._copy("dof_xyz", (self.n, 3), np.float64)

    @property
    def cell_edges(self):
        return self._copy("cell_edges", (self.nt, 6), np.int32)

    @property
    def cell_faces(self):
        return self._copy("cell_faces", (self.nt, 4), np.int32)

    def assembly_schedule(self):
        """The order-1/2 assembly kernel's work plan (host copy): per warp
        task the entity of each lane, (first step block, steps per local
        entity index, flags), and the step blocks (cells, then column-slot
        words, 32 lanes each)."""
        sz = np.zeros(4, dtype=np.int64)
        call("sucem_space_schedule_sizes", self._h, sz.ctypes.data_as(_native.c_i64p))
        nt_, nint, nblk, planes = [int(x) for x in sz]
        ent = self._copy("task_ent", (nt_, 32), np.int32)
        meta = self._copy("task_meta", (nt_, 4), np.int32)
        words = self._copy("step_words", (nblk, 1 + planes, 32), np.uint32)
        return dict(n_tasks_interior=nint, task_ent=ent, task_meta=meta, step_words=words)

    def entry_lists(self):
        """The order-3/4 assembly kernel's gather lists (host copy): CSR
        entry q sums the cell entries src[ptr[q]:ptr[q+1]], each coded
        (c * ndof_cell + a) * ndof_cell + b, in ascending cell order; perm[t]
        is the CSR entry of kernel thread t (each row's entries ordered by
        list length)."""
        if self.order < 3:
            raise ValueError("entry lists exist for basis orders 3 and 4 only")
        ptr = self._copy("entry_ptr", self.nnz + 1, np.int32)
        src = self._copy("entry_src", self.nt * self.ndof_cell ** 2, np.int32)
        perm = self._copy("entry_perm", self.nnz, np.int32)
        return ptr, src, perm

    def facet_closure_dofs(self, faces):
        """DOFs on the closure of the given facets (facet ids = face ids)."""
        faces = np.asarray(faces, dtype=np.int64)
        if faces.size == 0:
            return np.zeros(0, dtype=np.int32)
        cf = self.cell_faces
        mark = np.zeros(self.nf, dtype=bool)
        mark[faces] = True
        c, lf = np.nonzero(mark[cf])
        # local edges of local face lf are those not touching local vertex lf
        edge_verts = np.array([(2, 3), (1, 3), (1, 2), (0, 3), (0, 2), (0, 1)])
        on_face = (edge_verts[None, :, 0] != lf[:, None]) & (edge_verts[None, :, 1] != lf[:, None])
        edges = np.unique(self.cell_edges[c][on_face]).astype(np.int64)
        fids = np.unique(cf[c, lf]).astype(np.int64)
        de, df = self.dofs_edge, self.dofs_face
        parts = [de * edges + j for j in range(de)]
        parts += [de * self.ne + df * fids + j for j in range(df)]
        return np.sort(np.concatenate(parts)).astype(np.int32)

    def mesh(self):
        return self._mesh

    def dofmap(self):
        return DofMap(self)

    def dim(self):
        return self.n

    # -- device ------------------------------------------------------------
    def upload(self):
        from . import _device
        dev = _device.device()
        if self._uploaded != dev.index:
            call("sucem_space_upload", self._h, dev.index)
            self._uploaded = dev.index
        return self._h

    def device_ptr(self, what):
        self.upload()
        out = ctypes.c_void_p()
        call("sucem_space_device_ptr", self._h, _native.DEV[what], ctypes.byref(out))
        return out.value
