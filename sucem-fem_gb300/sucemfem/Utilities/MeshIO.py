"""``.femmesh`` mesh files (the format of the reference's sandbox sphere
meshes), replacing sucemfem/Utilities/MeshIO.py:38-117.

A file is a sequence of blocks ``BLOCK <name>`` ... ``ENDBLOCK``:

* ``nodes``: a count line, then ``<id> <x> <y> <z>`` per node (ids from 1);
* ``tets``: a count line, then ``<id> <property> <n1> <n2> <n3> <n4>`` per
  tetrahedron (ids and node numbers from 1);
* ``tris``: surface triangles, ignored (as by the reference).

Every id of a block must appear exactly once and a block must end with
``ENDBLOCK``; otherwise reading raises ``ValueError``."""
import os
import re

import numpy as np

from . import MeshConverters


class UninitialisedException(Exception):
    pass


def _uninit_error(fn):
    def check_fn(self):
        if not self.read:
            raise Exception("Call read_meshfile() method of %s first" % self.__class__)
        return fn(self)
    check_fn.__name__ = fn.__name__
    check_fn.__doc__ = fn.__doc__
    return check_fn


class FemmeshReader(object):
    """Reads a ``.femmesh`` file (MeshIO.py:38-110): ``read_meshfile()``,
    then ``get_nodes()`` (nv x 3 float64), ``get_tet_nodes()`` (nt x 4 int32,
    0-based, each row sorted), ``get_tet_property_nos()`` (the property
    number of every tetrahedron; the reference's reader keeps only the last
    one, MeshIO.py:73, an evident slip that is not reproduced) and the file's
    base and directory names."""
    block_start_re = re.compile(r"^BLOCK (.*)")
    read = False

    def __init__(self, mesh_filename):
        self.mesh_filename = mesh_filename
        self.block_parse_funs = dict(nodes=self._parse_nodes, tets=self._parse_tets,
                                     tris=self._skip_block)

    @staticmethod
    def _next(lines, what):
        for line in lines:
            if line.strip():
                return line.split()
        raise ValueError("unexpected end of file in block %s" % what)

    def _end(self, lines, what):
        if self._next(lines, what)[0] != "ENDBLOCK":
            raise ValueError("block %s: ENDBLOCK expected" % what)

    def _parse_nodes(self, lines):
        n = int(self._next(lines, "nodes")[0])
        nodes = np.full((n, 3), np.nan)
        seen = np.zeros(n, dtype=bool)
        for _ in range(n):
            sp = self._next(lines, "nodes")
            i = int(sp[0]) - 1
            if not 0 <= i < n or seen[i]:
                raise ValueError("block nodes: bad or repeated node number %s" % sp[0])
            nodes[i] = [float(x) for x in sp[1:4]]
            seen[i] = True
        self._end(lines, "nodes")
        self.no_nodes, self.nodes = n, nodes

    def _parse_tets(self, lines):
        n = int(self._next(lines, "tets")[0])
        tets = np.zeros((n, 4), dtype=np.int32)
        props = np.zeros(n, dtype=np.int32)
        seen = np.zeros(n, dtype=bool)
        for _ in range(n):
            sp = self._next(lines, "tets")
            i = int(sp[0]) - 1
            if not 0 <= i < n or seen[i]:
                raise ValueError("block tets: bad or repeated tetrahedron number %s" % sp[0])
            props[i] = int(sp[1])
            tets[i] = sorted(int(x) - 1 for x in sp[2:6])
            seen[i] = True
        self._end(lines, "tets")
        self.no_tets, self.tet_nodes, self.tet_property_nos = n, tets, props

    def _skip_block(self, lines):
        for line in lines:
            if line.split()[:1] == ["ENDBLOCK"]:
                return
        raise ValueError("unexpected end of file in a skipped block")

    def read_meshfile(self):
        with open(self.mesh_filename) as fo:
            lines = iter(fo)
            for line in lines:
                m = self.block_start_re.match(line)
                if not m:
                    continue
                name = m.groups()[0].strip()
                if name not in self.block_parse_funs:
                    raise ValueError("unknown block %r" % name)
                self.block_parse_funs[name](lines)
        for attr in ("nodes", "tet_nodes"):
            if not hasattr(self, attr):
                raise ValueError("%s: no %s block" % (self.mesh_filename,
                                                      "nodes" if attr == "nodes" else "tets"))
        if self.no_tets and self.tet_nodes.max() >= self.no_nodes:
            raise ValueError("%s: tetrahedron node number out of range" % self.mesh_filename)
        self.read = True

    @_uninit_error
    def get_mesh_filename(self):
        return os.path.basename(self.mesh_filename)

    @_uninit_error
    def get_mesh_dirname(self):
        return os.path.dirname(self.mesh_filename)

    @_uninit_error
    def get_tet_nodes(self):
        return self.tet_nodes

    @_uninit_error
    def get_tet_property_nos(self):
        return self.tet_property_nos

    @_uninit_error
    def get_nodes(self):
        return self.nodes


def femmesh_2_dolfin_mesh(femmesh_file):
    """A mesh object from a ``.femmesh`` file (MeshIO.py:113-117)."""
    return MeshConverters.femmesh_reader_2_dolfin_mesh(FemmeshReader(femmesh_file))
