"""Mesh conversions of sucemfem/Utilities/MeshConverters.py:22-68 on the
package's numpy-backed mesh object (the stand-in for dolfin.Mesh): a
"listmesh" is a dict with the vertex coordinates under 'Nodes' and the
tetrahedra under 'ElementNodes'."""
import numpy as np

from ..mesh import Mesh


def listmesh_2_dolfin_mesh(listmesh, reorder=False):
    """Mesh from listmesh['Nodes'] and listmesh['ElementNodes'].  The mesh
    object always keeps every cell's vertices sorted by global index (what
    DOLFIN's ``order()`` does for ``reorder=True``), so ``reorder`` has no
    further effect."""
    return Mesh(np.asarray(listmesh["Nodes"], dtype=np.float64),
                np.asarray(listmesh["ElementNodes"], dtype=np.int64))


def dolfin_mesh_2_listmesh(dolfin_mesh):
    """{'Nodes': coordinates copy, 'ElementNodes': int32 cells copy}."""
    return {"Nodes": dolfin_mesh.coordinates().copy(),
            "ElementNodes": np.array(dolfin_mesh.cells(), dtype=np.int32, copy=True)}


def femmesh_reader_2_dolfin_mesh(femmesh_reader, reorder=True):
    """Mesh from a MeshIO.FemmeshReader (read first if needed)."""
    if not femmesh_reader.read:
        femmesh_reader.read_meshfile()
    listmesh = dict(FemmeshFilename=femmesh_reader.get_mesh_filename(),
                    FemmeshDir=femmesh_reader.get_mesh_dirname(),
                    Nodes=femmesh_reader.get_nodes(),
                    ElementNodes=femmesh_reader.get_tet_nodes())
    return listmesh_2_dolfin_mesh(listmesh, reorder=reorder)
