"""``.femmesh`` reading (sucemfem/Utilities/MeshIO.py:38-117) and the mesh
converters (sucemfem/Utilities/MeshConverters.py:22-68) on the CPU."""
import os

import numpy as np
import pytest

from oracle import fem


def _write_femmesh(path, coords, cells, props, tris=None, seed=0):
    """A .femmesh file with the records of every block in a shuffled order
    and the nodes of every tetrahedron permuted (ids stay 1-based)."""
    rng = np.random.default_rng(seed)
    lines = ["BLOCK nodes", str(len(coords))]
    for i in rng.permutation(len(coords)):
        lines.append("%d %r %r %r" % (i + 1, *map(float, coords[i])))
    lines.append("ENDBLOCK")
    if tris is not None:
        lines += ["BLOCK tris", str(len(tris))]
        lines += ["%d 0 %d %d %d" % (i + 1, *(t + 1)) for i, t in enumerate(tris)]
        lines.append("ENDBLOCK")
    lines += ["BLOCK tets", str(len(cells))]
    for i in rng.permutation(len(cells)):
        lines.append("%d %d %d %d %d %d" % (i + 1, props[i], *(rng.permutation(cells[i]) + 1)))
    lines.append("ENDBLOCK")
    path.write_text("\n".join(lines) + "\n")


def _box(tmp_path):
    coords, cells = fem.box_mesh(1.0, 0.5, 0.75, 3, 2, 2)
    props = np.arange(len(cells)) % 3 + 1
    topo = fem.Topology(np.sort(cells, axis=1))
    tris = topo.faces[topo.exterior_faces()]
    p = tmp_path / "box.femmesh"
    _write_femmesh(p, coords, cells, props, tris)
    return p, coords, cells, props


def test_femmesh_reader_matches_the_written_mesh(tmp_path):
    from sucemfem.Utilities.MeshIO import FemmeshReader
    p, coords, cells, props = _box(tmp_path)
    r = FemmeshReader(str(p))
    with pytest.raises(Exception, match="read_meshfile"):
        r.get_nodes()
    r.read_meshfile()
    assert np.array_equal(r.get_nodes(), coords)
    assert r.get_tet_nodes().dtype == np.int32
    assert np.array_equal(r.get_tet_nodes(), np.sort(cells, axis=1))
    assert np.array_equal(r.get_tet_property_nos(), props)
    assert r.get_mesh_filename() == "box.femmesh"
    assert r.get_mesh_dirname() == str(tmp_path)


def test_femmesh_to_mesh_and_space(tmp_path):
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    from sucemfem.Utilities.MeshConverters import dolfin_mesh_2_listmesh, listmesh_2_dolfin_mesh
    from sucemfem.Utilities.MeshIO import femmesh_2_dolfin_mesh
    p, coords, cells, _ = _box(tmp_path)
    m = femmesh_2_dolfin_mesh(str(p))
    ref = Mesh(coords, cells)
    assert np.array_equal(m.coordinates(), ref.coordinates())
    assert np.array_equal(m.cells(), ref.cells())
    V, W = FunctionSpace(m, order=2), FunctionSpace(ref, order=2)
    assert (V.n, V.nnz) == (W.n, W.nnz)
    assert np.array_equal(V.cell_dofs, W.cell_dofs)
    lm = dolfin_mesh_2_listmesh(m)
    assert lm["ElementNodes"].dtype == np.int32
    m2 = listmesh_2_dolfin_mesh(lm, reorder=True)
    assert np.array_equal(m2.cells(), m.cells())


@pytest.mark.parametrize("bad", ["no_end", "repeat", "range", "unknown"])
def test_femmesh_reader_rejects_bad_files(tmp_path, bad):
    from sucemfem.Utilities.MeshIO import FemmeshReader
    body = {
        "no_end": "BLOCK nodes\n2\n1 0 0 0\n2 1 0 0\n",
        "repeat": "BLOCK nodes\n2\n1 0 0 0\n1 1 0 0\nENDBLOCK\n",
        "range": ("BLOCK nodes\n4\n1 0 0 0\n2 1 0 0\n3 0 1 0\n4 0 0 1\nENDBLOCK\n"
                  "BLOCK tets\n1\n1 1 1 2 3 9\nENDBLOCK\n"),
        "unknown": "BLOCK hexes\n0\nENDBLOCK\n",
    }[bad]
    p = tmp_path / "bad.femmesh"
    p.write_text(body)
    with pytest.raises(ValueError):
        FemmeshReader(str(p)).read_meshfile()


# the reference checkout is optional test data: point SUCEM_REFERENCE_ROOT
# at it to run this case
_REF = os.environ.get("SUCEM_REFERENCE_ROOT", "")
SANDBOX = os.path.join(_REF, "sandbox/solvers/meshes/sphere-r1m-4.femmesh") if _REF else ""


@pytest.mark.skipif(not SANDBOX or not os.path.exists(SANDBOX),
                    reason="SUCEM_REFERENCE_ROOT not set or its sandbox meshes not present")
def test_reference_sandbox_sphere_mesh():
    """One of the reference's own sphere meshes (read in place, not copied):
    block counts as declared (242 nodes, 659 tetrahedra), nodes on or inside
    the unit sphere, no degenerate tetrahedron, the volume close to that of
    the unit sphere."""
    from sucemfem.Utilities.MeshIO import FemmeshReader
    r = FemmeshReader(SANDBOX)
    r.read_meshfile()
    x, t = r.get_nodes(), r.get_tet_nodes()
    assert x.shape == (242, 3) and t.shape == (659, 4)
    assert np.linalg.norm(x, axis=1).max() < 1 + 1e-9
    e = x[t[:, 1:]] - x[t[:, :1]]
    vol = np.abs(np.linalg.det(e)) / 6
    assert vol.min() > 0
    assert abs(vol.sum() - 4 / 3 * np.pi) < 0.1 * 4 / 3 * np.pi
