"""CPU checks of the post-processing path: the oracle's surface power flux
pinned to the reference's golden (test_power_flux.py:54, SurfaceFlux on the
test's own DOLFIN XML mesh), and the DOLFIN XML mesh / mesh-function
readers against an independent parse and the oracle's facet numbering."""
import os
import xml.etree.ElementTree as ET

import numpy as np

from conftest import golden
from oracle import fem, postproc


def _parse(text):
    """Independent minimal parse of a DOLFIN XML mesh (tests only)."""
    root = ET.fromstring(text)
    verts = [e for e in root.iter() if e.tag.rsplit("}", 1)[-1] == "vertex"]
    tets = [e for e in root.iter() if e.tag.rsplit("}", 1)[-1] == "tetrahedron"]
    x = np.zeros((len(verts), 3))
    for v in verts:
        x[int(v.get("index"))] = [float(v.get(a)) for a in "xyz"]
    c = np.zeros((len(tets), 4), dtype=np.int64)
    for t in tets:
        c[int(t.get("index"))] = [int(t.get("v%d" % k)) for k in range(4)]
    return x, np.sort(c, axis=1)


def _write(tmp_path, name, text):
    p = os.path.join(str(tmp_path), name)
    with open(p, "w") as f:
        f.write(str(text))
    return p


def test_surface_flux_oracle_matches_reference_golden():
    g = golden("power_flux_solution_o2.npz")
    coords, cells = _parse(str(g["mesh_xml"]))
    A = fem.assemble(coords, cells, 2)
    k0 = 2 * np.pi * float(g["freq"]) / fem.C0
    v = postproc.surface_flux(coords, cells, 2, A.topo, A.dofmap, g["x"], k0)
    # the reference test: assertAlmostEqual(calc_flux(), 26.3586862457), 7 places
    assert abs(v - float(g["flux_surface"])) < 5e-8, v


def test_surface_flux_oracle_quadrature_converged():
    """The 3x3 rule is exact for the degree-3 integrand: a 6x6 rule agrees."""
    from oracle import n1curl_exact
    g = golden("power_flux_solution_o2.npz")
    coords, cells = _parse(str(g["mesh_xml"]))
    A = fem.assemble(coords, cells, 2)
    k0 = 2 * np.pi * float(g["freq"]) / fem.C0
    v3 = postproc.surface_flux(coords, cells, 2, A.topo, A.dofmap, g["x"], k0)
    orig = n1curl_exact._gauss_tri
    try:
        n1curl_exact._gauss_tri = lambda npts=6: orig(6)
        v6 = postproc.surface_flux(coords, cells, 2, A.topo, A.dofmap, g["x"], k0)
    finally:
        n1curl_exact._gauss_tri = orig
    assert abs(v3 - v6) < 1e-12 * abs(v3)


def test_xml_mesh_reader(tmp_path):
    from sucemfem.mesh import Mesh
    g = golden("power_flux_solution_o2.npz")
    p = _write(tmp_path, "m.xml", g["mesh_xml"])
    m = Mesh(p)
    x, c = _parse(str(g["mesh_xml"]))
    assert np.array_equal(m.coordinates(), x)
    assert np.array_equal(m.cells(), c)
    assert m.num_vertices() == 64 and m.num_cells() == 162


def test_xml_facet_function_marks_the_boundary(tmp_path):
    """The prism's facet-region function (functional_tests) marks the PEC
    walls with 1 in DOLFIN's facet numbering; in the space's numbering the
    marked facets are exactly the exterior ones."""
    from sucemfem.mesh import Mesh, MeshFunction
    g = golden("rectangular_prism_xml.npz")
    m = Mesh(_write(tmp_path, "prism.xml", g["mesh_xml"]))
    f = MeshFunction("uint", m, _write(tmp_path, "prism_facet_region.xml", g["facet_xml"]))
    assert f.dim == 2
    topo = fem.Topology(m.cells())
    assert len(f.array()) == topo.nf
    assert set(np.nonzero(f.array() == 1)[0]) == set(topo.exterior_faces())


def test_xml_reader_rejects_bad_input(tmp_path):
    import pytest
    from sucemfem.mesh import Mesh
    p = _write(tmp_path, "bad.xml", '<dolfin><mesh celltype="triangle" dim="2"><vertices size="0"/>'
               '<cells size="0"/></mesh></dolfin>')
    with pytest.raises(ValueError):
        Mesh(p)


def _ntff_case():
    g = golden("ntff_solution_o2.npz")
    coords, cells = fem.centred_cube(g["domain_size"], float(g["max_edge_len"]))
    return g, coords, cells


def test_surface_ntff_oracle_matches_reference_golden():
    """test_ntff.py:80-92: allclose(rtol 1e-12, atol 1e-7), unshifted cube."""
    g, coords, cells = _ntff_case()
    f = golden("surface_ntff_o2.npz")
    A = fem.assemble(coords, cells, 2)
    Et, Ep = postproc.ntff(coords, cells, 2, A.topo, A.dofmap, g["x"], float(g["freq"]),
                           f["theta_deg"], f["phi_deg"])
    E = np.stack([Et, Ep], axis=1)
    assert np.allclose(E, f["E_ff"], rtol=float(f["rtol"]), atol=float(f["atol"]))
    assert np.abs(E - f["E_ff"]).max() < 1e-8


def test_get_centred_cube_matches_oracle():
    from sucemfem.Utilities.MeshGenerators import get_centred_cube
    g, coords, cells = _ntff_case()
    m = get_centred_cube(g["domain_size"], float(g["max_edge_len"]))
    assert np.array_equal(m.cells(), cells)
    assert np.allclose(m.coordinates(), coords, rtol=0, atol=1e-15)
    # with the source translation (ntff_generate_dofs.py:51): the origin is
    # the centroid of the nearest containing cell
    m2 = get_centred_cube(g["domain_size"], float(g["max_edge_len"]), [0.0, 0.0, 0.0])
    c = int(fem.locate_cells(coords, cells, np.zeros(3))[0][0])
    assert np.allclose(m2.coordinates(), coords - coords[cells[c]].mean(0), atol=1e-15)
