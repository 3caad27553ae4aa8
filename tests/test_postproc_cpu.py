"""CPU checks of the post-processing path: the oracle's surface power flux
pinned to the reference's golden (test_power_flux.py:54, SurfaceFlux on the
test's own DOLFIN XML mesh), and the DOLFIN XML mesh / mesh-function
readers against an independent parse and the oracle's facet numbering."""
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

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


def test_variational_surface_flux_oracle_matches_reference_golden():
    """test_power_flux.py:77: assertAlmostEqual(calc_flux(), 26.9015957282-7.857e-08j)."""
    g = golden("power_flux_solution_o2.npz")
    coords, cells = _parse(str(g["mesh_xml"]))
    A = fem.assemble(coords, cells, 2)
    k0 = 2 * np.pi * float(g["freq"]) / fem.C0
    v = postproc.variational_surface_flux(coords, cells, 2, A.topo, A.dofmap, g["x"], k0)
    assert abs(v - complex(g["flux_variational"])) < 5e-8, v


def test_variational_ntff_oracle_matches_reference_golden():
    g, coords, cells = _ntff_case()
    f = golden("variational_ntff_o2.npz")
    A = fem.assemble(coords, cells, 2)
    Et, Ep = postproc.variational_ntff(coords, cells, 2, A.topo, A.dofmap, g["x"],
                                       float(g["freq"]), f["theta_deg"], f["phi_deg"])
    E = np.stack([Et, Ep], axis=1)
    assert np.allclose(E, f["E_ff"], rtol=float(f["rtol"]), atol=float(f["atol"]))
    assert np.abs(E - f["E_ff"]).max() < 1e-8


@pytest.mark.parametrize("order", [1, 2])
def test_boundary_dual_and_edge_cells_match_oracle(order):
    """Host-side tables of the product (no GPU): boundary DOF dual
    functionals and the boundary-edge cells against the oracle."""
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    from sucemfem.Interpolation.Interpolation import boundary_dual
    from sucemfem.PostProcessing.PostProcessing import boundary_edge_cells
    coords, cells = fem.box_mesh(1.0, 0.5, 0.75, 3, 2, 3)
    coords = fem.jitter_interior(coords, cells, 0.25, 0.2, seed=5)
    V = FunctionSpace(Mesh(coords, cells), order=order)
    A = fem.assemble(coords, cells, order)
    b, p, t = boundary_dual(V)
    assert np.array_equal(b, fem.pec_dofs(A.topo, order))
    rp, rt = postproc.dof_points_tangents(coords, cells, order, A.dofmap, b)
    assert np.allclose(p, rp, atol=1e-14) and np.allclose(t, rt, atol=1e-14)
    assert np.array_equal(boundary_edge_cells(V).astype(bool), postproc.boundary_edge_cells(A.topo))


def test_surface_interpolant_host_matches_oracle():
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    from sucemfem.Interpolation import SurfaceInterpolant
    from sucemfem.PostProcessing.variational_ntff import TransformTestingExpression
    coords, cells = fem.box_mesh(0.3, 0.2, 0.25, 3, 2, 3, origin=(-0.15, -0.1, -0.125))
    V = FunctionSpace(Mesh(coords, cells), order=2)
    A = fem.assemble(coords, cells, 2)
    rhat = np.array([0.3, -0.5, 0.8]) / np.linalg.norm([0.3, -0.5, 0.8])
    ahat = np.array([0.0, 0.8, 0.5])
    k0 = 21.0
    t = TransformTestingExpression()
    t.set_parms(rhat, ahat, k0)
    si = SurfaceInterpolant(V)
    si.set_interpolant_expression(*t.get_expression())
    got = si.calculate_interpolation()
    cf = np.cross(rhat, np.cross(ahat, rhat)) / k0
    ref = postproc.surface_interpolant(coords, cells, 2, A.topo, A.dofmap, V.n,
                                       lambda p: 1j * cf[None] * np.exp(1j * k0 * (p @ rhat))[:, None])
    assert np.abs(got - ref).max() < 1e-13 * np.abs(ref).max()
