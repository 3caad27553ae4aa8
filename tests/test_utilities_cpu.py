"""Small reference modules on the CPU: Geometry (sucemfem/tests/
test_Geometry.py restated on the package's meshes), Testing.ErrorMeasures,
PostProcessing.circuit, Utilities.MatrixIO, and the Romberg line integral
of Sources.PostProcess."""
import warnings

import numpy as np
import pytest
import scipy.integrate as si
import scipy.sparse as sps


def test_boundary_edges_unit_cube():
    """test_Geometry.py:31-60: UnitCube(1,1,1) has 18 boundary edges, each
    with all its nodes on one face of the cube."""
    from sucemfem import Geometry
    from sucemfem.mesh import EdgeFunction, UnitCube
    mesh = UnitCube(1, 1, 1)
    ef = EdgeFunction("uint", mesh)
    ef.set_all(0)
    Geometry.BoundaryEdges(mesh).mark(ef, 11)
    marked = np.nonzero(ef.array() == 11)[0]
    assert len(marked) == 18
    V = mesh.topology_space()
    x = mesh.coordinates()[V._copy("edges", (V.ne, 2), np.int32)[marked]]    # (18, 2, 3)
    on_face = ((np.abs(x) < 1e-12) | (np.abs(x - 1) < 1e-12)).all(axis=1).any(axis=1)
    assert on_face.all()


def test_boundary_edge_cells_inscribed_tet():
    """test_Geometry.py:62-76: every cell of the inscribed tet but the last
    touches the boundary through an edge; the same cells as the native
    boundary_edge_cells of the post-processing."""
    from sucemfem import Geometry
    from sucemfem.mesh import CellFunction
    from sucemfem.PostProcessing.PostProcessing import boundary_edge_cells
    from sucemfem.Testing.Meshes import InscribedTet
    mesh = InscribedTet().get_dolfin_mesh()
    cf = CellFunction("uint", mesh)
    Geometry.BoundaryEdgeCells(mesh).mark(cf, 3)
    want = np.full(mesh.num_cells(), 3)
    want[-1] = 0
    assert np.array_equal(cf.array(), want)
    assert np.array_equal(boundary_edge_cells(mesh.topology_space()) != 0, want != 0)


def test_boundary_edges_of_a_facet_subset():
    from sucemfem import Geometry
    from sucemfem.mesh import EdgeFunction, FaceFunction, UnitCube
    mesh = UnitCube(2, 2, 2)
    V = mesh.topology_space()
    faces = V._copy("faces", (V.nf, 3), np.int32)
    x = mesh.coordinates()[faces]
    on_x0 = (np.abs(x[:, :, 0]) < 1e-12).all(axis=1)
    ff = FaceFunction("uint", mesh)
    ff._ensure(V.nf)
    ff.array()[on_x0] = 7
    ef = EdgeFunction("uint", mesh)
    Geometry.BoundaryEdges(mesh, ff, 7).mark(ef, 1)
    edges = V._copy("edges", (V.ne, 2), np.int32)
    ex = mesh.coordinates()[edges[ef.array() == 1]]
    assert (np.abs(ex[:, :, 0]) < 1e-12).all()
    assert (ef.array() == 1).sum() == 16      # x = 0 face of a 2x2 split: 16 edges


def test_error_measures_and_s11():
    from sucemfem.PostProcessing.circuit import S11
    from sucemfem.Testing.ErrorMeasures import max_normalised_RMS, normalised_RMS
    a = np.array([1.0, 2.0, -4.0])
    d = np.array([1.1, 2.0, -3.0])
    assert normalised_RMS(a, d) == pytest.approx(100 * ((0.1 / 1) ** 2 + (1 / 4) ** 2))
    assert normalised_RMS(a, d, extra_error=[0, 0.2, 0]) == pytest.approx(
        100 * ((0.1 / 1) ** 2 + (0.2 / 2) ** 2 + (1 / 4) ** 2))
    assert max_normalised_RMS(a, d) == pytest.approx(100 * ((0.1 / 4) ** 2 + (1 / 4) ** 2))
    assert S11(50.0, 50.0) == 0
    assert np.allclose(S11([0.0, 1e30, 25 + 25j], 50.0), [-1.0, 1.0, (-25 + 25j) / (75 + 25j)])


def test_matrix_io_round_trip(tmp_path):
    from sucemfem.Utilities.MatrixIO import load_scipy_matrix_from_mat, save_scipy_matrix_as_mat
    A = sps.random(40, 30, density=0.1, random_state=1, format="csr")
    D = np.arange(12.0).reshape(3, 4)
    path = str(tmp_path / "mats")
    assert save_scipy_matrix_as_mat(path, "A", A)
    assert save_scipy_matrix_as_mat(path, "D", D)
    B = load_scipy_matrix_from_mat(path, "A")
    assert sps.isspmatrix_csr(B) and abs(B - A).max() == 0
    assert np.array_equal(load_scipy_matrix_from_mat(path, "D"), D)
    assert load_scipy_matrix_from_mat(path, "missing") is None
    # test_MatrixIO.py:52-76: complex sparse and a column vector
    C = sps.csr_matrix(np.random.default_rng(2).random((30, 20))
                       + 1j * np.random.default_rng(3).random((30, 20)))
    save_scipy_matrix_as_mat(path, "C", C)
    Cl = load_scipy_matrix_from_mat(path, "C")
    assert np.array_equal(Cl.data, C.data) and np.array_equal(Cl.indices, C.indices)
    assert np.array_equal(Cl.indptr, C.indptr)
    col = np.random.default_rng(4).random((50, 1))
    save_scipy_matrix_as_mat(path, "col", col)
    assert np.array_equal(load_scipy_matrix_from_mat(path, "col"), col)


def test_romberg_against_quadrature():
    from sucemfem.Sources.PostProcess import romberg
    for f, a, b in ((np.exp, 0.0, 1.0), (lambda t: 1 / (1 + t * t), -1.0, 2.0),
                    (lambda t: np.sin(5 * t) ** 2, 0.0, 1.3)):
        ref, _ = si.quad(f, a, b, epsabs=1e-12, epsrel=1e-12)
        assert romberg(f, a, b) == pytest.approx(ref, rel=1e-8, abs=1e-8)
    # columns stop independently: the same values as one column at a time
    two = romberg(lambda t: np.stack([np.exp(t), np.cos(7 * t)], axis=1), 0.0, 1.0)
    assert two[0] == romberg(np.exp, 0.0, 1.0)
    assert two[1] == romberg(lambda t: np.cos(7 * t), 0.0, 1.0)
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        romberg(lambda t: np.sqrt(np.abs(t - 0.3)), 0.0, 1.0, tol=1e-15, rtol=1e-15, divmax=4)
        assert any("divmax" in str(x.message) for x in w)


def test_voltage_along_line():
    from sucemfem.Sources.PostProcess import VoltageAlongLine
    # E = (y, x z, 1) from (0,0,0) to (1,2,3): integral of 2t + 6t^2 + 3 over [0, 1]
    v = VoltageAlongLine(lambda x, y, z: np.array([y, x * z, 1.0]))
    assert v.calculate_voltage(np.zeros(3), np.array([1.0, 2.0, 3.0])) == pytest.approx(6.0, rel=1e-10)


def test_paths_and_filament_far_field(tmp_path):
    from sucemfem.Consts import c0, mu0
    from sucemfem.Testing import Paths
    from sucemfem.Testing.Analytical.current_fillament_farfield import eval_E_theta
    f = tmp_path / "data.txt"
    f.write_text("x")
    mod = str(tmp_path / "test_mod.py")
    assert Paths.get_module_path(mod) == str(tmp_path)
    assert Paths.get_module_path_filename("data.txt", mod) == str(f)
    with Paths.get_module_path_file("data.txt", mod) as fo:
        assert fo.read() == "x"
    # broadside of a short filament: the Hertzian dipole j omega mu I L / (4 pi r)
    freq, L, I = 1e9, 1e-3, 2.0
    omega = 2 * np.pi * freq
    e = eval_E_theta(freq, L, I, np.pi / 2, r_val=3.0)
    assert e == pytest.approx(1j * omega * mu0 * I * L * np.exp(-1j * omega / c0 * 3.0)
                              / (4 * np.pi * 3.0), rel=1e-12)
    # the array factor sin(u)/u at an oblique angle, and zero on the axis
    th = 0.7
    u = omega / c0 * 0.4 / 2 * np.cos(th)
    assert abs(eval_E_theta(freq, 0.4, 1.0, th)) == pytest.approx(
        omega * mu0 * 0.4 / (4 * np.pi) * np.sin(th) * abs(np.sin(u) / u), rel=1e-12)
    assert eval_E_theta(freq, 0.4, 1.0, 0.0) == 0


def test_voltage_along_line_reference_cases():
    """sucemfem/Sources/tests/test_postprocessing.py:31-76 with the field
    given analytically: E = (0, 0, 2z) + j (0, 0, -z^2) between the test's
    end points gives 1 - j/3, its negative on the reversed paths, and 0
    along a line in the plane z = 1."""
    from sucemfem.Sources.PostProcess import VoltageAlongLine
    re = VoltageAlongLine(lambda x, y, z: np.array([0.0, 0.0, 2 * z]))
    im = VoltageAlongLine(lambda x, y, z: np.array([0.0, 0.0, -z * z]))
    cases = [((np.array([0.5, 0.35, 0]), np.array([0.5, 0.5, 1])), 1 - 1j / 3),
             ((np.array([0, 0, 0.0]), np.array([1, 1, 1.0])), 1 - 1j / 3),
             ((np.array([0.25, 0.5, 1 - 3e-16]), np.array([0.5, 0.75, 3e-16])), -(1 - 1j / 3)),
             ((np.array([1, 1, 1.0]), np.array([0, 0, 0.0])), -(1 - 1j / 3)),
             ((np.array([0, 0, 1.0]), np.array([1, 1, 1.0])), 0.0)]
    for (a, b), want in cases:
        got = re.calculate_voltage(a, b) + 1j * im.calculate_voltage(a, b)
        assert abs(got - want) < 1e-7, (a, b, got, want)
