"""GPU post-processing parity (through the C-ABI): the surface power flux
against the reference's golden (test_power_flux.py:54, 7 places, on the
test's own XML mesh) and the FP64 oracle, and the field at points against
the oracle."""
import os

import numpy as np
import pytest

from conftest import golden
from oracle import fem, postproc

pytestmark = pytest.mark.gpu


def _xml_space(tmp_path, text, order):
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    p = os.path.join(str(tmp_path), "m.xml")
    with open(p, "w") as f:
        f.write(str(text))
    m = Mesh(p)
    return m, FunctionSpace(m, order=order)


def test_surface_flux_reference_golden(tmp_path):
    from sucemfem.PostProcessing.power_flux import SurfaceFlux
    g = golden("power_flux_solution_o2.npz")
    m, V = _xml_space(tmp_path, g["mesh_xml"], 2)
    k0 = 2 * np.pi * float(g["freq"]) / fem.C0
    sf = SurfaceFlux(V)
    sf.set_k0(k0)
    sf.set_dofs(g["x"])
    v = sf.calc_flux()
    assert abs(v - float(g["flux_surface"])) < 5e-8, v
    A = fem.assemble(m.coordinates(), m.cells(), 2)
    ref = postproc.surface_flux(m.coordinates(), m.cells(), 2, A.topo, A.dofmap, g["x"], k0)
    assert abs(v - ref) < 1e-12 * abs(ref)
    assert sf.calc_flux() == v  # fixed-order reduction: bit-identical repeat


def test_surface_flux_complex64_dofs_and_mu(tmp_path):
    import torch
    from sucemfem import _device
    from sucemfem.PostProcessing.power_flux import SurfaceFlux
    g = golden("power_flux_solution_o2.npz")
    m, V = _xml_space(tmp_path, g["mesh_xml"], 2)
    k0 = 2 * np.pi * float(g["freq"]) / fem.C0
    mu = np.random.default_rng(3).uniform(1.0, 3.0, m.num_cells())
    A = fem.assemble(m.coordinates(), m.cells(), 2)
    ref = postproc.surface_flux(m.coordinates(), m.cells(), 2, A.topo, A.dofmap, g["x"], k0, mu)
    sf = SurfaceFlux(V)
    sf.set_k0(k0)
    sf.set_mur_function(mu)
    sf.set_dofs(g["x"])
    assert abs(sf.calc_flux() - ref) < 1e-12 * abs(ref)
    sf.set_dofs(torch.as_tensor(g["x"]).to(torch.complex64).to(_device.device()))
    assert abs(sf.calc_flux() - ref) < 1e-5 * abs(ref)


def test_surface_flux_order1_box():
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    from sucemfem.PostProcessing.power_flux import SurfaceFlux
    coords, cells = fem.box_mesh(1.0, 0.5, 0.75, 3, 2, 3)
    coords = fem.jitter_interior(coords, cells, 0.25, 0.2, seed=1)
    V = FunctionSpace(Mesh(coords, cells), order=1)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(V.n) + 1j * rng.standard_normal(V.n)
    A = fem.assemble(coords, cells, 1)
    ref = postproc.surface_flux(coords, cells, 1, A.topo, A.dofmap, x, 7.0)
    sf = SurfaceFlux(V)
    sf.set_k0(7.0)
    sf.set_dofs(x)
    assert abs(sf.calc_flux() - ref) < 1e-12 * max(1.0, abs(ref))


@pytest.mark.parametrize("order", [1, 2])
def test_reconstruct_points(order):
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    from sucemfem.PostProcessing import Reconstruct
    coords, cells = fem.box_mesh(1.0, 1.0, 1.0, 3, 3, 3)
    coords = fem.jitter_interior(coords, cells, 1 / 3, 0.2, seed=2)
    V = FunctionSpace(Mesh(coords, cells), order=order)
    A = fem.assemble(coords, cells, order)
    rng = np.random.default_rng(1)
    x = rng.standard_normal(V.n) + 1j * rng.standard_normal(V.n)
    pts = np.vstack([rng.uniform(0.02, 0.98, (40, 3)), [[0.5, 0.5, 0.5], [2.0, 0.5, 0.5]]])
    r = Reconstruct(V)
    r.set_dof_values(x)
    got = r.reconstruct_points(pts)
    ref = postproc.reconstruct_points(coords, cells, order, A.dofmap, x, pts)
    inside = ~np.isnan(ref[:, 0].real)
    assert inside.sum() == len(pts) - 1 and not inside[-1]
    assert np.all(np.isnan(got[~inside].real))
    err = np.abs(got[inside] - ref[inside]).max() / np.abs(ref[inside]).max()
    assert err < 1e-12, err


def test_surface_ntff_reference_golden():
    from sucemfem.PostProcessing.surface_ntff import NTFF
    from sucemfem.space import FunctionSpace
    from sucemfem.Utilities.MeshGenerators import get_centred_cube
    g = golden("ntff_solution_o2.npz")
    f = golden("surface_ntff_o2.npz")
    m = get_centred_cube(g["domain_size"], float(g["max_edge_len"]))
    V = FunctionSpace(m, order=2)
    dut = NTFF(V)
    dut.set_frequency(float(g["freq"]))
    dut.set_dofs(g["x"])
    E = np.array([dut.calc_pt(th, ph) for th, ph in zip(f["theta_deg"], f["phi_deg"])])
    assert np.allclose(E, f["E_ff"], rtol=float(f["rtol"]), atol=float(f["atol"]))
    A = fem.assemble(m.coordinates(), m.cells(), 2)
    Et, Ep = postproc.ntff(m.coordinates(), m.cells(), 2, A.topo, A.dofmap, g["x"],
                           float(g["freq"]), f["theta_deg"], f["phi_deg"])
    ref = np.stack([Et, Ep], axis=1)
    assert np.abs(E - ref).max() < 1e-12 * np.abs(ref).max()
    Et2, Ep2 = dut.calc_pts(f["theta_deg"], f["phi_deg"])
    assert np.array_equal(np.stack([Et2, Ep2], axis=1), E)  # fixed-order sums
    assert len(dut._L) == len(f["theta_deg"]) and len(dut._N) == len(f["theta_deg"])


def test_surface_ntff_order1_many_directions():
    from sucemfem.mesh import Mesh
    from sucemfem.PostProcessing.surface_ntff import NTFF
    from sucemfem.space import FunctionSpace
    coords, cells = fem.box_mesh(0.3, 0.2, 0.25, 3, 2, 3, origin=(-0.15, -0.1, -0.125))
    V = FunctionSpace(Mesh(coords, cells), order=1)
    rng = np.random.default_rng(4)
    x = rng.standard_normal(V.n) + 1j * rng.standard_normal(V.n)
    th = rng.uniform(0, 180, 50)
    ph = rng.uniform(0, 360, 50)
    dut = NTFF(V)
    dut.set_frequency(1e9)
    dut.set_dofs(x)
    Et, Ep = dut.calc_pts(th, ph)
    A = fem.assemble(coords, cells, 1)
    rt, rp = postproc.ntff(coords, cells, 1, A.topo, A.dofmap, x, 1e9, th, ph)
    scale = max(np.abs(rt).max(), np.abs(rp).max())
    assert np.abs(Et - rt).max() < 1e-12 * scale and np.abs(Ep - rp).max() < 1e-12 * scale


def test_variational_surface_flux_reference_golden(tmp_path):
    from sucemfem.PostProcessing.power_flux import VariationalSurfaceFlux
    g = golden("power_flux_solution_o2.npz")
    m, V = _xml_space(tmp_path, g["mesh_xml"], 2)
    k0 = 2 * np.pi * float(g["freq"]) / fem.C0
    dut = VariationalSurfaceFlux(V)
    dut.set_k0(k0)
    dut.set_dofs(g["x"])
    v = dut.calc_flux()
    assert abs(v - complex(g["flux_variational"])) < 5e-8, v
    A = fem.assemble(m.coordinates(), m.cells(), 2)
    ref = postproc.variational_surface_flux(m.coordinates(), m.cells(), 2, A.topo, A.dofmap,
                                            g["x"], k0)
    assert abs(v - ref) < 1e-12 * abs(ref)


def test_variational_ntff_reference_golden():
    from sucemfem.PostProcessing.variational_ntff import NTFF
    from sucemfem.space import FunctionSpace
    from sucemfem.Utilities.MeshGenerators import get_centred_cube
    g = golden("ntff_solution_o2.npz")
    f = golden("variational_ntff_o2.npz")
    m = get_centred_cube(g["domain_size"], float(g["max_edge_len"]))
    V = FunctionSpace(m, order=2)
    dut = NTFF(V)
    dut.set_frequency(float(g["freq"]))
    dut.set_dofs(g["x"])
    E = np.array([dut.calc_pt(th, ph) for th, ph in zip(f["theta_deg"], f["phi_deg"])])
    assert np.allclose(E, f["E_ff"], rtol=float(f["rtol"]), atol=float(f["atol"]))
    A = fem.assemble(m.coordinates(), m.cells(), 2)
    Et, Ep = postproc.variational_ntff(m.coordinates(), m.cells(), 2, A.topo, A.dofmap, g["x"],
                                       float(g["freq"]), f["theta_deg"], f["phi_deg"])
    ref = np.stack([Et, Ep], axis=1)
    assert np.abs(E - ref).max() < 1e-11 * np.abs(ref).max()


@pytest.mark.parametrize("order", [1, 2])
def test_em_functional_materials_and_domains(order):
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    from sucemfem.PostProcessing import CalcEMFunctional
    coords, cells = fem.box_mesh(1.0, 0.5, 0.75, 3, 2, 3)
    coords = fem.jitter_interior(coords, cells, 0.25, 0.2, seed=6)
    V = FunctionSpace(Mesh(coords, cells), order=order)
    A = fem.assemble(coords, cells, order)
    rng = np.random.default_rng(7)
    E = rng.standard_normal(V.n) + 1j * rng.standard_normal(V.n)
    gv = rng.standard_normal(V.n) + 1j * rng.standard_normal(V.n)
    eps = rng.uniform(1, 4, V.nt)
    mu = rng.uniform(1, 2, V.nt)
    dom = rng.integers(0, 3, V.nt)
    f = CalcEMFunctional(V)
    f.set_k0(5.5)
    f.set_E_dofs(E)
    f.set_g_dofs(gv)
    f.set_epsr_function(eps)
    f.set_mur_function(mu)
    f.set_cell_domains(dom, 2)
    got = f.calc_functional()
    ref = postproc.calc_em_functional(coords, cells, order, A.dofmap, E, gv, 5.5, dom == 2, eps, mu)
    assert abs(got - ref) < 1e-12 * abs(ref)


def test_plane_wave_dofs_match_host_interpolant():
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    from sucemfem.Interpolation import SurfaceInterpolant
    from sucemfem.PostProcessing.variational_ntff import NTFF, TransformTestingExpression
    coords, cells = fem.box_mesh(0.3, 0.2, 0.25, 3, 2, 3, origin=(-0.15, -0.1, -0.125))
    V = FunctionSpace(Mesh(coords, cells), order=2)
    rhat = np.array([0.3, -0.5, 0.8]) / np.linalg.norm([0.3, -0.5, 0.8])
    ahat = np.array([0.0, 0.8, 0.5])
    dut = NTFF(V)
    dut.set_k0(21.0)
    g = dut._testing_dofs(rhat[None], ahat[None])[0].cpu().numpy()
    t = TransformTestingExpression()
    t.set_parms(rhat, ahat, 21.0)
    si = SurfaceInterpolant(V)
    si.set_interpolant_expression(*t.get_expression())
    ref = si.calculate_interpolation()
    assert np.abs(g - ref).max() < 1e-13 * np.abs(ref).max()


def test_complex_voltage_along_line():
    """Sources/PostProcess.py:46-66: the complex line integral of E . l_hat
    with the field reconstructed on the GPU (each Romberg level's points in
    one batch) against the same Romberg integration of the oracle's field,
    real and imaginary parts as two separate integrals."""
    import warnings
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    from sucemfem.Sources.PostProcess import ComplexVoltageAlongLine, VoltageAlongLine
    coords, cells = fem.box_mesh(1.0, 1.0, 1.0, 3, 3, 3)
    coords = fem.jitter_interior(coords, cells, 1 / 3, 0.2, seed=4)
    V = FunctionSpace(Mesh(coords, cells), order=2)
    A = fem.assemble(coords, cells, 2)
    rng = np.random.default_rng(8)
    x = rng.standard_normal(V.n) + 1j * rng.standard_normal(V.n)
    start, end = np.array([0.1, 0.2, 0.3]), np.array([0.8, 0.7, 0.9])

    def oracle_E(part):
        def E(px, py, pz):
            e = postproc.reconstruct_points(coords, cells, 2, A.dofmap, x, np.array([[px, py, pz]]))[0]
            return e.real if part == 0 else e.imag
        return E
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        cv = ComplexVoltageAlongLine(V)
        cv.set_dofs(x)
        got = cv.calculate_voltage(start, end)
        ref = (VoltageAlongLine(oracle_E(0)).calculate_voltage(start, end)
               + 1j * VoltageAlongLine(oracle_E(1)).calculate_voltage(start, end))
    assert abs(got - ref) <= 1e-9 * abs(ref), (got, ref)


def test_em_functional_symmetry():
    """sucemfem/PostProcessing/tests/test_Postprocessing.py:31-52: the
    functional is symmetric in E and g (UnitCube(2,2,2), order 1, random
    complex DOFs, random k0); here to round-off, the two sums being taken in
    different orders."""
    from sucemfem.mesh import UnitCube
    from sucemfem.space import FunctionSpace
    from sucemfem.PostProcessing import CalcEMFunctional
    V = FunctionSpace(UnitCube(2, 2, 2), order=1)
    rng = np.random.default_rng(11)
    E = rng.random(V.n) + 1j * rng.random(V.n)
    g = rng.random(V.n) + 1j * rng.random(V.n)
    k0 = rng.random() * 10
    f = CalcEMFunctional(V)
    f.set_k0(k0)
    f.set_g_dofs(g)
    f.set_E_dofs(E)
    v1 = f.calc_functional()
    f.set_g_dofs(E)
    f.set_E_dofs(g)
    v2 = f.calc_functional()
    assert abs(v1 - v2) <= 1e-13 * abs(v1)
