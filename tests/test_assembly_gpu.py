"""GPU assembly parity against the FP64 oracle (through the C-ABI).

Tolerances: per-entry error divided by the largest |entry| of its row
(entries that cancel to ~0 have no meaningful relative error; rows whose
entries are all round-off are scaled by 1e-6 of the matrix's largest entry
instead; the ABC matrix B, whose mathematically-zero entries the oracle
computes by cancellation of O(1) terms, is scaled by its largest entry):
  FP64 kernels  <= 1e-12
  FP32 kernels  <= 2e-6
CSR pattern and DOF numbering are compared bit-exactly (CPU tests)."""
import numpy as np
import pytest

from conftest import golden
from oracle import fem

pytestmark = pytest.mark.gpu

TOL = {8: 1e-12, 4: 2e-6}


def _mesh(name):
    if name == "inscribed":
        return fem.inscribed_tet()
    if name == "box":
        return fem.box_mesh(1.0, 0.5, 0.75, 3, 2, 2)
    coords, cells = fem.unit_cube(3, 3, 3)
    return fem.jitter_interior(coords, cells, 1 / 3, 0.2, seed=0), cells


def _row_err(got, R, floor=1e-6):
    R = R.tocsr()
    rowmax = np.maximum.reduceat(np.abs(R.data), R.indptr[:-1])
    rowmax = np.maximum(rowmax, floor * np.abs(R.data).max())
    scale = np.repeat(rowmax, np.diff(R.indptr))
    return np.max(np.abs(got - R.data) / scale)


def _assemble(V, rb, eps, mu_inv, which="STB"):
    import torch
    from sucemfem import _device
    from sucemfem._native import call, ptr
    dev = _device.device()
    dt = torch.float32 if rb == 4 else torch.float64
    out = {k: torch.empty(V.nnz, dtype=dt, device=dev) if k in which else None for k in "STB"}
    de = None if eps is None else torch.as_tensor(eps, dtype=dt, device=dev)
    dm = None if mu_inv is None else torch.as_tensor(mu_inv, dtype=dt, device=dev)
    call("sucem_assemble", V.upload(), rb, ptr(de), ptr(dm), ptr(out["S"]), ptr(out["T"]),
         ptr(out["B"]), _device.stream_ptr())
    torch.cuda.synchronize()
    return {k: (v.double().cpu().numpy() if v is not None else None) for k, v in out.items()}


@pytest.mark.parametrize("rb", [8, 4])
@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("mesh", ["inscribed", "box", "jitter"])
def test_assembly_matches_oracle(rb, order, mesh):
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    coords, cells = _mesh(mesh)
    rng = np.random.default_rng(3)
    eps = rng.uniform(1, 4, len(cells))
    mu = rng.uniform(1, 2, len(cells))
    ref = fem.assemble(coords, cells, order, eps_r=eps, mu_r=mu)
    V = FunctionSpace(Mesh(coords, cells), order=order)
    got = _assemble(V, rb, eps, 1 / mu)
    for k, R in (("S", ref.S), ("T", ref.T), ("B", ref.B)):
        assert _row_err(got[k], R, 1.0 if k == "B" else 1e-6) <= TOL[rb], k


@pytest.mark.parametrize("rb", [8, 4])
def test_assembly_subsets_and_defaults(rb):
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    coords, cells = _mesh("box")
    ref = fem.assemble(coords, cells, 2)
    V = FunctionSpace(Mesh(coords, cells), order=2)
    got = _assemble(V, rb, None, None, which="T")
    assert got["S"] is None and got["B"] is None
    assert _row_err(got["T"], ref.T) <= TOL[rb]
    got = _assemble(V, rb, None, None, which="ST")
    assert _row_err(got["S"], ref.S) <= TOL[rb]


@pytest.mark.parametrize("rb", [8, 4])
@pytest.mark.parametrize("order", [1, 2])
def test_fused_helmholtz(rb, order):
    import torch
    from sucemfem import _device
    from sucemfem._native import call, ptr
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    coords, cells = _mesh("jitter")
    rng = np.random.default_rng(5)
    eps = rng.uniform(1, 4, len(cells))
    f = 299792458 / 0.4
    k0 = 2 * np.pi * f / 299792458
    ref = fem.assemble(coords, cells, order, eps_r=eps)
    V = FunctionSpace(Mesh(coords, cells), order=order)
    dt = torch.float32 if rb == 4 else torch.float64
    ct = torch.complex64 if rb == 4 else torch.complex128
    A = torch.empty(V.nnz, dtype=ct, device=_device.device())
    de = torch.as_tensor(eps, dtype=dt, device=_device.device())
    call("sucem_assemble_helmholtz", V.upload(), rb, ptr(de), None, k0, ptr(A), _device.stream_ptr())
    got = A.cpu().numpy().astype(np.complex128)
    re = ref.S.data - k0 ** 2 * ref.T.data
    im = k0 * ref.B.data
    scale = np.abs(ref.S.data) + k0 ** 2 * np.abs(ref.T.data) + k0 * np.abs(ref.B.data)
    rowmax = np.repeat(np.maximum.reduceat(scale, ref.S.indptr[:-1]), np.diff(ref.S.indptr))
    assert np.max(np.abs(got - (re + 1j * im)) / rowmax) <= 2 * TOL[rb]


def test_host_buffer_assembly():
    from sucemfem._native import call, ptr
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    coords, cells = _mesh("box")
    eps = np.linspace(1, 2, len(cells))
    ref = fem.assemble(coords, cells, 1, eps_r=eps)
    V = FunctionSpace(Mesh(coords, cells), order=1)
    V.upload()
    S = np.empty(V.nnz)
    T = np.empty(V.nnz)
    call("sucem_assemble_host", V.upload(), 8, ptr(eps), None, ptr(S), ptr(T), None)
    assert _row_err(S, ref.S) <= 1e-12 and _row_err(T, ref.T) <= 1e-12


def _driven(order, mesh_pair, materials=None, regions=None):
    from sucemfem.BoundaryConditions import ABCBoundaryCondition, BoundaryConditions
    from sucemfem.ProblemConfigurations.EMDrivenProblem import DrivenProblemABC
    from sucemfem.mesh import Mesh, MeshFunction
    mesh = Mesh(*mesh_pair)
    abc = ABCBoundaryCondition()
    abc.set_region_number(1)
    bcs = BoundaryConditions()
    bcs.add_boundary_condition(abc)
    dp = DrivenProblemABC()
    dp.set_mesh(mesh)
    dp.set_basis_order(order)
    mf = MeshFunction("uint", mesh, 3)
    mf.set_all(0)
    if regions is not None:
        mf.array()[:] = regions
    dp.set_material_regions(materials or {0: dict(eps_r=1, mu_r=1)})
    dp.set_region_meshfunction(mf)
    dp.set_boundary_conditions(bcs)
    return dp


def test_dropin_lhs_rhs_golden():
    """test_EMDrivenProblem.py:64-82 through the drop-in API."""
    from sucemfem.Sources import current_source, point_source
    g = golden("driven_inscribed_tet_o1.npz")
    dp = _driven(1, fem.inscribed_tet())
    cs = current_source.CurrentSources()
    src = point_source.PointCurrentSource()
    src.set_position(g["source_coord"])
    src.set_value(g["source_value"])
    cs.add_source(src)
    dp.set_sources(cs)
    dp.set_frequency(float(g["frequency"]))
    dp.init_problem()
    L = dp.get_LHS_matrix()
    assert L.dtype == np.complex128 and L.shape == (24, 24)
    assert not np.any(L.data == 0)
    assert np.allclose(L.toarray(), g["lhs"], rtol=1e-10, atol=3e-15)
    assert np.allclose(dp.get_RHS(), g["rhs"], rtol=1e-12, atol=1e-16)


def test_dropin_lhs_matches_scipy_semantics():
    rng = np.random.default_rng(0)
    coords, cells = fem.box_mesh(1, 1, 1, 3, 3, 3)
    eps = rng.uniform(1, 4, len(cells))
    regions = np.arange(len(cells))
    mats = {int(i): dict(eps_r=float(e), mu_r=1.0) for i, e in enumerate(eps)}
    dp = _driven(2, (coords, cells), mats, regions)
    from sucemfem.Sources import current_source
    dp.set_sources(current_source.CurrentSources())
    dp.set_frequency(299792458 / 0.4)
    dp.init_problem()
    L = dp.get_LHS_matrix()
    ref = fem.assemble(coords, cells, 2, eps_r=eps)
    R = fem.lhs_matrix(ref.S, ref.T, ref.B, 299792458 / 0.4)
    D = (L - R).tocsr()
    assert abs(D).max() <= 1e-12 * abs(R).max()


def test_fillament_golden_lowest_cell_rule():
    from sucemfem.Sources.fillament_current_source import FillamentCurrentSource
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    g = golden("fillament_source_o2.npz")
    V = FunctionSpace(Mesh(*fem.centred_cube(g["domain_size"], float(g["max_edge_len"]))), order=2)
    src = FillamentCurrentSource()
    src.set_function_space(V)
    src.set_no_integration_points(int(g["no_integration_points"]))
    src.set_source_endpoints(g["source_endpoints"])
    src.set_value(float(g["I"]))
    d, v = src.get_contribution()
    gd = dict(zip(g["dofnos"].tolist(), g["rhs_contribs"]))
    od = dict(zip(d.tolist(), v))
    keys = sorted(set(gd) | set(od))
    a = np.array([od.get(k, 0.0) for k in keys])
    b = np.array([gd.get(k, 0.0) for k in keys])
    assert np.allclose(a, b, rtol=1e-10, atol=1e-12)
    # negative direction flips the sign (test_fillament_source.py:71-84)
    src.set_source_endpoints(-g["source_endpoints"])
    d2, v2 = src.get_contribution()
    o2 = dict(zip(d2.tolist(), v2))
    assert np.allclose([o2.get(k, 0.0) for k in keys], -a, atol=1e-12)


def test_point_source_outside_mesh_raises():
    from sucemfem.Sources.point_source import calc_pointsource_contrib
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    V = FunctionSpace(Mesh(*fem.unit_cube(2, 2, 2)), order=1)
    with pytest.raises(ValueError, match="outside"):
        calc_pointsource_contrib(V, [2.0, 0.5, 0.5], [0, 0, 1.0])


@pytest.mark.parametrize("order", [1, 2])
def test_pec_rows_and_spmv(order):
    import torch
    from sucemfem import _device
    from sucemfem.matrix import GPUMatrix
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    coords, cells = fem.box_mesh(1.0, 0.5, 0.75, 4, 2, 3)
    ref = fem.assemble(coords, cells, order)
    V = FunctionSpace(Mesh(coords, cells), order=order)
    got = _assemble(V, 8, None, None, which="ST")
    S = GPUMatrix(V, torch.as_tensor(got["S"], device=_device.device()))
    S.ident_rows(V.boundary_dofs)
    Sr = fem.apply_pec(ref.S, fem.pec_dofs(ref.topo, order))
    assert np.abs(S.values.cpu().numpy() - Sr.data).max() <= 1e-12 * np.abs(Sr.data).max()
    x = np.random.default_rng(0).standard_normal(V.n)
    assert np.allclose(S * x, Sr @ x, rtol=1e-12, atol=1e-10)
    xc = x + 1j * np.random.default_rng(1).standard_normal(V.n)
    assert np.allclose(S * xc, Sr @ xc, rtol=1e-12, atol=1e-10)
    T = GPUMatrix(V, torch.as_tensor(got["T"], device=_device.device()))
    D = S - 2.5 * T
    assert np.allclose(D.values.cpu().numpy(), Sr.data - 2.5 * ref.T.data, rtol=0, atol=1e-12 * np.abs(Sr.data).max())
