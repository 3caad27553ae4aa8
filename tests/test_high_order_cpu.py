"""N1curl orders 3 and 4 on the CPU: the generated reference tables against
the independent float64 oracle element, the native space (DOF map, CSR
pattern, PEC DOFs) against the oracle, and the oracle itself against the
reference's higher-order functional tests (functional_tests/
test_EigenProblems.py:86-150: cavity wavenumbers within 1e-4 relative)."""
import os
import subprocess
import sys

import numpy as np
import pytest
import scipy.sparse.linalg as spla

from oracle import fem, n1curl_exact

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "sucem-fem_gb300", "csrc")


def _gen_tables():
    sys.path.insert(0, CSRC)
    try:
        import gen_tables
    finally:
        sys.path.remove(CSRC)
    return gen_tables


def _f(x):
    return np.array(x, dtype=object).astype(float)


@pytest.mark.parametrize("order", [3, 4])
def test_moment_tables_match_independent_oracle_element(order):
    """Exact rational tables (monomial moment matrices) vs quadrature of the
    oracle's SVD-built float64 basis: two independent constructions."""
    G = _gen_tables()
    KC, KM, KT = G.tables_moments(order)
    R = n1curl_exact.reference_tensors(order)
    for exact, quad in ((KC, fem._sym6(R["curl"])), (KM, fem._sym6(R["mass"]))):
        e = _f(exact)
        assert np.abs(e - quad).max() <= 1e-12 * np.abs(e).max()
    for f in range(4):
        va, vb, vc = (np.array(G.VERTS[i], dtype=float) for i in G.FACES[f])
        ta, tb = vb - va, vc - va
        F = R["face"][f]
        aa = np.einsum("p,q,abpq->ab", ta, ta, F)
        ab = np.einsum("p,q,abpq->ab", ta, tb, F) + np.einsum("p,q,abpq->ab", tb, ta, F)
        bb = np.einsum("p,q,abpq->ab", tb, tb, F)
        for exact, quad in zip(KT[f], (aa, ab, bb)):
            e = _f(exact)
            assert np.abs(e - quad).max() <= 1e-12 * max(np.abs(e).max(), 1e-300)


def test_orders_1_2_tables_unchanged_by_the_moment_path():
    G = _gen_tables()
    for order in (1, 2):
        KC, KM, KT, _ = G.tables(order)
        assert (KC, KM, KT) == G.tables_moments(order)


def test_committed_high_order_header_is_the_generator_output(tmp_path):
    lo, hi = tmp_path / "lo.h", tmp_path / "hi.h"
    subprocess.run([sys.executable, os.path.join(CSRC, "gen_tables.py"), str(lo), str(hi)], check=True)
    for name, path in (("n1curl_tables.h", lo), ("n1curl_tables_hi.h", hi)):
        with open(os.path.join(CSRC, name)) as a, open(path) as b:
            assert a.read() == b.read(), name


@pytest.mark.parametrize("order", [3, 4])
@pytest.mark.parametrize("dims", [(2, 2, 2), (3, 2, 4)])
def test_native_space_matches_oracle(order, dims):
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    c, t = fem.unit_cube(*dims)
    V = FunctionSpace(Mesh(c, t), order=order)
    topo = fem.Topology(np.sort(t, axis=1))
    dm, n = fem.dofmap(topo, order)
    ip, ix = fem.sparsity(dm, n)
    k = order
    assert V.ndof_cell == k * (k + 2) * (k + 3) // 2
    assert V.n == n == k * topo.ne + k * (k - 1) * topo.nf + k * (k - 1) * (k - 2) // 2 * topo.nt
    assert np.array_equal(V.cell_dofs, dm)
    assert np.array_equal(V.indptr, ip) and np.array_equal(V.indices, ix)
    assert np.array_equal(V.boundary_dofs, fem.pec_dofs(topo, order))
    assert np.array_equal(V.facet_closure_dofs(topo.exterior_faces()), fem.pec_dofs(topo, order))


@pytest.mark.parametrize("order", [3, 4])
def test_entry_lists_cover_every_cell_entry_once_in_cell_order(order):
    """The gather lists of the order-3/4 assembly: every cell entry (c, a, b)
    appears exactly once, under the CSR entry (cell_dofs[c, a],
    cell_dofs[c, b]), and each entry's list runs in ascending cell order (the
    fixed summation order); the thread order permutes each row's entries by
    list length."""
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    coords, cells = fem.box_mesh(1.0, 0.5, 0.75, 3, 2, 2)
    V = FunctionSpace(Mesh(coords, cells), order=order)
    nd, nt = V.ndof_cell, V.nt
    ptr, src, perm = V.entry_lists()
    rows = np.repeat(np.arange(V.n), np.diff(V.indptr))
    assert np.array_equal(np.sort(perm), np.arange(V.nnz))
    assert np.array_equal(rows[perm], rows)        # threads stay within their row
    n_list = np.diff(ptr)[perm]
    same_row = rows[1:] == rows[:-1]
    assert np.all(n_list[1:][same_row] >= n_list[:-1][same_row])
    assert ptr[0] == 0 and ptr[-1] == nt * nd * nd and np.all(np.diff(ptr) >= 1)
    assert np.array_equal(np.sort(src), np.arange(nt * nd * nd))
    c, ab = np.divmod(src.astype(np.int64), nd * nd)
    a, b = np.divmod(ab, nd)
    q = np.repeat(np.arange(V.nnz), np.diff(ptr))
    assert np.array_equal(V.cell_dofs[c, a], rows[q])
    assert np.array_equal(V.cell_dofs[c, b], V.indices[q])
    same = q[1:] == q[:-1]
    assert np.all(c[1:][same] > c[:-1][same])


def analytic_k(abd, steps):
    """test_EigenProblems.py:42-65 and the mode list of its tests (TE and TM
    modes counted twice when no index is zero)."""
    a, b, d = abd
    vals = []
    for m in range(steps):
        for n in range(steps):
            for l in range(steps):
                i = (m, n, l)
                k = np.sqrt((m / a) ** 2 + (n / b) ** 2 + (l / d) ** 2)
                if i.count(0) < 2:
                    vals.append(k)
                if i.count(0) == 0:
                    vals.append(k)
    return np.sort(vals)


def oracle_cavity_k(coords, cells, order, nev=10, sigma=1.1):
    """The nev smallest k^2 above sigma of the PEC-free oracle pencil (S, T),
    returned as k / pi like the reference test."""
    A = fem.assemble(coords, cells, order, with_abc=False)
    free = np.setdiff1d(np.arange(A.n), fem.pec_dofs(A.topo, order))
    S = A.S[free][:, free].tocsc()
    T = A.T[free][:, free].tocsc()
    w = spla.eigsh(S, k=nev, M=T, sigma=sigma, which="LA", return_eigenvectors=False)
    return np.sqrt(np.sort(w)) / np.pi


def prism_mesh(tmp_path):
    from sucemfem.mesh import Mesh, MeshFunction
    g = np.load(os.path.join(HERE, "golden", "rectangular_prism_xml.npz"))
    pm, pf = tmp_path / "prism.xml", tmp_path / "prism_facet_region.xml"
    pm.write_text(str(g["mesh_xml"]))
    pf.write_text(str(g["facet_xml"]))
    m = Mesh(str(pm))
    return m, MeshFunction("uint", m, str(pf))


def test_reference_cube_cavity_order3_on_the_oracle():
    """test_cube_resonant_cavity: UnitCube(4,4,4), order 3, sigma 1.1, ten
    modes, assert_array_almost_equal(errors, 0, 4)."""
    c, t = fem.unit_cube(4, 4, 4)
    res = oracle_cavity_k(c, t, 3)
    ref = analytic_k((1.0, 1.0, 1.0), 3)[:10]
    np.testing.assert_array_almost_equal(np.abs(res - ref) / ref, np.zeros(10), 4)


def test_reference_prism_cavity_order4_on_the_oracle(tmp_path):
    """test_gmsh_resonant_cavity: the rectangular prism mesh (1 x 0.5 x 0.25),
    PEC on facet region 1 (every exterior facet), order 4, sigma 1.1."""
    m, f = prism_mesh(tmp_path)
    topo = fem.Topology(np.sort(m.cells(), axis=1))
    assert set(np.nonzero(f.array() == 1)[0]) == set(topo.exterior_faces())
    res = oracle_cavity_k(m.coordinates(), m.cells(), 4)
    ref = analytic_k((1.0, 0.5, 0.25), 5)[:10]
    np.testing.assert_array_almost_equal(np.abs(res - ref) / ref, np.zeros(10), 4)


def test_high_order_space_rejects_order_1_2_only_host_queries():
    """The boundary dual functionals (interpolation onto the boundary) are
    provided for orders 1 and 2; an order-3 space refuses the host copy."""
    from sucemfem._native import COPY, call, ptr
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    c, t = fem.unit_cube(1, 1, 1)
    V = FunctionSpace(Mesh(c, t), order=3)
    out = np.zeros(V.n_boundary * 6)
    with pytest.raises(ValueError, match="orders 1 and 2"):
        call("sucem_space_copy", V._h, COPY["boundary_dual"], ptr(out))
    V2 = FunctionSpace(Mesh(c, t), order=2)
    out = np.zeros(V2.n_boundary * 6)
    call("sucem_space_copy", V2._h, COPY["boundary_dual"], ptr(out))
    assert np.isfinite(out).all() and np.abs(out).max() > 0


def test_entry_lists_exist_for_orders_3_4_only():
    """Orders 1-2 assemble through the entity schedule: an order-2 space has
    no gather lists and says so."""
    from sucemfem.mesh import Mesh
    from sucemfem.space import FunctionSpace
    c, t = fem.unit_cube(1, 1, 1)
    with pytest.raises(ValueError, match="orders 3 and 4"):
        FunctionSpace(Mesh(c, t), order=2).entry_lists()
