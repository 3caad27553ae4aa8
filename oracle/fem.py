"""FP64 CPU restatement of the reference's N1curl assembly path (the oracle).

TEST INFRASTRUCTURE ONLY.  Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of bench.py import this module; the product never does.

What it restates, with the reference call sites it follows:

* mesh entity numbering and the N1curl DOF map that the reference gets from
  ``dolfin.FunctionSpace`` (sucemfem/ProblemConfigurations/EMProblem.py:100-105):
  cells have their vertices sorted by global index (DOLFIN ``mesh.order()``),
  edges and faces are numbered by first encounter while walking the cells in
  order and each cell's local entities in UFC order (DOLFIN
  TopologyComputation), order-1 DOFs are the edges, order-2 DOFs are
  2*edge+{0,1} followed by 2*E + 2*face+{0,1} (the FFC dof map layout),
  orders 3 and 4 continue that entity-major layout (k per edge, k(k-1) per
  face, then the k(k-1)(k-2)/2 interior DOFs of every cell);
* the element forms: mass ``eps_r*inner(v,u)*dx`` and curl-curl
  ``dot(curl(v),curl(u))/mu_r*dx`` (sucemfem/Forms.py:71-85) and the ABC
  form ``inner(cross(n,v),cross(n,u))*ds`` over every exterior facet
  (sucemfem/BoundaryConditions/ABC.py:56-57);
* ``SystemMatrices.calc_system_matrices`` (sucemfem/SystemMatrices.py:46-58):
  every matrix on the cell-pair sparsity pattern with sorted columns and
  explicit zeros kept;
* the PEC essential condition (sucemfem/BoundaryConditions/essential.py:65-99):
  rows of DOFs on the closure of exterior facets zeroed, unit diagonal;
* ``get_LHS_matrix`` / ``get_RHS`` (sucemfem/ProblemConfigurations/
  EMDrivenProblem.py:67-80) and the point / filament sources
  (sucemfem/Sources/point_source.py:49-94,
  sucemfem/Sources/fillament_current_source.py:62-82).
"""
import numpy as np
import scipy.sparse as sps

from . import n1curl_exact

# UFC local edges / faces of a tetrahedron (vertex pairs / triples)
EDGES = np.array([(2, 3), (1, 3), (1, 2), (0, 3), (0, 2), (0, 1)])
FACES = np.array([(1, 2, 3), (0, 2, 3), (0, 1, 3), (0, 1, 2)])

# Consts.py:24-31
PI = np.pi
MU0 = np.pi * 4 * 1e-7
C0 = 299792458
EPS0 = 10 ** 7 / 4 / np.pi / C0 / C0
Z0 = MU0 * C0


# --------------------------------------------------------------------------
# meshes
# --------------------------------------------------------------------------
def unit_cube(nx, ny, nz):
    """DOLFIN UnitCube(nx,ny,nz): vertices x fastest, 6 tets per cube sharing
    the v0-v7 diagonal (the split seen in the reference's fixture mesh
    sucemfem/PostProcessing/tests/data/*_mesh.xml)."""
    ix, iy, iz = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    coords = np.stack([ix.transpose(2, 1, 0).ravel() / float(nx),
                       iy.transpose(2, 1, 0).ravel() / float(ny),
                       iz.transpose(2, 1, 0).ravel() / float(nz)], axis=1)
    cells = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                v0 = k * (nx + 1) * (ny + 1) + j * (nx + 1) + i
                v1 = v0 + 1
                v2 = v0 + (nx + 1)
                v3 = v1 + (nx + 1)
                v4 = v0 + (nx + 1) * (ny + 1)
                v5 = v1 + (nx + 1) * (ny + 1)
                v6 = v2 + (nx + 1) * (ny + 1)
                v7 = v3 + (nx + 1) * (ny + 1)
                cells += [(v0, v1, v3, v7), (v0, v1, v7, v5), (v0, v5, v7, v4),
                          (v0, v3, v2, v7), (v0, v6, v4, v7), (v0, v2, v6, v7)]
    return coords, np.sort(np.array(cells, dtype=np.int64), axis=1)


def box_mesh(lx, ly, lz, nx, ny, nz, origin=(0.0, 0.0, 0.0)):
    coords, cells = unit_cube(nx, ny, nz)
    coords = coords * np.array([lx, ly, lz]) + np.asarray(origin)
    return coords, cells


def centred_cube(domain_size, max_edge_len):
    """sucemfem/Utilities/MeshGenerators.py:26-35 (without the optional shift)."""
    domain_size = np.asarray(domain_size, dtype=np.float64)
    n = np.array(np.ceil(np.sqrt(2) * domain_size / max_edge_len), dtype=np.uint64)
    coords, cells = unit_cube(int(n[0]), int(n[1]), int(n[2]))
    coords = coords * domain_size
    coords = coords - domain_size / 2
    return coords, cells


def inscribed_tet():
    """sucemfem/Testing/Meshes.py:25-47."""
    coords = np.array([[-0.5, 0.5, -0.5], [0.5, 0.5, 0.5], [0.5, -0.5, -0.5],
                       [-0.5, -0.5, 0.5], [1. / 6, 1. / 6, -1. / 6],
                       [-1. / 6, 1. / 6, 1. / 6], [-1. / 6, -1. / 6, -1. / 6],
                       [1. / 6, -1. / 6, 1. / 6]])
    cells = np.array([[1, 4, 6, 7], [1, 3, 5, 7], [3, 4, 7, 8], [1, 2, 5, 6],
                      [2, 3, 5, 8], [2, 4, 6, 8], [4, 6, 7, 8], [1, 5, 6, 7],
                      [3, 5, 7, 8], [2, 5, 6, 8], [5, 6, 7, 8]]) - 1
    return coords, np.sort(cells, axis=1)


def jitter_interior(coords, cells, h, frac, seed):
    """Move interior vertices by uniform(-frac*h, frac*h) per coordinate."""
    rng = np.random.default_rng(seed)
    topo = Topology(cells)
    bverts = np.unique(topo.faces[topo.exterior_faces()].ravel())
    d = rng.uniform(-frac * h, frac * h, size=coords.shape)
    d[bverts] = 0.0
    return coords + d


# --------------------------------------------------------------------------
# topology and DOF map
# --------------------------------------------------------------------------
def _first_encounter(keys):
    """Number unique keys in order of first appearance."""
    uniq, first, inv = np.unique(keys, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")
    rank = np.empty_like(order)
    rank[order] = np.arange(len(order))
    return rank[inv].reshape(-1), len(uniq), uniq[order]


class Topology:
    def __init__(self, cells):
        cells = np.asarray(cells, dtype=np.int64)
        assert np.all(np.diff(cells, axis=1) > 0), "cells must be ordered"
        self.cells = cells
        nt = len(cells)
        nv = int(cells.max()) + 1
        ev = cells[:, EDGES]                      # (nt, 6, 2)
        ekey = ev[..., 0] * nv + ev[..., 1]
        eid, ne, ukeys = _first_encounter(ekey.ravel())
        self.cell_edges = eid.reshape(nt, 6)
        self.edges = np.stack([ukeys // nv, ukeys % nv], axis=1)
        fv = cells[:, FACES]                      # (nt, 4, 3)
        fkey = (fv[..., 0] * nv + fv[..., 1]) * nv + fv[..., 2]
        fid, nf, ufk = _first_encounter(fkey.ravel())
        self.cell_faces = fid.reshape(nt, 4)
        self.faces = np.stack([ufk // (nv * nv), (ufk // nv) % nv, ufk % nv], axis=1)
        self.nv, self.ne, self.nf, self.nt = nv, ne, nf, nt

    def exterior_faces(self):
        cnt = np.bincount(self.cell_faces.ravel(), minlength=self.nf)
        return np.nonzero(cnt == 1)[0]

    def exterior_facets(self):
        """(cell, local face) pairs for every exterior facet."""
        cnt = np.bincount(self.cell_faces.ravel(), minlength=self.nf)
        c, lf = np.nonzero(cnt[self.cell_faces] == 1)
        return c, lf


def dofmap(topo, order):
    """Cell DOF map of degree ``order``: k DOFs per edge (k*edge + j), then
    k(k-1) per face, then k(k-1)(k-2)/2 per cell interior, entity by entity
    (orders 1 and 2 are the FFC layouts above; orders 3 and 4 continue the
    same entity-major pattern, their interior DOFs being cell-local)."""
    if order not in (1, 2, 3, 4):
        raise ValueError("order must be 1, 2, 3 or 4")
    k = order
    de, df, dc = k, k * (k - 1), k * (k - 1) * (k - 2) // 2
    face0 = de * topo.ne
    cell0 = face0 + df * topo.nf
    nd = 6 * de + 4 * df + dc
    dm = np.empty((topo.nt, nd), dtype=np.int64)
    for j in range(de):
        dm[:, j:6 * de:de] = de * topo.cell_edges + j
    for j in range(df):
        dm[:, 6 * de + j:6 * de + 4 * df:df] = face0 + df * topo.cell_faces + j
    for j in range(dc):
        dm[:, 6 * de + 4 * df + j] = cell0 + dc * np.arange(topo.nt) + j
    return dm, cell0 + dc * topo.nt


def sparsity(dm, n):
    """Cell-pair CSR pattern (indptr, indices) with sorted columns."""
    nd = dm.shape[1]
    r = np.repeat(dm, nd, axis=1).ravel()
    c = np.tile(dm, (1, nd)).ravel()
    key = np.unique(r * n + c)
    rows = key // n
    cols = key % n
    indptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(indptr, rows + 1, 1)
    indptr = np.cumsum(indptr)
    return indptr, cols


# --------------------------------------------------------------------------
# element matrices
# --------------------------------------------------------------------------
_SYM = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]


def _sym6(K):
    """(n,n,3,3) -> (6,n,n) weights for the 6 unique entries of a symmetric metric."""
    out = []
    for p, q in _SYM:
        out.append(K[:, :, p, q] if p == q else K[:, :, p, q] + K[:, :, q, p])
    return np.array(out)


def geometry(coords, cells):
    x = coords[cells]                                  # (nt,4,3)
    J = np.stack([x[:, 1] - x[:, 0], x[:, 2] - x[:, 0], x[:, 3] - x[:, 0]], axis=2)  # columns
    det = np.linalg.det(J)
    Jinv = np.linalg.inv(J)
    return J, det, Jinv


def _metric6(G):
    return np.stack([G[:, p, q] for p, q in _SYM], axis=1)   # (nt,6)


def element_matrices(coords, cells, order, eps_r, mu_r):
    """Dense element matrices S_e, T_e: (nt, nd, nd)."""
    R = n1curl_exact.reference_tensors(order)
    Km = _sym6(R["mass"])
    Kc = _sym6(R["curl"])
    J, det, Jinv = geometry(coords, cells)
    adet = np.abs(det)
    Gt = np.einsum("cpi,cqi->cpq", Jinv, Jinv) * adet[:, None, None]     # |det| J^-1 J^-T
    Gs = np.einsum("cip,ciq->cpq", J, J) / adet[:, None, None]           # J^T J / |det|
    T = np.einsum("ck,kab->cab", _metric6(Gt), Km) * np.asarray(eps_r)[:, None, None]
    S = np.einsum("ck,kab->cab", _metric6(Gs), Kc) / np.asarray(mu_r)[:, None, None]
    return S, T


def facet_matrices(coords, cells, order, fc, flf):
    """ABC element contributions for exterior facets (cell fc, local face flf)."""
    R = n1curl_exact.reference_tensors(order)
    Kf = np.array([_sym6(R["face"][f]) for f in range(4)])   # (4,6,nd,nd)
    J, det, Jinv = geometry(coords, cells[fc])
    fv = cells[fc][np.arange(len(fc))[:, None], FACES[flf]]  # (m,3) global vertex ids
    p = coords[fv]
    cr = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    two_area = np.linalg.norm(cr, axis=1)
    n = cr / two_area[:, None]
    P = np.eye(3)[None] - n[:, :, None] * n[:, None, :]
    H = np.einsum("cpi,cij,cqj->cpq", Jinv, P, Jinv) * two_area[:, None, None]
    return np.einsum("ck,ckab->cab", _metric6(H), Kf[flf])


# --------------------------------------------------------------------------
# global assembly
# --------------------------------------------------------------------------
class Assembled:
    pass


def assemble(coords, cells, order, eps_r=None, mu_r=None, with_abc=True):
    """Assemble S, T (and B) on the DOLFIN cell-pair pattern.  Returns an
    object with csr matrices S, T, B (B None when with_abc is False), the
    topology, dof map and pattern."""
    coords = np.asarray(coords, dtype=np.float64)
    cells = np.sort(np.asarray(cells, dtype=np.int64), axis=1)
    nt = len(cells)
    eps_r = np.ones(nt) if eps_r is None else np.asarray(eps_r, dtype=np.float64)
    mu_r = np.ones(nt) if mu_r is None else np.asarray(mu_r, dtype=np.float64)
    topo = Topology(cells)
    dm, n = dofmap(topo, order)
    indptr, indices = sparsity(dm, n)
    nd = dm.shape[1]
    Se, Te = element_matrices(coords, cells, order, eps_r, mu_r)
    rows = np.repeat(dm, nd, axis=1).reshape(nt, nd, nd)
    cols = np.tile(dm, (1, nd)).reshape(nt, nd, nd)
    # position of (row, col) in the CSR arrays
    keyp = np.repeat(np.arange(n), np.diff(indptr)) * n + indices
    def to_csr(vals, r, c):
        pos = np.searchsorted(keyp, (r * n + c).ravel())
        data = np.zeros(len(indices))
        np.add.at(data, pos, vals.ravel())
        return sps.csr_matrix((data, indices.astype(np.int32), indptr.astype(np.int32)), shape=(n, n))
    out = Assembled()
    out.S = to_csr(Se, rows, cols)
    out.T = to_csr(Te, rows, cols)
    out.B = None
    if with_abc:
        fc, flf = topo.exterior_facets()
        Be = facet_matrices(coords, cells, order, fc, flf)
        out.B = to_csr(Be, rows[fc], cols[fc])
    out.topo, out.dofmap, out.n = topo, dm, n
    out.indptr, out.indices = indptr, indices
    out.order = order
    return out


def pec_dofs(topo, order):
    """DOFs on the closure of exterior facets (DirichletBC on DomainBoundary)."""
    fc, flf = topo.exterior_facets()
    fv = topo.cells[fc][np.arange(len(fc))[:, None], FACES[flf]]
    # local edges of each face: edges among the face vertices
    ev = topo.cells[:, EDGES]
    edge_set = set()
    for c, lf in zip(fc, flf):
        verts = set(topo.cells[c][list(FACES[lf])])
        for le in range(6):
            if set(ev[c, le]) <= verts:
                edge_set.add(int(topo.cell_edges[c, le]))
    edges = np.array(sorted(edge_set), dtype=np.int64)
    faces = np.unique(topo.cell_faces[fc, flf]).astype(np.int64)
    k = order
    de, df = k, k * (k - 1)
    parts = [de * edges + j for j in range(de)] + [de * topo.ne + df * faces + j for j in range(df)]
    return np.sort(np.concatenate(parts))


def apply_pec(A, dofs):
    """Zero the rows of ``dofs`` keeping the pattern, unit diagonal."""
    A = A.copy()
    for r in dofs:
        lo, hi = A.indptr[r], A.indptr[r + 1]
        A.data[lo:hi] = 0.0
        k = lo + np.searchsorted(A.indices[lo:hi], r)
        A.data[k] = 1.0
    return A


def lhs_matrix(S, T, B, frequency):
    """EMDrivenProblem.py:67-72, with scipy's own sparse arithmetic."""
    k0 = 2 * np.pi * frequency / C0
    return S - k0 ** 2 * T + 1j * k0 * B


# --------------------------------------------------------------------------
# sources
# --------------------------------------------------------------------------
def locate_cells(coords, cells, pts, tol=1e-12):
    """Candidate cells containing each point (barycentric test with tol)."""
    J, det, Jinv = geometry(coords, cells)
    out = []
    for p in np.atleast_2d(pts):
        X = np.einsum("cij,cj->ci", Jinv, p[None] - coords[cells[:, 0]])
        lam = np.concatenate([1 - X.sum(1, keepdims=True), X], axis=1)
        out.append(np.nonzero(np.all(lam >= -tol, axis=1))[0])
    return out


def basis_at(coords, cells, order, c, p):
    """Physical basis values (nd, 3) of cell c at point p."""
    fb, _ = n1curl_exact.basis_lambdas(order)
    J, det, Jinv = geometry(coords, cells[c:c + 1])
    X = Jinv[0] @ (np.asarray(p) - coords[cells[c, 0]])
    Nh = np.array([[float(v) for v in comp] for comp in fb(*X)])   # (nd,3)
    return Nh @ Jinv[0]          # rows: J^-T N_hat  == N_hat^T J^-1


def point_source_contrib(coords, cells, order, topo, dm, p, value, choose=min, cands=None):
    """point_source.py:49-94: (dofnos, N_i(p).value) for the cell chosen by
    ``choose`` among the cells that contain p (``cands``: those cells, when
    already located)."""
    if cands is None:
        cands = locate_cells(coords, cells, p)[0]
    if len(cands) == 0:
        raise ValueError("source point outside the mesh")
    c = int(choose(cands))
    vals = basis_at(coords, cells, order, c, p) @ np.asarray(value)
    return dm[c].copy(), vals


def fillament_contrib(coords, cells, order, topo, dm, endpoints, I, npts, choose=min):
    """fillament_current_source.py:62-82."""
    start, end = np.asarray(endpoints[0], float), np.asarray(endpoints[1], float)
    delta = end - start
    L = np.sqrt(np.sum(delta ** 2))
    vec = delta / L * I
    if npts == 1:
        pts = [start + delta * 0.5]
    else:
        pts = start + delta * np.linspace(0, 1, npts)[:, None]
    mag = vec * L / npts
    contribs = {}
    located = locate_cells(coords, cells, np.atleast_2d(pts))   # one geometry pass
    for p, cands in zip(pts, located):
        d, v = point_source_contrib(coords, cells, order, topo, dm, p, mag, choose, cands)
        for dn, vv in zip(d, v):
            contribs[int(dn)] = contribs.get(int(dn), 0.0) + vv
    dn = np.array(sorted(contribs))
    return dn, np.array([contribs[k] for k in dn])


def rhs_vector(n, frequency, dofnos, contribs):
    """EMDrivenProblem.py:74-80."""
    RHS = np.zeros(n, np.complex128)
    k0 = 2 * np.pi * frequency / C0
    RHS[dofnos] += -1j * k0 * Z0 * np.asarray(contribs)
    return RHS
