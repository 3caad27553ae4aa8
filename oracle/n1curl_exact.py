"""Exact (rational) N1curl reference element for the oracle.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module; it
is part of the oracle the GPU path is compared against.

Restates the Nedelec first-kind H(curl) element that the reference obtains
from FIAT through ``dolfin.FunctionSpace(mesh, "Nedelec 1st kind H(curl)",
order)`` (sucemfem/ProblemConfigurations/EMProblem.py:36,104-105).  FIAT is
an un-vendored dependency with no pinned version (the API era of the
reference is DOLFIN/FFC/FIAT 0.9.x-1.0); its published definition of the
element is restated here:

* reference cell: the UFC tetrahedron (0,0,0),(1,0,0),(0,1,0),(0,0,1),
  edges in UFC order (2,3),(1,3),(1,2),(0,3),(0,2),(0,1), face i opposite
  vertex i, face vertices in increasing local order;
* space of degree k: P_{k-1}^3 + x cross (homogeneous P_{k-1})^3;
* dual basis: tangential point evaluations u(p).t on every edge at the
  interior points of a lattice with k+1 intervals (t = v1 - v0 of the edge,
  not normalised), then for k >= 2 two tangential evaluations per face at
  the interior lattice points (tangents v1-v0 and v2-v0 of the face), then
  for k >= 3 the three Cartesian components at every interior point of the
  cell lattice (cell-local DOFs: any fixed order is a valid convention);
* physical basis through the covariant Piola map N = J^-T N_hat.

For orders 1 and 2 the basis is computed in exact rational arithmetic with
sympy, the reference tensors by exact-degree Gauss quadrature of it; the
result is pinned against the reference's golden fixtures by
tests/test_oracle_golden.py.  Orders 3 and 4 use an independent float64
construction (``numeric_basis``); their pins are the reference's own
higher-order functional tests (cavity eigenvalues,
functional_tests/test_EigenProblems.py:86,150), run on this oracle in
tests/test_high_order_cpu.py.
"""
from functools import lru_cache

import sympy as sp

X, Y, Z = sp.symbols("x y z")
XYZ = (X, Y, Z)

REF_VERTS = [sp.Matrix([0, 0, 0]), sp.Matrix([1, 0, 0]),
             sp.Matrix([0, 1, 0]), sp.Matrix([0, 0, 1])]
# UFC local edge and face numbering of a tetrahedron
EDGES = [(2, 3), (1, 3), (1, 2), (0, 3), (0, 2), (0, 1)]
FACES = [(1, 2, 3), (0, 2, 3), (0, 1, 3), (0, 1, 2)]


def _span(order):
    """Spanning set of N1curl_order: P_{k-1}^3 + x cross homog P_{k-1}^3."""
    k = order
    out = []
    monos_full = [X**a * Y**b * Z**c for a in range(k) for b in range(k)
                  for c in range(k) if a + b + c <= k - 1]
    for m in monos_full:
        for d in range(3):
            v = [0, 0, 0]
            v[d] = m
            out.append(sp.Matrix(v))
    monos_h = [X**a * Y**b * Z**c for a in range(k) for b in range(k)
               for c in range(k) if a + b + c == k - 1]
    xv = sp.Matrix([X, Y, Z])
    for m in monos_h:
        for d in range(3):
            q = [0, 0, 0]
            q[d] = m
            out.append(xv.cross(sp.Matrix(q)))
    return out


def _lattice_edge(a, b, n):
    va, vb = REF_VERTS[a], REF_VERTS[b]
    return [va + sp.Rational(i, n) * (vb - va) for i in range(1, n)]


def _lattice_face(a, b, c, n):
    va, vb, vc = REF_VERTS[a], REF_VERTS[b], REF_VERTS[c]
    pts = []
    for j in range(1, n):
        for i in range(1, n - j):
            pts.append(va + sp.Rational(i, n) * (vb - va) + sp.Rational(j, n) * (vc - va))
    return pts


def dof_functionals(order):
    """List of (point, tangent) pairs; DOF = u(point) . tangent."""
    n = order + 1
    dofs = []
    for (a, b) in EDGES:
        t = REF_VERTS[b] - REF_VERTS[a]
        for p in _lattice_edge(a, b, n):
            dofs.append((p, t))
    if order >= 2:
        for (a, b, c) in FACES:
            t0 = REF_VERTS[b] - REF_VERTS[a]
            t1 = REF_VERTS[c] - REF_VERTS[a]
            for p in _lattice_face(a, b, c, n):
                dofs.append((p, t0))
                dofs.append((p, t1))
    if order >= 3:
        # interior points, the three Cartesian components each
        for l in range(1, n):
            for j in range(1, n - l):
                for i in range(1, n - l - j):
                    p = sp.Matrix([sp.Rational(i, n), sp.Rational(j, n), sp.Rational(l, n)])
                    for d in range(3):
                        e = [0, 0, 0]
                        e[d] = 1
                        dofs.append((p, sp.Matrix(e)))
    return dofs


def _eval(v, p):
    return v.subs({X: p[0], Y: p[1], Z: p[2]})


@lru_cache(maxsize=None)
def basis(order):
    """Nodal (dual) basis on the reference tet, as a list of sympy 3-vectors."""
    span = _span(order)
    # independent subset of the spanning set
    polys = []
    monos = set()
    for v in span:
        for comp in v:
            monos.update(sp.Poly(comp, *XYZ).monoms())
    monos = sorted(monos)
    rows = []
    for v in span:
        row = []
        for comp in v:
            pc = sp.Poly(comp, *XYZ)
            row.extend(pc.coeff_monomial(m) for m in monos)
        rows.append(row)
    M = sp.Matrix(rows)
    _, piv = M.T.rref()
    indep = [span[i] for i in piv]
    dofs = dof_functionals(order)
    assert len(indep) == len(dofs), (len(indep), len(dofs))
    D = sp.Matrix(len(dofs), len(indep),
                  lambda i, j: (_eval(indep[j], dofs[i][0]).T * dofs[i][1])[0])
    C = D.inv()
    out = []
    for i in range(len(dofs)):
        v = sp.zeros(3, 1)
        for j in range(len(indep)):
            v += C[j, i] * indep[j]
        out.append(sp.simplify(v))
    return out


def curl(v):
    return sp.Matrix([sp.diff(v[2], Y) - sp.diff(v[1], Z),
                      sp.diff(v[0], Z) - sp.diff(v[2], X),
                      sp.diff(v[1], X) - sp.diff(v[0], Y)])


def _gauss_tet(npts=6):
    """Collapsed (Duffy) Gauss-Legendre rule on the reference tet, exact to
    polynomial degree 2*npts-3 in x,y,z."""
    import numpy as np
    g, w = np.polynomial.legendre.leggauss(npts)
    g = 0.5 * (g + 1.0)
    w = 0.5 * w
    U, V, W = np.meshgrid(g, g, g, indexing="ij")
    WU, WV, WW = np.meshgrid(w, w, w, indexing="ij")
    x = U
    y = V * (1 - U)
    z = W * (1 - U) * (1 - V)
    wt = WU * WV * WW * (1 - U) ** 2 * (1 - V)
    return np.stack([x.ravel(), y.ravel(), z.ravel()]), wt.ravel()


def _gauss_tri(npts=6):
    """Collapsed Gauss-Legendre rule on the unit triangle in (s,t)."""
    import numpy as np
    g, w = np.polynomial.legendre.leggauss(npts)
    g = 0.5 * (g + 1.0)
    w = 0.5 * w
    U, V = np.meshgrid(g, g, indexing="ij")
    WU, WV = np.meshgrid(w, w, indexing="ij")
    s = U
    t = V * (1 - U)
    wt = WU * WV * (1 - U)
    return s.ravel(), t.ravel(), wt.ravel()


# ---- orders 3 and 4: float64 construction (sympy is too slow there) ----
def _monos(deg):
    return [(a, b, c) for a in range(deg + 1) for b in range(deg + 1 - a) for c in range(deg + 1 - a - b)]


@lru_cache(maxsize=None)
def numeric_basis(order):
    """Reference basis of degree ``order`` in float64: coefficients
    coef[a, p, m] of component p of basis function a over the monomials
    _monos(order)[m].  The space P_{k-1}^3 + x cross homog P_{k-1}^3 is
    spanned by an orthonormal basis of its coefficient vectors (SVD), then
    made dual to ``dof_functionals`` by inverting the functional matrix."""
    import numpy as np
    k = order
    mons = _monos(k)
    idx = {m: i for i, m in enumerate(mons)}
    nm = len(mons)
    vecs = []
    for m in mons:
        if sum(m) <= k - 1:
            for d in range(3):
                v = np.zeros((3, nm))
                v[d, idx[m]] = 1.0
                vecs.append(v)
    for m in mons:
        if sum(m) == k - 1:
            for d in range(3):
                # x cross (e_d m): component i gets eps_{i j d} x_j m
                v = np.zeros((3, nm))
                for i in range(3):
                    for j in range(3):
                        eps = np.linalg.det(np.eye(3)[[i, j, d]]) if len({i, j, d}) == 3 else 0.0
                        if eps:
                            e = list(m)
                            e[j] += 1
                            v[i, idx[tuple(e)]] += eps
                vecs.append(v)
    A = np.array(vecs).reshape(len(vecs), 3 * nm)
    _, sv, vt = np.linalg.svd(A, full_matrices=False)
    r = int((sv > 1e-10 * sv[0]).sum())
    span = vt[:r].reshape(r, 3, nm)
    dofs = dof_functionals(order)
    assert r == len(dofs), (r, len(dofs))
    P = np.array([[float(x) for x in p] for p, _ in dofs])
    T = np.array([[float(x) for x in t] for _, t in dofs])
    mv = np.array([[np.prod(np.asarray(p) ** np.asarray(m)) for m in mons] for p in P])  # (n, nm)
    D = np.einsum("id,jdm,im->ij", T, span, mv)
    C = np.linalg.inv(D)           # basis_a = sum_j C[j, a] span_j
    return np.einsum("ja,jdm->adm", C, span), mons


def _numeric_eval(coef, mons, x, y, z):
    import numpy as np
    mv = np.array([x ** m[0] * y ** m[1] * z ** m[2] for m in mons])   # (nm, nq)
    return np.einsum("adm,mq->adq", coef, mv)


def _numeric_curl(coef, mons):
    import numpy as np
    idx = {m: i for i, m in enumerate(mons)}
    def deriv(c, d):
        out = np.zeros_like(c)
        for m, i in idx.items():
            if m[d] > 0:
                e = list(m)
                e[d] -= 1
                out[..., idx[tuple(e)]] += m[d] * c[..., i]
        return out
    cx = deriv(coef[:, 2], 1) - deriv(coef[:, 1], 2)
    cy = deriv(coef[:, 0], 2) - deriv(coef[:, 2], 0)
    cz = deriv(coef[:, 1], 0) - deriv(coef[:, 0], 1)
    return np.stack([cx, cy, cz], axis=1)


@lru_cache(maxsize=None)
def reference_tensors(order):
    """Reference tensors by exact-degree quadrature of the basis (exact
    sympy basis for orders 1-2, the float64 one of ``numeric_basis`` for
    orders 3-4).

    Returns numpy arrays
      'mass'[a,b,p,q]   = int_ref N_a,p N_b,q dX
      'curl'[a,b,p,q]   = int_ref curlN_a,p curlN_b,q dX
      'face'[f,a,b,p,q] = int_{face f, (s,t) measure} N_a,p N_b,q
    """
    import numpy as np
    if order >= 3:
        coef, mons = numeric_basis(order)
        ccoef = _numeric_curl(coef, mons)
        fb = lambda x, y, z: _numeric_eval(coef, mons, x, y, z)
        fc = lambda x, y, z: _numeric_eval(ccoef, mons, x, y, z)
        ev = lambda f, x, y, z: f(np.asarray(x, float), np.asarray(y, float), np.asarray(z, float))
    else:
        fb, fc = basis_lambdas(order)

        def ev(f, x, y, z):
            vals = f(x, y, z)
            return np.array([[np.broadcast_to(np.asarray(c, dtype=float), x.shape) for c in v]
                             for v in vals])
    pts, wt = _gauss_tet()
    Nv = ev(fb, *pts)            # (n, 3, nq)
    Cv = ev(fc, *pts)
    mass = np.einsum("apk,bqk,k->abpq", Nv, Nv, wt)
    cc = np.einsum("apk,bqk,k->abpq", Cv, Cv, wt)
    s, t, wf = _gauss_tri()
    faces = []
    for f in range(4):
        a, b, c = FACES[f]
        va, vb, vc = [np.array([float(q) for q in REF_VERTS[i]]) for i in (a, b, c)]
        xyz = va[:, None] + s[None] * (vb - va)[:, None] + t[None] * (vc - va)[:, None]
        Fv = ev(fb, *xyz)
        faces.append(np.einsum("apk,bqk,k->abpq", Fv, Fv, wf))
    return {"mass": mass, "curl": cc, "face": np.array(faces)}


@lru_cache(maxsize=None)
def basis_lambdas(order):
    """numpy-callable reference basis values and curls: f(x,y,z) -> list."""
    B = basis(order)
    fb = sp.lambdify(XYZ, [list(v) for v in B], "numpy")
    fc = sp.lambdify(XYZ, [list(curl(v)) for v in B], "numpy")
    return fb, fc
