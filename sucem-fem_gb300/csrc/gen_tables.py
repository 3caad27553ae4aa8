"""Generate ``n1curl_tables.h`` (orders 1 and 2) and ``n1curl_tables_hi.h``
(orders 3 and 4): reference-element constants of the Nedelec first-kind
H(curl) element.

The element is the one the reference requests with
``dolfin.FunctionSpace(mesh, "Nedelec 1st kind H(curl)", order)``
(sucemfem/ProblemConfigurations/EMProblem.py:36,104-105), i.e. FIAT's
definition: UFC reference tetrahedron, space P_{k-1}^3 + x cross
homogeneous P_{k-1}^3, dual basis of tangential point evaluations on the
edges (interior lattice points of k+1 intervals, unnormalised tangent
v1-v0), for k >= 2 two tangential evaluations per interior face-lattice
point (tangents v1-v0, v2-v0 of the face; the centroid for k = 2) and for
k >= 3 the three components at every interior cell-lattice point (see
``dofs``).  Orders 3 and 4 carry only the assembly tables KC, KM, KT.

Everything is computed in exact rational arithmetic (``fractions``) with no
third-party package, so the same script runs on any host.  Written tables
(all ``double``; the kernels convert to float where needed), with the six
unique entries of a symmetric 3x3 metric ordered (00,11,22,01,02,12) and
off-diagonal weights symmetrised (K_pq + K_qp):

* ``KC<o>[6][n][n]``     int_ref curl N_a,p curl N_b,q
* ``KM<o>[6][n][n]``     int_ref N_a,p N_b,q
* ``KT<o>[4][3][n][n]``  tangential face tensors of reference face f with
                         edge vectors a = v1-v0, b = v2-v0 of the face:
                         int (N_a.a)(N_b.a), int (N_a.a)(N_b.b)+(N_a.b)(N_b.a),
                         int (N_a.b)(N_b.b) in the parameter measure ds dt.
                         The physical ABC block of face f is then
                         (|b|^2 KT[0] - (a.b) KT[1] + |a|^2 KT[2]) / |a x b|
                         with a, b the physical face edge vectors (tangential
                         components are exact, so off-face DOFs give exact 0).
* ``NB<o>[n][3][10]``    monomial coefficients of N_a,p in
                         1,x,y,z,x^2,y^2,z^2,xy,xz,yz (point sources)
* ``DUAL<o>[n][6]``      the dual functional of local DOF a: reference
                         point (0..2) and tangent (3..5), DOF(u) = u(p).t
                         (interpolation of expressions onto the space)
"""
from fractions import Fraction as F
from math import factorial
import os
import sys

VERTS = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)]
EDGES = [(2, 3), (1, 3), (1, 2), (0, 3), (0, 2), (0, 1)]
FACES = [(1, 2, 3), (0, 2, 3), (0, 1, 3), (0, 1, 2)]
SYM = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
MONO10 = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (2, 0, 0), (0, 2, 0),
          (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1)]


# ---- sparse polynomials: dict {exponent tuple: Fraction} -------------------
def padd(a, b, s=1):
    out = dict(a)
    for k, v in b.items():
        out[k] = out.get(k, 0) + s * v
    return {k: v for k, v in out.items() if v != 0}


def pmul(a, b):
    out = {}
    for ka, va in a.items():
        for kb, vb in b.items():
            k = tuple(x + y for x, y in zip(ka, kb))
            out[k] = out.get(k, 0) + va * vb
    return {k: v for k, v in out.items() if v != 0}


def pscale(a, s):
    return {k: v * s for k, v in a.items() if v * s != 0}


def pdiff(a, d):
    out = {}
    for k, v in a.items():
        if k[d] > 0:
            kk = list(k)
            kk[d] -= 1
            out[tuple(kk)] = out.get(tuple(kk), 0) + v * k[d]
    return out


def peval(a, pt):
    tot = F(0)
    for k, v in a.items():
        term = v
        for e, x in zip(k, pt):
            term *= F(x) ** e
        tot += term
    return tot


def mono(e):
    return {tuple(e): F(1)}


def int_tet(a):
    return sum(v * F(factorial(k[0]) * factorial(k[1]) * factorial(k[2]),
                     factorial(k[0] + k[1] + k[2] + 3)) for k, v in a.items())


def int_face(a, f):
    """Integral over reference face f in the parameter measure ds dt."""
    va, vb, vc = (VERTS[i] for i in FACES[f])
    # each coordinate as an affine polynomial in (s, t)
    coord = []
    for d in range(3):
        c = {}
        if va[d]:
            c[(0, 0)] = F(va[d])
        if vb[d] - va[d]:
            c[(1, 0)] = F(vb[d] - va[d])
        if vc[d] - va[d]:
            c[(0, 1)] = F(vc[d] - va[d])
        coord.append(c)
    tot = {}
    for k, v in a.items():
        term = {(0, 0): v}
        for d in range(3):
            for _ in range(k[d]):
                term = pmul(term, coord[d])
        tot = padd(tot, term)
    return sum(v * F(factorial(k[0]) * factorial(k[1]), factorial(k[0] + k[1] + 2))
               for k, v in tot.items())


# ---- element ---------------------------------------------------------------
def span(order):
    k = order
    vecs = []
    full = [(a, b, c) for a in range(k) for b in range(k) for c in range(k) if a + b + c <= k - 1]
    for m in full:
        for d in range(3):
            v = [{}, {}, {}]
            v[d] = mono(m)
            vecs.append(v)
    homog = [(a, b, c) for a in range(k) for b in range(k) for c in range(k) if a + b + c == k - 1]
    X = [mono((1, 0, 0)), mono((0, 1, 0)), mono((0, 0, 1))]
    for m in homog:
        for d in range(3):
            q = [{}, {}, {}]
            q[d] = mono(m)
            # x cross q
            vecs.append([padd(pmul(X[1], q[2]), pmul(X[2], q[1]), -1),
                         padd(pmul(X[2], q[0]), pmul(X[0], q[2]), -1),
                         padd(pmul(X[0], q[1]), pmul(X[1], q[0]), -1)])
    return vecs


def dofs(order):
    """FIAT's dual basis of the degree-k element as (point, vector) pairs,
    DOF(u) = u(point) . vector: tangential evaluations at the interior
    points of a (k+1)-interval lattice on every edge (tangent v1-v0), two
    per interior face-lattice point (face tangents v1-v0, v2-v0) for k >= 2,
    and the three Cartesian components at every interior cell-lattice point
    for k >= 3 (these are cell-local, so their order inside the cell is a
    local convention)."""
    n = order + 1
    out = []
    for a, b in EDGES:
        t = [VERTS[b][d] - VERTS[a][d] for d in range(3)]
        for i in range(1, n):
            out.append(([VERTS[a][d] + F(i, n) * t[d] for d in range(3)], t))
    if order >= 2:
        for a, b, c in FACES:
            t0 = [VERTS[b][d] - VERTS[a][d] for d in range(3)]
            t1 = [VERTS[c][d] - VERTS[a][d] for d in range(3)]
            for j in range(1, n):
                for i in range(1, n - j):
                    p = [VERTS[a][d] + F(i, n) * t0[d] + F(j, n) * t1[d] for d in range(3)]
                    out.append((p, t0))
                    out.append((p, t1))
    if order >= 3:
        for l in range(1, n):
            for j in range(1, n - l):
                for i in range(1, n - l - j):
                    for d in range(3):
                        e = [0, 0, 0]
                        e[d] = 1
                        out.append(([F(i, n), F(j, n), F(l, n)], e))
    return out


def solve(A, B):
    """Exact Gauss-Jordan: solve A X = B (lists of Fractions)."""
    n = len(A)
    M = [list(A[i]) + list(B[i]) for i in range(n)]
    for c in range(n):
        p = next(r for r in range(c, n) if M[r][c] != 0)
        M[c], M[p] = M[p], M[c]
        piv = M[c][c]
        M[c] = [x / piv for x in M[c]]
        for r in range(n):
            if r != c and M[r][c] != 0:
                f = M[r][c]
                M[r] = [x - f * y for x, y in zip(M[r], M[c])]
    return [row[n:] for row in M]


def independent(vecs):
    """Greedy independent subset of vector polynomials."""
    keys = sorted({(d, k) for v in vecs for d in range(3) for k in v[d]})
    basis_rows, chosen = [], []
    for v in vecs:
        row = [v[d].get(k, F(0)) for d, k in keys]
        for piv_col, brow in basis_rows:
            if row[piv_col] != 0:
                f = row[piv_col] / brow[piv_col]
                row = [x - f * y for x, y in zip(row, brow)]
        nz = next((i for i, x in enumerate(row) if x != 0), None)
        if nz is not None:
            basis_rows.append((nz, row))
            chosen.append(v)
    return chosen


def basis(order):
    phis = independent(span(order))
    L = dofs(order)
    n = len(L)
    assert len(phis) == n
    D = [[sum(peval(phis[j][d], p) * t[d] for d in range(3)) for j in range(n)] for p, t in L]
    # N_i = sum_j C[j][i] phi_j with D C = I
    C = solve(D, [[F(int(i == j)) for j in range(n)] for i in range(n)])
    out = []
    for i in range(n):
        v = [{}, {}, {}]
        for j in range(n):
            if C[j][i] != 0:
                for d in range(3):
                    v[d] = padd(v[d], pscale(phis[j][d], C[j][i]))
        out.append(v)
    return out


def curl(v):
    return [padd(pdiff(v[2], 1), pdiff(v[1], 2), -1),
            padd(pdiff(v[0], 2), pdiff(v[2], 0), -1),
            padd(pdiff(v[1], 0), pdiff(v[0], 1), -1)]


def tables(order):
    N = basis(order)
    C = [curl(v) for v in N]
    n = len(N)

    def sym6(fn):
        out = [[[F(0)] * n for _ in range(n)] for _ in range(6)]
        for a in range(n):
            for b in range(n):
                for m, (p, q) in enumerate(SYM):
                    val = fn(a, b, p, q)
                    if p != q:
                        val += fn(a, b, q, p)
                    out[m][a][b] = val
        return out

    KC = sym6(lambda a, b, p, q: int_tet(pmul(C[a][p], C[b][q])))
    KM = sym6(lambda a, b, p, q: int_tet(pmul(N[a][p], N[b][q])))
    KT = []
    for f in range(4):
        va, vb, vc = (VERTS[i] for i in FACES[f])
        ta = [vb[d] - va[d] for d in range(3)]
        tb = [vc[d] - va[d] for d in range(3)]

        def tang(a, t):
            out = {}
            for d in range(3):
                if t[d]:
                    out = padd(out, pscale(N[a][d], F(t[d])))
            return out
        Na = [tang(a, ta) for a in range(n)]
        Nb = [tang(a, tb) for a in range(n)]
        aa = [[int_face(pmul(Na[a], Na[b]), f) for b in range(n)] for a in range(n)]
        ab = [[int_face(pmul(Na[a], Nb[b]), f) + int_face(pmul(Nb[a], Na[b]), f) for b in range(n)]
              for a in range(n)]
        bb = [[int_face(pmul(Nb[a], Nb[b]), f) for b in range(n)] for a in range(n)]
        KT.append([aa, ab, bb])
    NB = [[[N[a][p].get(e, F(0)) for e in MONO10] for p in range(3)] for a in range(n)]
    return KC, KM, KT, NB


def monos(deg):
    """Monomial exponents of total degree <= deg."""
    return [(a, b, s - a - b) for s in range(deg + 1) for a in range(s, -1, -1)
            for b in range(s - a, -1, -1)]


def matmul(A, B):
    Bt = list(zip(*B))
    return [[sum(x * y for x, y in zip(r, col) if x and y) for col in Bt] for r in A]


def tables_moments(order):
    """KC, KM, KT of any order through exact monomial moment matrices: with
    C the coefficients of the basis components over the monomials m_i and
    M_ij = int m_i m_j, every table is a product C M C^T (orders 1 and 2
    give exactly the tables of ``tables``)."""
    N = basis(order)
    n = len(N)
    Cu = [curl(v) for v in N]
    mN, mC = monos(order), monos(order - 1)

    def coef(polys, ms):
        idx = {m: i for i, m in enumerate(ms)}
        rows = []
        for v in polys:
            for p in range(3):
                r = [F(0)] * len(ms)
                for e, c in v[p].items():
                    r[idx[e]] = c
                rows.append(r)
        return rows  # row 3a + p

    def moments(ms):
        return [[F(factorial(a[0] + b[0]) * factorial(a[1] + b[1]) * factorial(a[2] + b[2]),
                   factorial(sum(a) + sum(b) + 3)) for b in ms] for a in ms]

    CN, CC = coef(N, mN), coef(Cu, mC)
    PN = matmul(matmul(CN, moments(mN)), [list(r) for r in zip(*CN)])
    PC = matmul(matmul(CC, moments(mC)), [list(r) for r in zip(*CC)])

    def sym6(P):
        out = [[[F(0)] * n for _ in range(n)] for _ in range(6)]
        for m, (p, q) in enumerate(SYM):
            for a in range(n):
                for b in range(n):
                    val = P[3 * a + p][3 * b + q]
                    if p != q:
                        val += P[3 * a + q][3 * b + p]
                    out[m][a][b] = val
        return out

    KT = []
    for f in range(4):
        va, vb, vc = (VERTS[i] for i in FACES[f])
        ta = [vb[d] - va[d] for d in range(3)]
        tb = [vc[d] - va[d] for d in range(3)]
        Mf = [[int_face(mono(tuple(x + y for x, y in zip(a, b))), f) for b in mN] for a in mN]
        Ta = [[sum(CN[3 * a + d][i] * ta[d] for d in range(3)) for i in range(len(mN))]
              for a in range(n)]
        Tb = [[sum(CN[3 * a + d][i] * tb[d] for d in range(3)) for i in range(len(mN))]
              for a in range(n)]
        TaM, TbM = matmul(Ta, Mf), matmul(Tb, Mf)
        TaT, TbT = [list(r) for r in zip(*Ta)], [list(r) for r in zip(*Tb)]
        ab1 = matmul(TaM, TbT)
        KT.append([matmul(TaM, TaT), [[ab1[a][b] + ab1[b][a] for b in range(n)] for a in range(n)],
                   matmul(TbM, TbT)])
    return sym6(PC), sym6(PN), KT


def _chain(terms):
    """Straight-line FMA chain for sum(coef * g[m]) over the nonzero terms
    (constants rounded to the kernel's type R at compile time)."""
    expr = None
    for m, c in terms:
        k = "R(%r)" % float(c)
        expr = "g[%d] * %s" % (m, k) if expr is None else "fma(g[%d], %s, %s)" % (m, k, expr)
    return expr


def _f32(x):
    """Nearest float32 of a Fraction (round half to even), as a Fraction."""
    import struct
    f = float(x)
    r = struct.unpack("f", struct.pack("f", f))[0]
    # struct rounds the double; fix double rounding by checking neighbours
    if r == 0.0:
        return F(0)
    cands = [r]
    for d in (-1, 1):
        b = struct.unpack("I", struct.pack("f", r))[0] + d
        c = struct.unpack("f", struct.pack("I", b & 0xFFFFFFFF))[0]
        if c == c and abs(c) != float("inf"):
            cands.append(c)
    return min((F(c) for c in cands), key=lambda c: (abs(c - x), c))


def _dot2(name, terms):
    """Compensated sum of coef * g[m] into Dot2 `name`: the float kernels
    get each constant as float hi + lo and add the products with error-free
    transformations, the double kernels a plain FMA chain."""
    parts = ["Dot2<R> %s;" % name]
    for m, c in terms:
        hi = _f32(c)
        parts.append("%s.add(g, %d, %r, %rf, %rf);" % (name, m, float(c), float(hi),
                                                       float(_f32(c - hi))))
    return " ".join(parts)


def contract_code():
    """Device code for the element-matrix rows of one local entity of an
    order-1 or order-2 cell, with the reference constants inlined (zero
    constants dropped):

      Rows<ORDER, FACE, LE>::fused(g, fn)  calls fn(j, b, v) with
          v = sum_m g[m] KC[m][a][b] + g[6 + m] KM[m][a][b]
      Rows<ORDER, FACE, LE>::split(g, fn)  calls fn(j, b, s, t) with the
          Dot2 sums s = sum_m g[m] KC[m][a][b], t = sum_m g[6 + m] KM[m][a][b]:
          compensated dot products.  In single precision the terms of an
          element entry can cancel (to a few percent of their size on
          regular meshes, to far less on jittered ones), and a plain FMA
          chain, or coefficients rounded to float, then loses the 1e-6
          relative accuracy the separate matrices are held to; the
          single-precision split form therefore takes g as 24 values (the 12
          coefficients rounded to float, then their rests) and hands each
          sum on unrounded (s.s + s.c) for a double-float accumulation

    for every column b of the cell and the entity's local DOFs a (j-th):
    edge LE of order k -> a = k*LE + j, face LE of order 2 -> a = 12 + 2*LE + j.
    The entity-per-lane assembly kernel calls them with the cell's metric
    coefficients g (12 values, S then T)."""
    out = ["// Generated by gen_tables.py: N1curl element-matrix rows of one local",
           "// entity with the reference constants inlined.  Do not edit; rerun the",
           "// generator.  See contract_code() in gen_tables.py for the contract.",
           "#pragma once", "", "namespace sucem {", "namespace contract {", "",
           "#ifdef __CUDA_ARCH__",
           "#define SUCEM_FMUL(a, b) __fmul_rn(a, b)",
           "#define SUCEM_FADD(a, b) __fadd_rn(a, b)",
           "#define SUCEM_FSUB(a, b) __fsub_rn(a, b)",
           "#else  // host builds of this header (tests) compile with -ffp-contract=off",
           "#define SUCEM_FMUL(a, b) ((a) * (b))",
           "#define SUCEM_FADD(a, b) ((a) + (b))",
           "#define SUCEM_FSUB(a, b) ((a) - (b))",
           "#endif",
           "",
           "// sum of g[m] * k over the added terms.  float: the coefficients come",
           "// as hi + lo pairs (g[m] + g[m + 12]) and so do the constants (kh the",
           "// nearest float of k, klo the rest); s + c is kept with every product",
           "// hi * kh split exactly (p + e) and every sum step exact (TwoSum), and",
           "// the small cross terms added to c; the intrinsics are never fused",
           "// into FMAs.  double: a plain FMA chain.",
           "template <class R>",
           "struct Dot2;",
           "template <>",
           "struct Dot2<float> {",
           "  float s = 0.f, c = 0.f;",
           "  __device__ __forceinline__ void add(const float* g, int m, double, float kh, float klo) {",
           "    const float gh = g[m], gl = g[m + 12];",
           "    const float p = SUCEM_FMUL(gh, kh);",
           "    const float e = fmaf(gh, kh, -p);",
           "    const float t = SUCEM_FADD(s, p);",
           "    const float z = SUCEM_FSUB(t, s);",
           "    const float d = SUCEM_FADD(SUCEM_FSUB(s, SUCEM_FSUB(t, z)), SUCEM_FSUB(p, z));",
           "    s = t;",
           "    c = fmaf(gh, klo, fmaf(gl, kh, SUCEM_FADD(c, SUCEM_FADD(d, e))));",
           "  }",
           "  __device__ __forceinline__ float sum() const { return SUCEM_FADD(s, c); }",
           "};",
           "template <>",
           "struct Dot2<double> {",
           "  double s = 0.0;",
           "  __device__ __forceinline__ void add(const double* g, int m, double k, float, float) {",
           "    s = fma(g[m], k, s);",
           "  }",
           "  __device__ __forceinline__ double sum() const { return s; }",
           "};",
           "",
           "template <int ORDER, bool FACE, int LE>", "struct Rows;", ""]
    for order in (1, 2):
        KC, KM, _, _ = tables(order)
        n = len(KC[0])
        kinds = [(False, 6)] + ([(True, 4)] if order == 2 else [])
        for face, nle in kinds:
            for le in range(nle):
                rows = ([12 + 2 * le, 13 + 2 * le] if face else
                        [order * le + j for j in range(order)])
                fused, split = [], []
                for j, a in enumerate(rows):
                    for b in range(n):
                        ts = [(m, KC[m][a][b]) for m in range(6) if KC[m][a][b] != 0]
                        tt = [(6 + m, KM[m][a][b]) for m in range(6) if KM[m][a][b] != 0]
                        if ts or tt:
                            fused.append("    fn(%d, %d, %s);" % (j, b, _chain(ts + tt)))
                        split.append("    { %s %s fn(%d, %d, sd, td); }" % (
                            _dot2("sd", ts), _dot2("td", tt), j, b))
                out += ["template <>",
                        "struct Rows<%d, %s, %d> {" % (order, "true" if face else "false", le),
                        "  template <class R, class Fn>",
                        "  static __device__ __forceinline__ void fused(const R* g, Fn&& fn) {"]
                out += fused
                out += ["  }", "  template <class R, class Fn>",
                        "  static __device__ __forceinline__ void split(const R* g, Fn&& fn) {"]
                out += split
                out += ["  }", "};", ""]
    out += ["}  // namespace contract", "}  // namespace sucem", ""]
    return "\n".join(out)


def _fmt(x, depth):
    if isinstance(x, list):
        inner = ",".join(_fmt(y, depth + 1) for y in x)
        return "{" + inner + "}" + ("\n" if depth <= 1 else "")
    return "0" if x == 0 else repr(float(x))


def main(path, path_hi, path_contract=None):
    lines = ["// Generated by gen_tables.py: N1curl reference-element constants.",
             "// Do not edit; rerun the generator.", "#pragma once", ""]
    for order in (1, 2):
        KC, KM, KT, NB = tables(order)
        n = len(NB)
        lines.append("static const double KC%d[6][%d][%d] = %s;" % (order, n, n, _fmt(KC, 0)))
        lines.append("static const double KM%d[6][%d][%d] = %s;" % (order, n, n, _fmt(KM, 0)))
        lines.append("static const double KT%d[4][3][%d][%d] = %s;" % (order, n, n, _fmt(KT, 0)))
        lines.append("static const double NB%d[%d][3][10] = %s;" % (order, n, _fmt(NB, 0)))
        DU = [[F(x) for x in p] + [F(x) for x in t] for p, t in dofs(order)]
        lines.append("static const double DUAL%d[%d][6] = %s;" % (order, n, _fmt(DU, 0)))
        lines.append("")
    with open(path, "w") as f:
        f.write("\n".join(lines))
    # orders 3 and 4: the assembly tables only (their own translation unit)
    lines = ["// Generated by gen_tables.py: N1curl reference-element constants of",
             "// orders 3 and 4.  Do not edit; rerun the generator.", "#pragma once", ""]
    for order in (3, 4):
        KC, KM, KT = tables_moments(order)
        n = len(KC[0])
        lines.append("static const double KC%d[6][%d][%d] = %s;" % (order, n, n, _fmt(KC, 0)))
        lines.append("static const double KM%d[6][%d][%d] = %s;" % (order, n, n, _fmt(KM, 0)))
        lines.append("static const double KT%d[4][3][%d][%d] = %s;" % (order, n, n, _fmt(KT, 0)))
        lines.append("")
    with open(path_hi, "w") as f:
        f.write("\n".join(lines))
    if path_contract:
        with open(path_contract, "w") as f:
            f.write(contract_code())


if __name__ == "__main__":
    here = os.path.dirname(os.path.abspath(__file__))
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(here, "n1curl_tables.h"),
         sys.argv[2] if len(sys.argv) > 2 else os.path.join(here, "n1curl_tables_hi.h"),
         sys.argv[3] if len(sys.argv) > 3 else os.path.join(here, "n1curl_contract.h"))
