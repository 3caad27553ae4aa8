"""FP64 CPU restatement of the reference's field post-processing (the
oracle).

TEST INFRASTRUCTURE ONLY.  Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of bench.py import this module; the product never does.

What it restates, with the reference call sites it follows:

* ``Reconstruct.reconstruct_points`` (sucemfem/PostProcessing/
  PostProcessing.py:27-60): E(p) = sum_i x_i N_i(p) at arbitrary points
  (covariant Piola map of FIAT's N1curl basis);
* ``SurfaceFlux.calc_flux`` (sucemfem/PostProcessing/power_flux.py:11-60):
  the real power flux through the whole boundary,
  (1/(k0 Z0)) * int_{ds} n . (E_r x (-curl E_i / mu_r) + E_i x (curl E_r / mu_r))
  with the outward facet normal n; curl N_i by the contravariant Piola map.
  The integrand is a polynomial of degree <= 2*order - 1 on each facet; a
  3 x 3 collapsed Gauss rule integrates it exactly.
* ``NTFF.calc_pt`` (sucemfem/PostProcessing/surface_ntff.py:29-155): the
  equivalent currents J = n x H, H = j curl E / (k0 Z0) and M = -n x E
  radiated to (theta, phi): N = int J e^{j k0 r'.r_hat}, L likewise,
  E_theta = -r_fac (L_phi + Z0 N_theta), E_phi = r_fac (L_theta - Z0 N_phi),
  r_fac = j k0 e^{-j k0} / (4 pi).  The integrand is not polynomial; the
  facet rule is the 3 x 3 collapsed Gauss-Jacobi rule (Gauss-Jacobi
  alpha = 1 in the collapsed direction), which reproduces the reference's
  far fields to 5e-9 (a converged rule differs from them by 2e-8).
"""
import numpy as np

from . import fem, n1curl_exact

REF_VERTS = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])


def _basis(order, X):
    """Reference basis values and curls at reference points X (nq, 3):
    arrays (nd, 3, nq)."""
    fb, fc = n1curl_exact.basis_lambdas(order)
    def ev(f):
        vals = f(X[:, 0], X[:, 1], X[:, 2])
        return np.array([[np.broadcast_to(np.asarray(c, dtype=float), (len(X),)) for c in v]
                         for v in vals])
    return ev(fb), ev(fc)


def reconstruct_points(coords, cells, order, dm, x, pts, choose=min):
    """E at each point (npts, 3) complex; the cell containing a point is the
    one ``choose`` picks among the candidates (the GPU path takes the lowest
    index); points outside the mesh give NaN."""
    out = np.full((len(pts), 3), np.nan + 0j)
    cands = fem.locate_cells(coords, cells, pts)
    for i, p in enumerate(pts):
        if len(cands[i]) == 0:
            continue
        c = int(choose(cands[i]))
        N = fem.basis_at(coords, cells, order, c, p)       # (nd, 3) physical
        out[i] = np.asarray(x)[dm[c]] @ N
    return out


def surface_flux(coords, cells, order, topo, dm, x, k0, mu_r=None):
    """power_flux.py:11-60 SurfaceFlux.calc_flux over every exterior facet."""
    s, t, w = n1curl_exact._gauss_tri(3)
    fc_, lf_ = topo.exterior_facets()
    J, det, Jinv = fem.geometry(coords, cells[fc_])
    x = np.asarray(x)
    total = 0.0
    cache = {}
    for i in range(len(fc_)):
        c, lf = int(fc_[i]), int(lf_[i])
        if lf not in cache:
            a, b, d = fem.FACES[lf]
            X = (REF_VERTS[a][None] + s[:, None] * (REF_VERTS[b] - REF_VERTS[a])[None]
                 + t[:, None] * (REF_VERTS[d] - REF_VERTS[a])[None])
            cache[lf] = _basis(order, X)
        Nh, Ch = cache[lf]
        N = np.einsum("arq,ri->aiq", Nh, Jinv[i])              # J^-T N_hat
        C = np.einsum("ir,arq->aiq", J[i], Ch) / det[i]        # J curl N_hat / det J
        xe = x[dm[c]]
        E = np.einsum("a,aiq->iq", xe, N)
        CE = np.einsum("a,aiq->iq", xe, C)
        mur = 1.0 if mu_r is None else float(mu_r[c])
        v = coords[cells[c][fem.FACES[lf]]]
        cr = np.cross(v[1] - v[0], v[2] - v[0])
        if np.dot(cr, v[0] - coords[cells[c][lf]]) < 0:       # outward
            cr = -cr
        n = cr / np.linalg.norm(cr)
        Er, Ei, Cr, Ci = E.real, E.imag, CE.real, CE.imag
        f = np.einsum("i,iq->q", n, np.cross(Er, -Ci / mur, axis=0) + np.cross(Ei, Cr / mur, axis=0))
        total += np.sum(w * f) * np.linalg.norm(cr)
    return total / (k0 * fem.Z0)


def gauss_jacobi_tri(n=3):
    """Collapsed Gauss-Jacobi rule on the unit triangle: (s, t, w)."""
    import scipy.special as ssp
    xa, wa = ssp.roots_jacobi(n, 1.0, 0.0)
    xb, wb = ssp.roots_legendre(n)
    u = 0.5 * (xa[:, None] + 1.0) * np.ones((1, n))
    v = np.ones((n, 1)) * 0.5 * (xb[None, :] + 1.0)
    w = 0.125 * wa[:, None] * wb[None, :]
    return u.ravel(), (v * (1 - u)).ravel(), w.ravel()


def ntff(coords, cells, order, topo, dm, x, frequency, theta_deg, phi_deg, rule=None,
         full=False):
    """surface_ntff.py:120-155 NTFF.calc_pt for each direction:
    (E_theta, E_phi) arrays (full=True: also L_theta, L_phi, N_theta, N_phi)."""
    s, t, w = gauss_jacobi_tri(3) if rule is None else rule
    k0 = 2 * np.pi * frequency / fem.C0
    fc_, lf_ = topo.exterior_facets()
    J, det, Jinv = fem.geometry(coords, cells[fc_])
    x = np.asarray(x)
    cache = {}
    P, W, Jc, M = [], [], [], []
    for i in range(len(fc_)):
        c, lf = int(fc_[i]), int(lf_[i])
        if lf not in cache:
            a, b, d = fem.FACES[lf]
            X = (REF_VERTS[a][None] + s[:, None] * (REF_VERTS[b] - REF_VERTS[a])[None]
                 + t[:, None] * (REF_VERTS[d] - REF_VERTS[a])[None])
            cache[lf] = (_basis(order, X), X)
        (Nh, Ch), X = cache[lf]
        N = np.einsum("arq,ri->aiq", Nh, Jinv[i])
        C = np.einsum("ir,arq->aiq", J[i], Ch) / det[i]
        xe = x[dm[c]]
        E = np.einsum("a,aiq->iq", xe, N)
        CE = np.einsum("a,aiq->iq", xe, C)
        v = coords[cells[c][fem.FACES[lf]]]
        cr = np.cross(v[1] - v[0], v[2] - v[0])
        if np.dot(cr, v[0] - coords[cells[c][lf]]) < 0:
            cr = -cr
        n = cr / np.linalg.norm(cr)
        H = 1j * CE / (k0 * fem.Z0)
        P.append(coords[cells[c][0]][:, None] + J[i] @ X.T)
        W.append(w * np.linalg.norm(cr))
        Jc.append(np.cross(n[:, None], H, axis=0))
        M.append(-np.cross(n[:, None], E, axis=0))
    P, W = np.concatenate(P, axis=1), np.concatenate(W)
    Jc, M = np.concatenate(Jc, axis=1), np.concatenate(M, axis=1)
    Et, Ep, LN = [], [], []
    for th_d, ph_d in zip(np.atleast_1d(theta_deg), np.atleast_1d(phi_deg)):
        th, ph = np.deg2rad(th_d), np.deg2rad(ph_d)
        rhat = np.array([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)])
        thh = np.array([np.cos(th) * np.cos(ph), np.cos(th) * np.sin(ph), -np.sin(th)])
        phh = np.array([-np.sin(ph), np.cos(ph), 0.0])
        e = np.exp(1j * k0 * (rhat @ P)) * W
        Nv, Lv = Jc @ e, M @ e
        rf = 1j * k0 * np.exp(-1j * k0) / (4 * np.pi)
        Et.append(-rf * (phh @ Lv + fem.Z0 * (thh @ Nv)))
        Ep.append(rf * (thh @ Lv - fem.Z0 * (phh @ Nv)))
        LN.append([thh @ Lv, phh @ Lv, thh @ Nv, phh @ Nv])
    if full:
        LN = np.array(LN)
        return np.array(Et), np.array(Ep), LN[:, 0], LN[:, 1], LN[:, 2], LN[:, 3]
    return np.array(Et), np.array(Ep)


# --------------------------------------------------------------------------
# variational post-processing (CalcEMFunctional and its users)
# --------------------------------------------------------------------------
def boundary_edge_cells(topo):
    """Geometry.BoundaryEdgeCells (sucemfem/Geometry.py:76-90): cells that
    have an edge lying on the boundary (an edge of an exterior facet)."""
    fc, lf = topo.exterior_facets()
    bedges = set()
    for c, f in zip(fc, lf):
        verts = set(topo.cells[c][list(fem.FACES[f])])
        for le in range(6):
            if set(topo.cells[c][list(fem.EDGES[le])]) <= verts:
                bedges.add(int(topo.cell_edges[c, le]))
    be = np.zeros(topo.ne, dtype=bool)
    be[list(bedges)] = True
    return np.any(be[topo.cell_edges], axis=1)


def calc_em_functional(coords, cells, order, dm, E, g, k0, cell_mask=None, eps_r=None,
                       mu_r=None):
    """CalcEMFunctional.calc_functional (PostProcessing.py:62-173):
    int curl E . curl g / mu_r - k0^2 eps_r E . g over the marked cells
    (bilinear, no conjugation)."""
    nt = len(cells)
    eps = np.ones(nt) if eps_r is None else np.asarray(eps_r, dtype=float)
    mu = np.ones(nt) if mu_r is None else np.asarray(mu_r, dtype=float)
    S, T = fem.element_matrices(coords, cells, order, eps, mu)
    sel = np.arange(nt) if cell_mask is None else np.nonzero(cell_mask)[0]
    Ec, gc = np.asarray(E)[dm[sel]], np.asarray(g)[dm[sel]]
    A = S[sel] - k0 ** 2 * T[sel]
    return np.einsum("ca,cab,cb->", gc, A, Ec)


def variational_surface_flux(coords, cells, order, topo, dm, x, k0):
    """VariationalSurfaceFlux.calc_flux (power_flux.py:62-133): the functional
    over the boundary-edge cells with g = j conj(x_D) / (k0 Z0), x_D the DOF
    vector restricted to the boundary DOFs (DirichletBC of E on the domain
    boundary applied to a zero vector); the flux is its conjugate."""
    xd = np.zeros(len(x), dtype=complex)
    b = fem.pec_dofs(topo, order)
    xd[b] = np.asarray(x)[b]
    g = 1j * np.conj(xd) / k0 / fem.Z0
    return np.conj(calc_em_functional(coords, cells, order, dm, x, g, k0,
                                      boundary_edge_cells(topo)))


def dof_points_tangents(coords, cells, order, dm, dofs):
    """Physical point and tangent of each DOF's dual functional (the DOF of
    u is u(p) . t): the reference (point, tangent) of FIAT's N1curl dual
    basis mapped by the first cell holding the DOF (x = x0 + J X, t = J t)."""
    ref = n1curl_exact.dof_functionals(order)
    nd = dm.shape[1]
    owner = np.full(int(dm.max()) + 1, -1, dtype=np.int64)
    flat = dm.ravel()
    first = np.unique(flat, return_index=True)
    owner[first[0]] = first[1]
    idx = owner[np.asarray(dofs)]
    cell, loc = idx // nd, idx % nd
    J, det, Jinv = fem.geometry(coords, cells[cell])
    P = np.array([[float(v) for v in ref[l][0]] for l in loc])
    T = np.array([[float(v) for v in ref[l][1]] for l in loc])
    pts = coords[cells[cell, 0]] + np.einsum("cij,cj->ci", J, P)
    tans = np.einsum("cij,cj->ci", J, T)
    return pts, tans


def surface_interpolant(coords, cells, order, topo, dm, n, f):
    """SurfaceInterpolant.calculate_interpolation
    (sucemfem/Interpolation/Interpolation.py:26-82): the expression's DOFs
    (dual functionals) on the boundary DOFs, zero elsewhere.  f maps points
    (m, 3) to complex vectors (m, 3)."""
    b = fem.pec_dofs(topo, order)
    pts, tans = dof_points_tangents(coords, cells, order, dm, b)
    g = np.zeros(n, dtype=complex)
    g[b] = np.sum(tans * f(pts), axis=1)
    return g


def variational_ntff(coords, cells, order, topo, dm, x, frequency, theta_deg, phi_deg):
    """variational_ntff.py:68-131 NTFF.calc_pt: the H-field part by the
    functional over the boundary-edge cells with the plane-wave testing
    function g = interp(j/k0 rhat x (ahat x rhat) e^{j k0 rhat.r}), the
    E-field part L from the surface forms."""
    k0 = 2 * np.pi * frequency / fem.C0
    mask = boundary_edge_cells(topo)
    n = len(x)
    _, _, Lt, Lp, _, _ = ntff(coords, cells, order, topo, dm, x, frequency, theta_deg, phi_deg,
                              full=True)
    Et, Ep = [], []
    for i, (th_d, ph_d) in enumerate(zip(np.atleast_1d(theta_deg), np.atleast_1d(phi_deg))):
        th, ph = np.deg2rad(th_d), np.deg2rad(ph_d)
        rhat = np.array([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)])
        thh = np.array([np.cos(th) * np.cos(ph), np.cos(th) * np.sin(ph), -np.sin(th)])
        phh = np.array([-np.sin(ph), np.cos(ph), 0.0])
        EH = []
        for ahat in (thh, phh):
            cf = np.cross(rhat, np.cross(ahat, rhat)) / k0
            g = surface_interpolant(coords, cells, order, topo, dm, n,
                                    lambda p: 1j * cf[None] * np.exp(1j * k0 * (p @ rhat))[:, None])
            EH.append(calc_em_functional(coords, cells, order, dm, x, g, k0, mask))
        rf = 1j * k0 * np.exp(-1j * k0) / (4 * np.pi)
        Et.append(rf * (-Lp[i] + EH[0]))
        Ep.append(rf * (Lt[i] + EH[1]))
    return np.array(Et), np.array(Ep)
