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


def ntff(coords, cells, order, topo, dm, x, frequency, theta_deg, phi_deg, rule=None):
    """surface_ntff.py:120-155 NTFF.calc_pt for each direction:
    (E_theta, E_phi) arrays."""
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
    Et, Ep = [], []
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
    return np.array(Et), np.array(Ep)
