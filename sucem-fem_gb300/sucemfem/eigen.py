"""Shift-invert Lanczos for S x = k^2 T x on the GPU, batched over
independent problems.

Replaces DefaultEigenSolver.solve_problem
(sucemfem/ProblemConfigurations/EMVectorWaveEigenproblem.py:61-105): the
reference factorises S - sigma*M with dolfin.LUSolver and runs ARPACK on
(S - sigma M)^-1 M, returning mu = 1/(k^2 - sigma).

Here, per problem (segment of a stacked vector):
  * the PEC-constrained DOFs are eliminated (with identity rows on both
    matrices the reference's pencil has a spurious k^2 = 1 per constrained
    DOF and S - sigma M is singular for sigma = 1);
  * K = S - sigma T is factorised once by the multifrontal LU in float32;
    each application of OP = K^-1 T does one float64 refinement step;
  * Lanczos in the T inner product with full (two-pass) reorthogonalisation
    in float64, all problems advanced together (one LU solve and segmented
    inner products per step);
  * the Ritz vectors of the nev largest mu (the smallest k^2 above sigma)
    are refined by a float64 Rayleigh-Ritz projection of (S, T).
The tridiagonal and the nev x nev projected problems are solved on the host
(as ARPACK's dense parts are)."""
import ctypes

import numpy as np
import scipy.linalg as sla
import torch

from . import _device, _native
from ._native import c_vp, call, ptr
from .lu import SparseLU
from .solvers import DeviceCSR, Vec

_native.declare("sucem_seg_dot", ctypes.c_int,
                [ctypes.c_int, c_vp, c_vp, ctypes.c_int64, ctypes.c_int, c_vp, c_vp, c_vp])
_native.declare("sucem_seg_axpy", ctypes.c_int,
                [ctypes.c_int, c_vp, ctypes.c_int64, c_vp, c_vp, ctypes.c_int64, ctypes.c_int, c_vp,
                 c_vp, c_vp, c_vp])
_native.declare("sucem_gather", ctypes.c_int, [ctypes.c_int64, ctypes.c_int, c_vp, c_vp, c_vp, c_vp])
_native.declare("sucem_combine", ctypes.c_int,
                [ctypes.c_int64, ctypes.c_int, ctypes.c_double, c_vp, ctypes.c_double, c_vp,
                 ctypes.c_double, c_vp, c_vp, ctypes.c_int, c_vp])


def reduced_pattern(indptr, indices, keep_order, device=None):
    """reduced_pattern on the GPU (torch index operations on ``device``),
    the same arrays returned as numpy: a stacked pattern of tens of millions
    of entries takes seconds through numpy on the host."""
    if device is None:
        return _reduced_pattern_host(indptr, indices, keep_order)
    n = len(indptr) - 1
    ip = torch.as_tensor(np.asarray(indptr, dtype=np.int64), device=device)
    ix = torch.as_tensor(np.asarray(indices, dtype=np.int64), device=device)
    ko = torch.as_tensor(np.asarray(keep_order, dtype=np.int64), device=device)
    new = torch.full((n,), -1, dtype=torch.int64, device=device)
    new[ko] = torch.arange(len(keep_order), device=device)
    nc = new[ix]
    rl = ip[1:] - ip[:-1]
    m = (nc >= 0) & torch.repeat_interleave(new >= 0, rl)
    q_all = torch.nonzero(m).squeeze(1)
    cz = torch.zeros(len(m) + 1, dtype=torch.int64, device=device)
    cz[1:] = torch.cumsum(m.to(torch.int64), 0)
    cnt = cz[ip[1:]] - cz[ip[:-1]]          # kept entries per old row
    start = cz[ip[:-1]]                      # their first position in q_all
    lens = cnt[ko]
    r_ip = torch.zeros(len(keep_order) + 1, dtype=torch.int64, device=device)
    r_ip[1:] = torch.cumsum(lens, 0)
    total = int(r_ip[-1])
    idx = torch.repeat_interleave(start[ko] - r_ip[:-1], lens) + torch.arange(total, device=device)
    q = q_all[idx]
    cols = nc[q]
    rows_new = torch.repeat_interleave(torch.arange(len(keep_order), device=device), lens)
    if total > 1 and not bool(((cols[1:] > cols[:-1]) | (rows_new[1:] != rows_new[:-1])).all()):
        key = rows_new * (len(keep_order) + 1) + cols
        order = torch.argsort(key)
        q, cols = q[order], cols[order]
    return (r_ip.cpu().numpy(), cols.to(torch.int32).cpu().numpy(), q.cpu().numpy(),
            new.cpu().numpy())


def _reduced_pattern_host(indptr, indices, keep_order):
    """CSR of the sub-matrix on the DOFs ``keep_order`` (old ids, in their new
    order).  Returns (indptr, indices, value_index into the full CSR)."""
    n = len(indptr) - 1
    indptr = np.asarray(indptr, dtype=np.int64)
    new = np.full(n, -1, dtype=np.int64)
    new[keep_order] = np.arange(len(keep_order))
    nc = new[indices]
    # kept entries of every old row, in their CSR order; the new rows are
    # the kept old rows in the new order, each row's entries a contiguous
    # run of q_all (gathered without a sort)
    kept_row = new >= 0
    m = nc >= 0
    m &= np.repeat(kept_row, np.diff(indptr))
    q_all = np.nonzero(m)[0]
    cnt = np.add.reduceat(m.astype(np.int64), indptr[:-1]) if len(m) else np.zeros(n, np.int64)
    cnt[np.diff(indptr) == 0] = 0  # reduceat takes the next element for empty rows
    start = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    lens = cnt[keep_order]
    r_ip = np.concatenate([[0], np.cumsum(lens)])
    idx = np.repeat(start[keep_order] - r_ip[:-1], lens) + np.arange(r_ip[-1])
    q = q_all[idx]
    cols = nc[q]
    # the new column ids keep the old order inside a row when the new
    # numbering is increasing in the old one over each row's columns (it is
    # for segment-contiguous reorderings of disjoint problems); else sort
    inrow = np.ones(len(cols), dtype=bool)
    inrow[r_ip[1:-1][lens[1:] > 0]] = False
    if len(cols) > 1 and not np.all((np.diff(cols) > 0) | ~inrow[1:]):
        rows_new = np.repeat(np.arange(len(keep_order)), lens)
        order = np.lexsort((cols, rows_new))
        q, cols = q[order], cols[order]
    return r_ip, cols.astype(np.int32), q.astype(np.int64), new


class BatchedShiftInvertLanczos:
    """Eigenpairs nearest above sigma for every problem of a stacked space.

    V: FunctionSpace (possibly several disjoint meshes); S, T: device float64
    values on V's pattern; constrained: DOFs to eliminate; dof_segment: the
    problem id of every DOF (None = one problem)."""

    def __init__(self, V, S, T, constrained, sigma, dof_segment=None, leaf_size=96):
        self.V = V
        self.sigma = float(sigma)
        n = V.n
        seg = np.zeros(n, dtype=np.int64) if dof_segment is None else np.asarray(dof_segment)
        free = np.ones(n, dtype=bool)
        free[np.asarray(constrained, dtype=np.int64)] = False
        keep = np.nonzero(free)[0]
        keep = keep[np.lexsort((keep, seg[keep]))]         # contiguous segments
        self.keep = keep
        self.nseg = int(seg.max()) + 1 if n else 0
        counts = np.bincount(seg[keep], minlength=self.nseg)
        self.seg_ptr_h = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        dev = _device.device()
        ip, ix, qidx, new = reduced_pattern(V.indptr, V.indices, keep, device=dev)
        self.n = len(keep)
        self.seg_ptr = torch.as_tensor(self.seg_ptr_h, device=dev)
        self.seg_of = torch.as_tensor(np.repeat(np.arange(self.nseg), counts).astype(np.int32), device=dev)
        self.qidx = torch.as_tensor(qidx, device=dev)
        self.ip, self.ix = ip, ix
        vals = {}
        for name, full in (("S", S), ("T", T)):
            v = torch.empty(len(qidx), dtype=torch.float64, device=dev)
            call("sucem_gather", len(qidx), 8, ptr(self.qidx), ptr(full), ptr(v), _device.stream_ptr())
            vals[name] = v
        K = torch.empty_like(vals["S"])
        call("sucem_combine", len(qidx), 8, 1.0, ptr(vals["S"]), -self.sigma, ptr(vals["T"]), 0.0,
             None, ptr(K), 0, _device.stream_ptr())
        self.S = DeviceCSR(ip, ix, vals["S"], self.n)
        self.T = DeviceCSR(self.S.indptr, self.S.indices, vals["T"], self.n)
        self.K = DeviceCSR(self.S.indptr, self.S.indices, K, self.n)
        cd = V.cell_dofs.astype(np.int64)
        cd_new = new[cd].astype(np.int32)
        cx = V.mesh().coordinates()[V.cells].mean(1)
        self.lu = SparseLU(ip, ix, leaf_size=leaf_size, cells=(cd_new, cx))
        self.vec = Vec()
        self.stats = {}

    # ---- segmented helpers ----
    def _segdot(self, X, y, nvec):
        out = torch.empty(nvec * self.nseg, dtype=torch.float64, device=y.device)
        call("sucem_seg_dot", self.nseg, ptr(self.seg_ptr), ptr(X), X.stride(0) if X.dim() > 1 else self.n,
             nvec, ptr(y), ptr(out), _device.stream_ptr())
        return out

    def _segaxpy(self, X, nvec, a, b, y):
        call("sucem_seg_axpy", self.nseg, ptr(self.seg_ptr), self.n, ptr(self.seg_of), ptr(X),
             X.stride(0) if X.dim() > 1 else self.n, nvec, ptr(a), ptr(b), ptr(y), _device.stream_ptr())

    def factor(self, precision="fp32"):
        if precision == "fp64":
            self.lu.factor(self.K.values, "f64")
        else:
            K32 = self.K.values.to(torch.float32)
            self.lu.factor(K32, "f32")
        self.precision = precision
        return self

    def _op(self, v, out):
        """out = K^-1 T v with one float64 refinement step."""
        tv = self.T.matvec(v)
        self.lu.solve(tv, out)
        if self.precision != "fp64":
            r = self.K.matvec(out)
            self.vec.axpby(1.0, tv, -1.0, r)       # r = tv - K out
            d = self.lu.solve(r)
            self.vec.axpby(1.0, d, 1.0, out)
        return out

    def solve(self, nev, ncv=None, tol=1e-10, maxiter=8, seed=0, precision="fp32"):
        """Returns (k2 (nseg, nev) float64, vectors (nseg, nev, n_free) on device
        in the reduced numbering)."""
        self.factor(precision)
        dev = _device.device()
        nseg, n = self.nseg, self.n
        sizes = np.diff(self.seg_ptr_h)
        m0 = int(min(max(2 * nev + 1, ncv or 0, nev + 20), sizes.min()))
        # convergence checks every 8 steps after the first m0 (each check is
        # one tridiagonal eigensolve per problem on the host, ~0.1 ms each;
        # a step is two LU solves of the stacked problem), up to maxiter
        # doublings of m0 or the smallest problem's size
        m_max = int(min(m0 * 2 ** (maxiter - 1), sizes.min()))
        checkpoints = list(range(m0, m_max + 1, 8))
        if checkpoints[-1] != m_max:
            checkpoints.append(m_max)
        res = self._lanczos(nev, checkpoints, seed)
        if res is None:
            raise RuntimeError("Lanczos did not converge within %d steps" % checkpoints[-1])
        Y, theta, m = res
        k2, Z = self._rayleigh_ritz(Y, nev)
        self.stats.update(m=m, theta=theta)
        return k2, Z

    def _lanczos(self, nev, checkpoints, seed):
        """One Lanczos run extended through the checkpoints until the nev
        wanted Ritz values of every segment have converged."""
        dev = _device.device()
        nseg, n = self.nseg, self.n
        m = checkpoints[-1]
        Vb = torch.empty((m + 1, n), dtype=torch.float64, device=dev)
        g = torch.Generator(device="cpu").manual_seed(seed)
        Vb[0].copy_(torch.rand(n, generator=g, dtype=torch.float64) - 0.5)
        nrm = self._segdot(Vb[0], self.T.matvec(Vb[0]), 1)
        self._segaxpy(Vb[0], 0, torch.zeros(1, device=dev, dtype=torch.float64), 1.0 / torch.sqrt(nrm),
                      Vb[0])
        alpha = np.zeros((nseg, m))
        beta = np.zeros((nseg, m))
        ones = torch.ones(nseg, dtype=torch.float64, device=dev)
        w = torch.empty(n, dtype=torch.float64, device=dev)
        for j in range(m):
            self._op(Vb[j], w)
            tw = self.T.matvec(w)
            h1 = self._segdot(Vb[:j + 1], tw, j + 1)
            self._segaxpy(Vb[:j + 1], j + 1, -h1, ones, w)
            tw = self.T.matvec(w)
            h2 = self._segdot(Vb[:j + 1], tw, j + 1)
            self._segaxpy(Vb[:j + 1], j + 1, -h2, ones, w)
            tw = self.T.matvec(w)
            bn = self._segdot(w, tw, 1)
            hh = (h1 + h2).view(j + 1, nseg).cpu().numpy()
            alpha[:, j] = hh[j]
            b = np.sqrt(np.maximum(bn.cpu().numpy(), 0.0))
            beta[:, j] = b
            inv = torch.as_tensor(np.where(b > 0, 1.0 / np.maximum(b, 1e-300), 0.0), device=dev)
            Vb[j + 1].zero_()
            self._segaxpy(w, 1, inv, torch.zeros(nseg, dtype=torch.float64, device=dev), Vb[j + 1])
            if j + 1 in checkpoints:
                done = self._ritz(nev, j + 1, alpha, beta, Vb)
                if done is not None:
                    return done[0], done[1], j + 1
        return None

    def _ritz(self, nev, m, alpha, beta, Vb):
        """Ritz values per segment after m steps; None unless all converged."""
        nseg, n = self.nseg, self.n
        coef = np.zeros((m, nseg * nev))
        thetas = np.zeros((nseg, nev))
        for s in range(nseg):
            th, Sv = sla.eigh_tridiagonal(alpha[s, :m], beta[s, :m - 1])
            idx = np.argsort(th)[::-1][:nev]           # largest mu = smallest k^2 above sigma
            resid = np.abs(beta[s, m - 1] * Sv[m - 1, idx])
            if np.any(resid > 1e-8 * np.maximum(np.abs(th[idx]), 1e-300)):
                return None
            thetas[s] = th[idx]
            for i, q in enumerate(idx):
                coef[:, i * nseg + s] = Sv[:, q]
        # Ritz vectors Y_i = sum_j coef[j, i] v_j (per segment)
        dev = Vb.device
        Y = torch.zeros((nev, n), dtype=torch.float64, device=dev)
        zeros = torch.zeros(nseg, dtype=torch.float64, device=dev)
        for i in range(nev):
            a = torch.as_tensor(np.ascontiguousarray(coef[:, i * nseg:(i + 1) * nseg]).ravel(), device=dev)
            self._segaxpy(Vb[:m], m, a, zeros, Y[i])
        return Y, thetas

    def _rayleigh_ritz(self, Y, nev):
        """float64 projection of (S, T) onto each segment's Ritz vectors."""
        nseg = self.nseg
        SY = torch.stack([self.S.matvec(Y[i]) for i in range(nev)])
        TY = torch.stack([self.T.matvec(Y[i]) for i in range(nev)])
        A = np.zeros((nseg, nev, nev))
        B = np.zeros((nseg, nev, nev))
        for k in range(nev):
            A[:, :, k] = self._segdot(Y, SY[k], nev).view(nev, nseg).cpu().numpy().T
            B[:, :, k] = self._segdot(Y, TY[k], nev).view(nev, nseg).cpu().numpy().T
        k2 = np.zeros((nseg, nev))
        coef = np.zeros((nev, nseg * nev))
        for s in range(nseg):
            As = 0.5 * (A[s] + A[s].T)
            Bs = 0.5 * (B[s] + B[s].T)
            w, C = sla.eigh(As, Bs)
            k2[s] = w
            for i in range(nev):
                coef[:, i * nseg + s] = C[:, i]
        Z = torch.zeros_like(Y)
        zeros = torch.zeros(nseg, dtype=torch.float64, device=Y.device)
        for i in range(nev):
            a = torch.as_tensor(np.ascontiguousarray(coef[:, i * nseg:(i + 1) * nseg]).ravel(),
                                device=Y.device)
            self._segaxpy(Y, nev, a, zeros, Z[i])
        return k2, Z

    def full_vectors(self, Z, seg=0):
        """(nev, n) complex128 host array: eigenvectors of segment ``seg`` in the
        original DOF numbering, zeros on constrained DOFs, unit 2-norm."""
        lo, hi = self.seg_ptr_h[seg], self.seg_ptr_h[seg + 1]
        Zh = Z[:, lo:hi].cpu().numpy()
        out = np.zeros((Z.shape[0], self.V.n), dtype=np.complex128)
        out[:, self.keep[lo:hi]] = Zh
        out /= np.linalg.norm(out, axis=1, keepdims=True)
        return out
