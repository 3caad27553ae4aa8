"""Linear-system solvers with the interface of
sucemfem/Utilities/LinalgSolvers.py:30-322, running on the GPU.

* preconditioner 'ilu'  -> the GPU multifrontal LU of A (a complete
  factorisation; the reference's spilu(drop_tol=1e-8, fill_factor=10) is
  nearly complete too, and fails with "Factor is exactly singular" on the
  driven N1curl systems of this path);
* preconditioner 'diagonal' -> Jacobi; None -> no preconditioner;
* BiCGStabSolver / GMRESSolver: Krylov iterations on device vectors with
  the reference's per-iteration residual logging;
* UMFPACKSolver: direct solve by the GPU LU (+ double refinement).

FACTOR_PRECISION selects the LU precision: 'fp64' (default, the drop-in
numbers) or 'fp32' (complex64/float32 factor; the Krylov iteration then
refines in double precision).  The tolerance defaults to the reference's
old scipy default (1e-5 relative residual); set ``solver.tol``."""
import time

import numpy as np
import scipy.sparse
import torch

from .. import _device
from ..lu import SparseLU
from ..solvers import DeviceCSR, Vec

FACTOR_PRECISION = "fp64"


def _symmetric_pattern(A):
    """CSR with the structure of |A| + |A|^T (explicit zeros added) and the
    values of A; sorted columns."""
    A = scipy.sparse.csr_matrix(A)
    P = (abs(A) + abs(A).T).tocsr()
    P.sort_indices()
    rows = np.repeat(np.arange(P.shape[0]), np.diff(P.indptr))
    vals = np.asarray(A[rows, P.indices]).ravel() if P.nnz else np.zeros(0, A.dtype)
    return P.indptr.astype(np.int32), P.indices.astype(np.int32), vals.astype(A.dtype)


class _DeviceSystem:
    def __init__(self, A):
        self.n = A.shape[0]
        self.complex = np.iscomplexobj(A.data) if scipy.sparse.issparse(A) else np.iscomplexobj(A)
        ip, ix, vals = _symmetric_pattern(A)
        self.dtype = torch.complex128 if self.complex else torch.float64
        self.csr = DeviceCSR(ip, ix, torch.as_tensor(vals, device=_device.device()).to(self.dtype), self.n)
        self.ip, self.ix = ip, ix
        self.vec = Vec()
        self._lu = None

    def lu(self):
        if self._lu is None:
            self._lu = SparseLU(self.ip, self.ix, None, leaf_size=64)
            if FACTOR_PRECISION == "fp32":
                v = self.csr.values.to(torch.complex64 if self.complex else torch.float32)
                self._lu.factor(v, "c64" if self.complex else "f32")
            else:
                self._lu.factor(self.csr.values, "c128" if self.complex else "f64")
        return self._lu

    def to_dev(self, b):
        return torch.as_tensor(np.asarray(b, dtype=np.complex128 if self.complex else np.float64)
                               .reshape(-1), device=_device.device()).to(self.dtype)


class SystemSolverBase:
    tol = 1e-5
    maxiter = None

    def __init__(self, A, preconditioner_type=None):
        self._logging_data = {"time": [], "id": [], "res": []}
        self._user_callbacks = []
        self._timestamp("init")
        self._A = A
        self._sys = _DeviceSystem(A)
        self.set_preconditioner(preconditioner_type)
        self._callback_count = 0

    def _call_solver(self):
        raise Exception("Solver driver not implemented.")

    def add_user_callback(self, cb):
        self._user_callbacks.append(cb)

    def _callback(self, res):
        self._callback_count += 1
        self._timestamp(self._callback_count, res=res)

    def _timestamp(self, id, res=np.nan):
        self._logging_data["time"].append(time.time())
        self._logging_data["id"].append(id)
        self._logging_data["res"].append(res)
        for cb in self._user_callbacks:
            cb(self, res)

    def set_b(self, b):
        self._b = b

    def set_preconditioner(self, M_type):
        self._timestamp("preconditioner::start")
        self._M_type = M_type.lower() if isinstance(M_type, str) else None
        s = self._sys
        if M_type is None:
            self._M = None
        elif M_type.lower() == "diagonal":
            diag = np.asarray(scipy.sparse.csr_matrix(self._A).diagonal())
            inv = torch.as_tensor(1.0 / diag, device=_device.device()).to(s.dtype)
            self._M = lambda r, out, inv=inv: out.copy_(r * inv)
        elif M_type.lower() == "ilu":
            lu = s.lu()
            self._M = lambda r, out, lu=lu: lu.solve(r, out)
        else:
            print("Warning: Preconditioner type '%s' not recognised. Not using preconditioner." % M_type)
            self._M = None
        self._timestamp("preconditioner::end")

    def _apply_M(self, r, out):
        if self._M is None:
            return out.copy_(r)
        return self._M(r, out)

    def solve(self, b):
        self._timestamp("solve::begin")
        self.set_b(b)
        x, info = self._call_solver()
        self.info = info
        self._timestamp("solve::end")
        return x

    def get_logging_data(self):
        return self._logging_data

    def _get_time_for_id(self, id):
        return self._logging_data["time"][self._logging_data["id"].index(id)]

    def _get_elapsed_time(self, id0, id1, force_total=False):
        if force_total:
            return self._logging_data["time"][-1] - self._logging_data["time"][0]
        return self._get_time_for_id(id1) - self._get_time_for_id(id0)

    def print_logging_data(self):
        for k in self._logging_data:
            print(k)
            print(self._logging_data[k])

    def print_timing_info(self):
        print("solve time:", self._get_elapsed_time("solve::begin", "solve::end"))
        print("preconditioner time:",
              self._get_elapsed_time("preconditioner::start", "preconditioner::end"))
        print("total time:", self._get_elapsed_time(None, None, True))

    def plot_convergence(self, x_is_time=False, show_plot=False, label=None, style="-"):
        import pylab as P  # optional dependency, as in the reference
        y = np.log10(np.array(self._logging_data["res"], dtype=np.float64))
        idx = np.where(np.isfinite(y))[0]
        x = np.array([self._logging_data["id"][i] for i in idx]) if not x_is_time else \
            np.array(self._logging_data["time"])[idx] - self._logging_data["time"][0]
        P.plot(x, y[idx], style, label=label)
        P.grid(True)
        if show_plot:
            P.show()


class BiCGStabSolver(SystemSolverBase):
    """Preconditioned BiCGStab (right preconditioning) on the GPU, every
    scalar on the device (sucemfem.krylov): the host reads a status word
    once per batch of iterations (per iteration with the LU
    preconditioner), not once per dot product.  Real systems (whose LU is
    real) take the host-driven iteration of HostBiCGStabSolver.  The
    residual log gets the final relative residual (the iteration does not
    stop for the host)."""
    batch = 32

    def _call_solver(self):
        from ..krylov import bicgstab
        s = self._sys
        if not s.complex:
            return HostBiCGStabSolver._call_solver(self)
        b = s.to_dev(self._b)
        A = s.csr
        M = None
        if self._M is not None:
            M = s.lu() if self._M_type == "ilu" else "diagonal"
        x, info = bicgstab(A, b, precond=M, tol=self.tol, maxit=self.maxiter or 10 * s.n,
                           batch=self.batch)
        self._callback(info["residual"])
        self.info_device = info
        xh = x.cpu().numpy()
        if info["status"] == 1:
            return xh, 0
        if info["status"] == 2:
            return xh, info["iterations"]
        return xh, -10 if info["status"] == -1 else -11


class HostBiCGStabSolver(SystemSolverBase):
    """The same BiCGStab driven from the host (one synchronisation per dot
    product), kept as the cross-check of the device-resident solver."""

    def _call_solver(self):
        s = self._sys
        v = s.vec
        b = s.to_dev(self._b)
        n = s.n
        bn = v.norm(b)
        x = torch.zeros_like(b)
        if bn == 0:
            return x.cpu().numpy(), 0
        r = b.clone()
        rhat = r.clone()
        p = torch.zeros_like(b)
        vv = torch.zeros_like(b)
        phat = torch.empty_like(b)
        shat = torch.empty_like(b)
        rho = alpha = omega = 1.0
        maxit = self.maxiter or 10 * n
        for it in range(1, maxit + 1):
            rho_new = v.dot(rhat, r, True)
            if rho_new == 0:
                return x.cpu().numpy(), -10
            beta = (rho_new / rho) * (alpha / omega) if it > 1 else 0.0
            rho = rho_new
            if it == 1:
                p.copy_(r)
            else:
                v.axpby(-omega, vv, 1.0, p)            # p = p - omega v
                v.axpby(1.0, r, beta, p)               # p = r + beta p
            self._apply_M(p, phat)
            s.csr.matvec(phat, vv)
            alpha = rho / v.dot(rhat, vv, True)
            v.axpby(alpha, phat, 1.0, x)               # x += alpha phat
            v.axpby(-alpha, vv, 1.0, r)                # r = s
            res = v.norm(r) / bn
            if res <= self.tol:
                self._callback(res)
                return x.cpu().numpy(), 0
            self._apply_M(r, shat)
            t = s.csr.matvec(shat)
            tt = v.dot(t, t, True)
            omega = v.dot(t, r, True) / tt if tt != 0 else 0.0
            v.axpby(omega, shat, 1.0, x)
            v.axpby(-omega, t, 1.0, r)
            res = v.norm(r) / bn
            self._callback(res)
            if res <= self.tol:
                return x.cpu().numpy(), 0
            if omega == 0:
                return x.cpu().numpy(), -11
        return x.cpu().numpy(), maxit


class GMRESSolver(SystemSolverBase):
    """Restarted, right-preconditioned GMRES on the GPU."""
    restart = 20

    def _call_solver(self):
        from ..solvers import RefinedDirectSolver
        s = self._sys
        b = s.to_dev(self._b)

        class _P:
            def __init__(self, outer):
                self.outer = outer

            def solve(self, r, out=None):
                out = torch.empty_like(r) if out is None else out
                return self.outer._apply_M(r, out)
        rs = RefinedDirectSolver(s.csr, _P(self))
        rs._precond = lambda r, out: self._apply_M(r, out)
        x, info = rs.solve(b, tol=self.tol, maxit=max(1, (self.maxiter or 10 * s.n) // self.restart),
                           method="gmres", restart=self.restart)
        for h in info["history"][1:]:
            self._callback(h)
        return x.cpu().numpy(), 0 if info["converged"] else info["iterations"]


class UMFPACKSolver(SystemSolverBase):
    """Direct solve by the GPU multifrontal LU (the reference's UMFPACK route),
    refined in double precision when the factor is single precision."""

    def __init__(self, A, preconditioner_type=None):
        super().__init__(A, None)

    def _call_solver(self):
        from ..solvers import RefinedDirectSolver
        s = self._sys
        b = s.to_dev(self._b)
        rs = RefinedDirectSolver(s.csr, s.lu())
        x, info = rs.solve(b, tol=1e-14 if FACTOR_PRECISION == "fp64" else 1e-12, maxit=5,
                           method="ir")
        return x.cpu().numpy(), 0

    def plot_convergence(self, *a, **k):
        print("Direct solver has no convergence history")


class PyAMGSolver(SystemSolverBase):
    """The reference's optional algebraic-multigrid solver runs pyamg on the
    host.  This library solves on the GPU only, so it refuses instead of
    falling back to a CPU solve; use UMFPACKSolver (GPU LU) or the Krylov
    solvers."""

    def _call_solver(self):
        raise NotImplementedError(
            "PyAMGSolver is a CPU (pyamg) solver and this build has no CPU fallback; "
            "use UMFPACKSolver, BiCGStabSolver or GMRESSolver")


def calculate_residual(A, x, b):
    """||A x - b|| (sucemfem/Utilities/LinalgSolvers.py:297-305)."""
    return np.linalg.norm(A * x - b.reshape(x.shape))


def solve_sparse_system(A, b, preconditioner_type="ilu"):
    """BiCGStab with the given preconditioner (default: the GPU LU)."""
    solver = BiCGStabSolver(A, preconditioner_type)
    return solver.solve(b)
