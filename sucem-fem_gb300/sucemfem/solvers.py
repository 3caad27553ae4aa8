"""GPU solve path: device CSR, vector kernels, and the direct + refinement
driven solver.

Precision pattern: the matrix is factorised by the multifrontal LU in
single precision (complex64 / float32) and the solution is refined in
double precision against the FP64-assembled matrix (FGMRES or classical
iterative refinement, residual r = b - A x in complex128).  The plain FP64
path factorises in double precision.  Replaces the reference's driven
solves (sucemfem/Utilities/LinalgSolvers.py:239-322: BiCGStab + spilu,
GMRES, UMFPACK)."""
import ctypes
import time

import numpy as np
import torch

from . import _device, _native
from ._native import c_vp, call, ptr

_native.declare("sucem_spmv_csr", ctypes.c_int,
                [ctypes.c_int64, ctypes.c_int64, c_vp, c_vp, ctypes.c_int, c_vp, c_vp, c_vp, c_vp])
_native.declare("sucem_vec_axpby", ctypes.c_int,
                [ctypes.c_int64, ctypes.c_int, ctypes.c_double, ctypes.c_double, c_vp,
                 ctypes.c_double, ctypes.c_double, c_vp, c_vp])
_native.declare("sucem_vec_dot_work_bytes", ctypes.c_int64, [])
_native.declare("sucem_vec_dot", ctypes.c_int,
                [ctypes.c_int64, ctypes.c_int, c_vp, c_vp, ctypes.c_int, c_vp, c_vp, c_vp])
_native.declare("sucem_vec_convert", ctypes.c_int,
                [ctypes.c_int64, ctypes.c_int, c_vp, ctypes.c_int, c_vp, c_vp])
_native.declare("sucem_vec_gs_work_bytes", ctypes.c_int64, [ctypes.c_int])
_native.declare("sucem_vec_gs", ctypes.c_int,
                [ctypes.c_int64, ctypes.c_int, c_vp, ctypes.c_int64, ctypes.c_int, c_vp, c_vp, c_vp,
                 c_vp])

DT = {torch.float32: _native.F32, torch.float64: _native.F64,
      torch.complex64: _native.C64, torch.complex128: _native.C128}


class Vec:
    """Vector kernels of libsucem_gb300 on device tensors."""

    def __init__(self):
        nbytes = _native.lib().sucem_vec_dot_work_bytes()
        self.work = torch.empty(int(nbytes) // 8, dtype=torch.float64, device=_device.device())
        self.out = torch.empty(2, dtype=torch.float64, device=_device.device())

    def axpby(self, a, x, b, y):
        a, b = complex(a), complex(b)
        call("sucem_vec_axpby", y.numel(), DT[y.dtype], a.real, a.imag, ptr(x), b.real, b.imag,
             ptr(y), _device.stream_ptr())
        return y

    def dot(self, x, y, conj=True):
        call("sucem_vec_dot", x.numel(), DT[x.dtype], ptr(x), ptr(y), int(conj), ptr(self.work),
             ptr(self.out), _device.stream_ptr())
        o = self.out.cpu().numpy()
        return complex(o[0], o[1]) if x.is_complex() else float(o[0])

    def gs(self, V, k, w):
        """Orthogonalise w (in place) against rows 0..k-1 of the 2-D device
        tensor V by block Gram-Schmidt on the device (two classical passes);
        returns (coefficients as a numpy array of k values, norm of w)."""
        if getattr(self, "_gs_k", -1) < k:
            nb = int(_native.lib().sucem_vec_gs_work_bytes(k))
            self._gs_work = torch.empty((nb + 7) // 8, dtype=torch.float64, device=w.device)
            self._gs_h = torch.empty(2 * (k + 1), dtype=torch.float64, device=w.device)
            self._gs_k = k
        call("sucem_vec_gs", w.numel(), DT[w.dtype], ptr(V), V.stride(0), k, ptr(w),
             ptr(self._gs_work), ptr(self._gs_h), _device.stream_ptr())
        hv = self._gs_h[:2 * (k + 1)].cpu().numpy()
        c = hv[0:2 * k:2] + 1j * hv[1:2 * k:2] if w.is_complex() else hv[0:2 * k:2].copy()
        return c, float(np.sqrt(max(hv[2 * k], 0.0)))

    def norm(self, x):
        return float(np.sqrt(abs(self.dot(x, x, True).real if x.is_complex() else self.dot(x, x))))

    def convert(self, src, dst):
        rs = 4 if src.dtype in (torch.float32, torch.complex64) else 8
        rd = 4 if dst.dtype in (torch.float32, torch.complex64) else 8
        count = src.numel() * (2 if src.is_complex() else 1)
        call("sucem_vec_convert", count, rd, ptr(dst), rs, ptr(src), _device.stream_ptr())
        return dst


class DeviceCSR:
    """CSR matrix on the device (int32 indices)."""

    def __init__(self, indptr, indices, values, n=None):
        dev = _device.device()
        self.indptr = indptr if torch.is_tensor(indptr) else torch.as_tensor(
            np.asarray(indptr, dtype=np.int32), device=dev)
        self.indices = indices if torch.is_tensor(indices) else torch.as_tensor(
            np.asarray(indices, dtype=np.int32), device=dev)
        self.values = values
        self.n = int(n if n is not None else self.indptr.numel() - 1)
        self.nnz = int(self.indices.numel())

    @classmethod
    def from_scipy(cls, A, dtype=torch.complex128):
        A = A.tocsr()
        A.sort_indices()
        vals = torch.as_tensor(np.asarray(A.data), device=_device.device()).to(dtype)
        return cls(A.indptr, A.indices, vals, A.shape[0])

    def matvec(self, x, y=None, values=None):
        v = self.values if values is None else values
        if y is None:
            y = torch.empty(self.n, dtype=v.dtype, device=v.device)
        call("sucem_spmv_csr", self.n, self.nnz, ptr(self.indptr), ptr(self.indices), DT[v.dtype],
             ptr(v), ptr(x), ptr(y), _device.stream_ptr())
        return y


class RefinedDirectSolver:
    """x = A^-1 b by a (single or double precision) multifrontal LU and
    double-precision refinement against ``A64``.

    A64: DeviceCSR with complex128/float64 values (the accuracy reference).
    lu: SparseLU on the same pattern, factorised by ``factor(values32)``."""

    def __init__(self, A64, lu):
        self.A = A64
        self.lu = lu
        self.vec = Vec()
        self.history = []

    def factor(self, values, dtype):
        self.lu.factor(values, dtype)
        return self

    def _precond(self, r, out):
        return self.lu.solve(r, out)

    def solve(self, b, tol=1e-10, maxit=50, method="gmres", restart=30):
        """b: device tensor (A's dtype).  Returns (x, info)."""
        if method == "ir":
            return self._solve_ir(b, tol, maxit)
        return self._solve_fgmres(b, tol, maxit, restart)

    def _solve_ir(self, b, tol, maxit):
        v = self.vec
        bn = v.norm(b)
        x = torch.zeros_like(b)
        r = b.clone()
        d = torch.empty_like(b)
        hist = []
        for it in range(maxit + 1):
            rn = v.norm(r) / (bn if bn > 0 else 1.0)
            hist.append(rn)
            if rn <= tol or it == maxit:
                break
            self._precond(r, d)
            v.axpby(1.0, d, 1.0, x)
            self.A.matvec(x, r)
            v.axpby(1.0, b, -1.0, r)           # r = b - A x
        self.history = hist
        return x, dict(iterations=len(hist) - 1, residual=hist[-1], converged=hist[-1] <= tol,
                       history=hist)

    def _solve_fgmres(self, b, tol, maxit, m):
        """Right-preconditioned flexible GMRES in double precision."""
        v = self.vec
        bn = v.norm(b)
        if bn == 0:
            return torch.zeros_like(b), dict(iterations=0, residual=0.0, converged=True, history=[0.0])
        x = torch.zeros_like(b)
        r = b.clone()
        hist = [1.0]
        total = 0
        cplx = b.is_complex()
        for outer in range(maxit):
            beta = v.norm(r)
            if beta / bn <= tol:
                break
            # the Krylov basis as the rows of one device matrix, so that a
            # whole Arnoldi step's orthogonalisation is one device call
            # (classical Gram-Schmidt with one reorthogonalisation) and one
            # copy of its coefficients to the host
            Vb = torch.empty((m + 1, b.numel()), dtype=b.dtype, device=b.device)
            v.axpby(1.0 / beta, r, 0.0, Vb[0])
            Z = []
            H = np.zeros((m + 1, m), dtype=np.complex128)
            g = np.zeros(m + 1, dtype=np.complex128)
            g[0] = beta
            cs = np.zeros(m, dtype=np.complex128)
            sn = np.zeros(m, dtype=np.complex128)
            k_used = 0
            for j in range(m):
                z = torch.empty_like(b)
                self._precond(Vb[j], z)
                Z.append(z)
                w = Vb[j + 1]
                self.A.matvec(z, w)
                hcol, hn = v.gs(Vb, j + 1, w)
                H[:j + 1, j] = hcol
                H[j + 1, j] = hn
                # Givens rotations G = [[conj(c), conj(s)], [-s, c]] with
                # c = a/|(a,b)|, s = b/|(a,b)| map (a, b) to (|(a,b)|, 0)
                for i in range(j):
                    t = np.conj(cs[i]) * H[i, j] + np.conj(sn[i]) * H[i + 1, j]
                    H[i + 1, j] = -sn[i] * H[i, j] + cs[i] * H[i + 1, j]
                    H[i, j] = t
                den = np.sqrt(abs(H[j, j]) ** 2 + abs(H[j + 1, j]) ** 2)
                cs[j] = H[j, j] / den if den else 1.0
                sn[j] = H[j + 1, j] / den if den else 0.0
                H[j, j] = den
                H[j + 1, j] = 0
                g[j + 1] = -sn[j] * g[j]
                g[j] = np.conj(cs[j]) * g[j]
                k_used = j + 1
                total += 1
                est = abs(g[j + 1]) / bn
                hist.append(est)
                if est <= tol or hn == 0:
                    break
                v.axpby(0.0, None, 1.0 / hn, w)  # w /= hn in place
            y = np.linalg.solve(np.triu(H[:k_used, :k_used]), g[:k_used])
            for i in range(k_used):
                yi = complex(y[i]) if cplx else float(np.real(y[i]))
                v.axpby(yi, Z[i], 1.0, x)
            self.A.matvec(x, r)
            v.axpby(1.0, b, -1.0, r)
            true_res = v.norm(r) / bn
            hist[-1] = true_res
            if true_res <= tol:
                break
        res = v.norm(r) / bn
        self.history = hist
        return x, dict(iterations=total, residual=res, converged=res <= tol, history=hist)


def lu_for_space(V, leaf_size=128):
    """SparseLU of a FunctionSpace's full pattern with the element ordering."""
    from .lu import SparseLU
    cx = V.mesh().coordinates()[V.cells].mean(1)
    return SparseLU(V.indptr, V.indices, leaf_size=leaf_size, cells=(V.cell_dofs, cx))


class DrivenSolver:
    """Assemble and solve (S - k0^2 T + j k0 B) x = b on the GPU.

    precision 'fp32-ir': complex64 LU of the FP64-assembled matrix rounded
    to single precision, the FP64 matrix for the FGMRES refinement (the
    refinement needs the FP64 matrix anyway, and its rounding is the most
    accurate single-precision input: on the 20^3 order-2 box it takes 5
    refinement iterations where the single-precision assembly's matrix,
    2e-7 of its row scale off, takes 6); 'fp32-asm': the LU input from the
    single-precision assembly instead; 'fp64': everything in double."""

    def __init__(self, V, eps_r=None, mu_r_inv=None, lu=None):
        self.V = V
        self.h = V.upload()
        dev = _device.device()
        self.eps = None if eps_r is None else np.asarray(eps_r, dtype=np.float64)
        self.mu_inv = None if mu_r_inv is None else np.asarray(mu_r_inv, dtype=np.float64)
        self.lu = lu if lu is not None else lu_for_space(V)
        self.indptr = torch.as_tensor(V.indptr.astype(np.int32), device=dev)
        self.indices = torch.as_tensor(V.indices, device=dev)
        self._coef = {}
        self.A64 = None
        self.A32 = None

    def _coefs(self, rb):
        if rb not in self._coef:
            dt = _device.REAL[rb]
            e = None if self.eps is None else _device.to_dev(self.eps, dt)
            m = None if self.mu_inv is None else _device.to_dev(self.mu_inv, dt)
            self._coef[rb] = (e, m)
        return self._coef[rb]

    def assemble(self, k0, real_bytes):
        e, m = self._coefs(real_bytes)
        A = torch.empty(self.V.nnz, dtype=_device.COMPLEX[real_bytes], device=_device.device())
        call("sucem_assemble_helmholtz", self.h, real_bytes, ptr(e), ptr(m), float(k0), ptr(A),
             _device.stream_ptr())
        return A

    def solve(self, k0, b, precision="fp32-ir", tol=1e-10, method="gmres", maxit=30):
        """b: numpy or device complex128 RHS.  Returns (x device c128, info)."""
        t0 = time.perf_counter()
        if not torch.is_tensor(b):
            b = _device.to_dev(np.asarray(b, dtype=np.complex128))
        self.A64 = self.assemble(k0, 8)
        A = DeviceCSR(self.indptr, self.indices, self.A64, self.V.n)
        rs = RefinedDirectSolver(A, self.lu)
        if precision == "fp64":
            rs.factor(self.A64, "c128")
        else:
            if precision == "fp32-asm":
                self.A32 = self.assemble(k0, 4)
            else:
                self.A32 = rs.vec.convert(self.A64, torch.empty(self.V.nnz, dtype=torch.complex64,
                                                                 device=self.A64.device))
            rs.factor(self.A32, "c64")
        x, info = rs.solve(b, tol=tol, method=method, maxit=maxit)
        info["perturbed_pivots"] = self.lu.perturbed()
        info["seconds"] = time.perf_counter() - t0
        info["precision"] = precision
        return x, info
