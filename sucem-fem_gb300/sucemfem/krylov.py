"""Device-resident preconditioned BiCGStab (libsucem_gb300 sucem_bicgstab).

Every scalar of the iteration stays in device memory and the dot products
are reduced on the device; without an LU preconditioner a batch of
iterations is one CUDA graph replay, after which the host reads a single
status word.  Replaces the reference's BiCGStabSolver
(sucemfem/Utilities/LinalgSolvers.py:239-248) behind the drop-in solver
classes, and serves as a single-precision inner solver."""
import ctypes

import numpy as np
import torch

from . import _device, _native
from ._native import c_vp, call, ptr

_native.declare("sucem_bicgstab_work_bytes", ctypes.c_int64, [ctypes.c_int64, ctypes.c_int])
_native.declare("sucem_bicgstab", ctypes.c_int,
                [ctypes.c_int64, c_vp, c_vp, ctypes.c_int, c_vp, c_vp, c_vp, ctypes.c_int, c_vp,
                 ctypes.c_double, ctypes.c_int, ctypes.c_int, c_vp, ctypes.c_int64, c_vp, c_vp])

STATUS = {1: "converged", 2: "iteration limit", -1: "breakdown (rho = 0)",
          -2: "breakdown (omega = 0)"}


def bicgstab(csr, b, x0=None, precond=None, tol=1e-8, maxit=None, batch=32):
    """Solve csr x = b.  csr: DeviceCSR with complex64 or complex128 values;
    b: device vector of the same dtype.  precond: None, 'diagonal', or a
    factorised SparseLU of the same matrix.  Stops at ||b - A x|| <= tol
    ||b|| (recurrence residual) or after maxit iterations.  Returns (x,
    info) with info = iterations, residual, status, converged, host_syncs."""
    from .lu import SparseLU
    dt = csr.values.dtype
    if dt not in (torch.complex64, torch.complex128) or b.dtype != dt:
        raise ValueError("bicgstab: complex64 or complex128 matrix and right-hand side of one dtype")
    code = _native.C64 if dt == torch.complex64 else _native.C128
    x = torch.zeros_like(b) if x0 is None else x0.clone()
    nbytes = int(_native.lib().sucem_bicgstab_work_bytes(csr.n, code))
    work = torch.empty(nbytes, dtype=torch.uint8, device=b.device)
    if precond is None:
        pc, luh = 0, None
    elif isinstance(precond, str) and precond.lower() == "diagonal":
        pc, luh = 1, None
    elif isinstance(precond, SparseLU):
        pc, luh = 2, precond._h
    else:
        raise ValueError("precond: None, 'diagonal' or a SparseLU")
    info = np.zeros(4, dtype=np.float64)
    call("sucem_bicgstab", csr.n, ptr(csr.indptr), ptr(csr.indices), code, ptr(csr.values),
         ptr(b), ptr(x), pc, luh, float(tol), int(maxit if maxit is not None else 10 * csr.n),
         int(batch), ptr(work), nbytes, ptr(info), _device.stream_ptr())
    st = int(info[2])
    return x, dict(iterations=int(info[0]), residual=float(info[1]), status=st,
                   status_text=STATUS.get(st, "?"), converged=st == 1, host_syncs=int(info[3]))
