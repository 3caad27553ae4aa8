"""GPU multifrontal sparse LU (libsucem_gb300 sucem_lu_*).

The direct-solver replacement for dolfin.LUSolver / UMFPACK / spilu used by
the reference (sucemfem/ProblemConfigurations/EMVectorWaveEigenproblem.py:
76-85, sucemfem/Utilities/LinalgSolvers.py:118-121,262-277)."""
import ctypes

import numpy as np

from . import _device, _native
from ._native import c_vp, call, ptr

_native.declare("sucem_lu_analyse", ctypes.c_int,
                [ctypes.c_int64, c_vp, c_vp, c_vp, ctypes.c_int, ctypes.POINTER(c_vp)])
_native.declare("sucem_lu_destroy", None, [c_vp])
_native.declare("sucem_lu_info", ctypes.c_int, [c_vp, c_vp])
_native.declare("sucem_lu_copy_perm", ctypes.c_int, [c_vp, c_vp])
_native.declare("sucem_lu_fronts", ctypes.c_int, [c_vp, c_vp])
_native.declare("sucem_selftest_bounded_wait", ctypes.c_int,
                [ctypes.c_int, ctypes.POINTER(ctypes.c_int)])
_native.declare("sucem_lu_factor", ctypes.c_int, [c_vp, ctypes.c_int, c_vp, ctypes.c_double, c_vp])
_native.declare("sucem_lu_solve", ctypes.c_int, [c_vp, ctypes.c_int, c_vp, c_vp, c_vp])
_native.declare("sucem_lu_perturbed", ctypes.c_int, [c_vp])
_native.declare("sucem_lu_kernel_stats", ctypes.c_int, [c_vp, c_vp])
_native.declare("sucem_lu_status", ctypes.c_int, [c_vp])
_native.declare("sucem_lu_inject_timeout", ctypes.c_int, [c_vp])
_native.declare("sucem_lu_configure", ctypes.c_int, [c_vp, ctypes.c_int, ctypes.c_int])

DTYPES = {"f32": _native.F32, "f64": _native.F64, "c64": _native.C64, "c128": _native.C128}


_native.declare("sucem_lu_analyse_cells", ctypes.c_int,
                [ctypes.c_int64, c_vp, c_vp, ctypes.c_int64, ctypes.c_int, c_vp, c_vp, ctypes.c_int,
                 ctypes.POINTER(c_vp)])


class SparseLU:
    """Symbolic analysis on construction (host); factor/solve on the GPU.

    With ``cells=(cell_dofs, cell_xyz)`` the element-based nested dissection
    is used (interface separators); otherwise DOF coordinates ``xyz``."""

    def __init__(self, indptr, indices, xyz=None, leaf_size=96, cells=None):
        self.n = len(indptr) - 1
        ip = np.ascontiguousarray(indptr, dtype=np.int32)
        ix = np.ascontiguousarray(indices, dtype=np.int32)
        h = c_vp()
        if cells is not None:
            cd = np.ascontiguousarray(cells[0], dtype=np.int32)
            cx = np.ascontiguousarray(cells[1], dtype=np.float64).reshape(len(cd), 3)
            call("sucem_lu_analyse_cells", self.n, ptr(ip), ptr(ix), len(cd), cd.shape[1], ptr(cd),
                 ptr(cx), int(leaf_size), ctypes.byref(h))
        else:
            if xyz is not None:
                xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(self.n, 3)
            call("sucem_lu_analyse", self.n, ptr(ip), ptr(ix), ptr(xyz), int(leaf_size),
                 ctypes.byref(h))
        self._h = h
        info = np.zeros(7)
        call("sucem_lu_info", self._h, ptr(info))
        self.info = dict(n=int(info[0]), nnz=int(info[1]), nodes=int(info[2]), levels=int(info[3]),
                         arena=int(info[4]), flops=float(info[5]), max_front=int(info[6]))
        self.dtype = None
        self.params = (0, 0)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _native._lib is not None:
            _native._lib.sucem_lu_destroy(h)
            self._h = None

    def fronts(self):
        """Assembly tree as an int64 array of (level, pivots k, front size f)
        rows, one per tree node."""
        out = np.empty((self.info["nodes"], 3), dtype=np.int64)
        call("sucem_lu_fronts", self._h, ptr(out))
        return out

    def perm(self):
        p = np.empty(self.n, dtype=np.int64)
        call("sucem_lu_copy_perm", self._h, ptr(p))
        return p

    def factor(self, values, dtype, pivot_tol=None, stream=None):
        """values: device tensor of nnz entries in CSR order."""
        code = DTYPES[dtype]
        if pivot_tol is None:
            pivot_tol = 1e-7 if dtype in ("f32", "c64") else 1e-14
        call("sucem_lu_factor", self._h, code, ptr(values), float(pivot_tol),
             stream if stream is not None else _device.stream_ptr())
        self.dtype = dtype
        return self

    def configure(self, superpanel=0, panel_min_k=0):
        """Plan parameters of the single-precision factorisation (0 =
        default): super-panel width (multiple of 64) and the pivot-block
        threshold of the tensor-core panel updates.  Takes effect at the
        next factor()."""
        call("sucem_lu_configure", self._h, int(superpanel), int(panel_min_k))
        self.params = (int(superpanel), int(panel_min_k))
        return self

    @staticmethod
    def selftest_bounded_wait(polls=2000):
        """True when a device wait that nothing completes gives up after
        ``polls`` polls and its kernel returns (the failure detection of the
        tensor-core update)."""
        out = ctypes.c_int(-1)
        call("sucem_selftest_bounded_wait", int(polls), ctypes.byref(out))
        return out.value == 1

    def check(self):
        """Wait for the last factorisation and raise RuntimeError when it
        cannot be used (a bounded wait of its tensor-core update gave up)."""
        call("sucem_lu_status", self._h)
        return self

    def _inject_timeout(self):
        """Test hook: mark the last factorisation as if its tensor-core
        update had given up waiting (host write of the device flag)."""
        call("sucem_lu_inject_timeout", self._h)

    def perturbed(self):
        """Number of replaced (perturbed) pivots of the last factorisation."""
        v = _native.lib().sucem_lu_perturbed(self._h)
        if v < 0:
            raise RuntimeError("LU factorisation: a tensor-core update gave up waiting "
                               "(bounded wait expired); the factor is invalid")
        return v

    def kernel_stats(self):
        """Tensor-core Schur updates of the last complex64 factorisation:
        launches, summed device time (ms, CUDA events on the factor's stream)
        and algorithmic flops."""
        out = np.zeros(3, dtype=np.float64)
        call("sucem_lu_kernel_stats", self._h, ptr(out))
        return {"launches": int(out[0]), "ms": float(out[1]), "flops": float(out[2])}

    def solve(self, b, x=None, stream=None):
        """b: device tensor (factor dtype, or complex128/float64 for a
        single-precision factor).  Returns x (same dtype as b)."""
        import torch
        io = {torch.float32: _native.F32, torch.float64: _native.F64,
              torch.complex64: _native.C64, torch.complex128: _native.C128}[b.dtype]
        if x is None:
            x = torch.empty_like(b)
        call("sucem_lu_solve", self._h, io, ptr(b), ptr(x),
             stream if stream is not None else _device.stream_ptr())
        return x
