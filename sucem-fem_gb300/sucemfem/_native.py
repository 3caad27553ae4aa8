"""ctypes binding of libsucem_gb300.so (declarations: include/sucem_gb300.h).

The library is built in-tree (sucem-fem_gb300/build_native.py).  There is
no fallback: if the library cannot be loaded every GPU entry point raises.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_HERE, "libsucem_gb300.so")

SUCEM_OK = 0
ERR_ARG, ERR_MEMORY, ERR_CUDA, ERR_STATE, ERR_NOCONV, ERR_BREAKDOWN = -1, -2, -3, -4, -5, -6

COPY = dict(indptr=0, indices=1, cell_dofs=2, boundary_dofs=3, edges=4, faces=5, cells=6, ext_mask=7,
            cell_edges=8, cell_faces=9, dof_xyz=10, boundary_dual=11, task_ent=12, task_meta=13,
            step_words=14, entry_ptr=15, entry_src=16, entry_perm=17)
DEV = dict(indptr=0, indices=1, cell_dofs=2, boundary_dofs=3)

_lib = None

c_i64p = ctypes.POINTER(ctypes.c_int64)
c_vp = ctypes.c_void_p


class SolverError(RuntimeError):
    """Raised for non-convergence or breakdown reported by the library."""

    def __init__(self, msg, code):
        super().__init__(msg)
        self.code = code


# (name, restype, argtypes); every int-returning function is checked
_SIGS = [
    ("sucem_version", ctypes.c_int, []),
    ("sucem_last_error", ctypes.c_char_p, []),
    ("sucem_launch_count", ctypes.c_longlong, []),
    ("sucem_space_create", ctypes.c_int,
     [c_vp, ctypes.c_int64, c_vp, ctypes.c_int64, ctypes.c_int, ctypes.POINTER(c_vp)]),
    ("sucem_space_destroy", None, [c_vp]),
    ("sucem_space_sizes", ctypes.c_int, [c_vp, c_i64p]),
    ("sucem_space_copy", ctypes.c_int, [c_vp, ctypes.c_int, c_vp]),
    ("sucem_space_schedule_sizes", ctypes.c_int, [c_vp, c_i64p]),
    ("sucem_space_upload", ctypes.c_int, [c_vp, ctypes.c_int]),
    ("sucem_space_device_ptr", ctypes.c_int, [c_vp, ctypes.c_int, ctypes.POINTER(c_vp)]),
    ("sucem_assemble", ctypes.c_int,
     [c_vp, ctypes.c_int, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
    ("sucem_assemble_helmholtz", ctypes.c_int,
     [c_vp, ctypes.c_int, c_vp, c_vp, ctypes.c_double, c_vp, c_vp]),
    ("sucem_assemble_host", ctypes.c_int, [c_vp, ctypes.c_int, c_vp, c_vp, c_vp, c_vp, c_vp]),
    ("sucem_apply_essential", ctypes.c_int, [c_vp, ctypes.c_int, c_vp, c_vp, ctypes.c_int64, c_vp]),
    ("sucem_spmv", ctypes.c_int, [c_vp, ctypes.c_int, c_vp, c_vp, c_vp, c_vp]),
    ("sucem_combine", ctypes.c_int,
     [ctypes.c_int64, ctypes.c_int, ctypes.c_double, c_vp, ctypes.c_double, c_vp,
      ctypes.c_double, c_vp, c_vp, ctypes.c_int, c_vp]),
    ("sucem_compact_count", ctypes.c_int, [c_vp, ctypes.c_int, c_vp, c_vp, c_vp, c_vp]),
    ("sucem_compact_fill", ctypes.c_int, [c_vp, ctypes.c_int, c_vp, c_vp, c_vp, c_vp, c_vp]),
    ("sucem_point_sources", ctypes.c_int, [c_vp, c_vp, c_vp, ctypes.c_int, c_vp, c_vp, c_vp]),
    ("sucem_compact_count_noalloc", ctypes.c_int, [c_vp, ctypes.c_int, c_vp, c_vp, c_vp]),
]

F32, F64, C64, C128 = 0, 1, 2, 3

OPTIONAL_SIGS = []   # filled by modules that declare further entry points


def exported_symbols():
    """Names the header declares (used by the CPU export test)."""
    return [s[0] for s in _SIGS] + [s[0] for s in OPTIONAL_SIGS]


def declare(name, restype, argtypes):
    OPTIONAL_SIGS.append((name, restype, argtypes))
    if _lib is not None:
        f = getattr(_lib, name)
        f.restype, f.argtypes = restype, argtypes


def lib():
    """Load the native library (raises if it is missing or stale)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                "libsucem_gb300.so not built; run __graft_entry__.build() "
                "(or python sucem-fem_gb300/build_native.py)")
        l = ctypes.CDLL(LIB_PATH)
        for name, res, args in _SIGS + OPTIONAL_SIGS:
            f = getattr(l, name)
            f.restype, f.argtypes = res, args
        _lib = l
    return _lib


def check(rc, what=""):
    if rc == SUCEM_OK:
        return
    msg = lib().sucem_last_error().decode(errors="replace")
    text = "%s: %s" % (what, msg) if what else msg
    if rc == ERR_ARG:
        raise ValueError(text)
    if rc == ERR_MEMORY:
        raise MemoryError(text)
    if rc in (ERR_NOCONV, ERR_BREAKDOWN):
        raise SolverError(text, rc)
    raise RuntimeError(text)


def call(name, *args):
    rc = getattr(lib(), name)(*args)
    check(rc, name)
    return rc


def ptr(a):
    """Address of a numpy array or torch tensor (None -> NULL)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return c_vp(a.data_ptr())
    return c_vp(a.ctypes.data)
