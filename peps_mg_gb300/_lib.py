"""ctypes binding of libpeps_mg.so (the C-ABI declared in include/peps_mg.h).

The library is built in-tree by peps_mg_gb300/build.py.  There is no fallback: if the
shared library is missing or cannot be loaded, importing the solver raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libpeps_mg.so")

PMG_OK, PMG_EINVAL, PMG_ENOMEM, PMG_EDIVERGED, PMG_ETIMEOUT, PMG_ECUDA = range(6)
PMG_CGS, PMG_CGA, PMG_CGPSA = 0, 1, 2
PMG_COARSE_RBGS, PMG_COARSE_CG = 0, 1
PMG_FP64, PMG_MIXED, PMG_FP64_FAST = 0, 1, 2

c_int, c_double, c_float, c_void_p = ctypes.c_int, ctypes.c_double, ctypes.c_float, ctypes.c_void_p


class PmgConfig(ctypes.Structure):
    _fields_ = [("nx", c_int), ("ny", c_int), ("nz", c_int),
                ("dxm", c_void_p), ("dxg", c_void_p), ("xg", c_void_p),
                ("dym", c_void_p), ("dyg", c_void_p), ("yg", c_void_p),
                ("dzm", c_void_p), ("dzg", c_void_p), ("zg", c_void_p),
                ("number_of_levels", c_int), ("number_of_vcycles", c_int),
                ("aggregation_method", c_int), ("cga_level", c_int), ("cgpsa_level", c_int * 3),
                ("coarse_solver", c_int), ("precision", c_int), ("mixed_inner_cycles", c_int)]


class PmgReport(ctypes.Structure):
    _fields_ = [("cycles", c_int), ("converged", c_int), ("res0", c_double), ("final_ratio", c_double),
                ("history", ctypes.POINTER(c_double)), ("coarse_iterations", ctypes.POINTER(c_int)),
                ("elapsed_ms", c_float), ("inner_cycles", c_int)]


# symbol -> argtypes (restype int unless noted)
_SIGS = {
    "pmg_create": [ctypes.POINTER(c_void_p), ctypes.POINTER(PmgConfig), c_void_p],
    "pmg_solve_vcycle": [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_double, c_double,
                         ctypes.POINTER(PmgReport)],
    "pmg_destroy": [c_void_p],
    "pmg_level_sizes": [c_int, c_int, c_int, c_int, c_int, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int)],
    "pmg_level_dims": [c_void_p, c_int, ctypes.POINTER(c_int)],
    "pmg_level_mesh": [c_void_p, c_int, c_int, c_void_p, c_void_p, c_void_p],
    "pmg_coarsest_levels": [c_void_p, ctypes.POINTER(c_int)],
    "pmg_mv_mul": [c_void_p, c_int, c_void_p, c_void_p],
    "pmg_vv_dot": [c_void_p, c_int, c_void_p, c_void_p, ctypes.POINTER(c_double)],
    "pmg_residual": [c_void_p, c_int, c_void_p, c_void_p, c_void_p],
    "pmg_rbgs_iterator": [c_void_p, c_int, c_void_p, c_void_p, c_int, c_double],
    "pmg_rbgs_solver": [c_void_p, c_int, c_void_p, c_void_p, c_int, c_double, c_double,
                        ctypes.POINTER(c_int), ctypes.POINTER(c_double)],
    "pmg_cg_iterator": [c_void_p, c_int, c_void_p, c_void_p, c_int],
    "pmg_cg_solver": [c_void_p, c_int, c_void_p, c_void_p, c_int, c_double, ctypes.POINTER(c_int),
                      ctypes.POINTER(c_double)],
    "pmg_restriction": [c_void_p, c_int, c_void_p, c_void_p],
    "pmg_prolongation": [c_void_p, c_int, c_void_p, c_void_p],
    "pmg_prolong_add": [c_void_p, c_int, c_void_p, c_void_p],
    "pmg_adjoint": [c_void_p, c_void_p, c_void_p, ctypes.POINTER(c_double), c_int, c_double, c_double,
                    ctypes.POINTER(PmgReport)],
    "pmg_batch_create": [ctypes.POINTER(c_void_p), c_int, ctypes.POINTER(c_int), c_void_p, c_int, c_void_p],
    "pmg_batch_layout": [c_void_p, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(c_int)],
    "pmg_batch_solve": [c_void_p, c_void_p, c_void_p, c_int, c_double, c_double, c_int, ctypes.POINTER(c_int),
                        ctypes.POINTER(c_double), ctypes.POINTER(c_float)],
    "pmg_batch_destroy": [c_void_p],
    "pmg_dd_create": [ctypes.POINTER(c_void_p), ctypes.POINTER(PmgConfig), ctypes.POINTER(c_int), c_void_p],
    "pmg_dd_solve": [c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_double, c_double, ctypes.POINTER(PmgReport)],
    "pmg_dd_destroy": [c_void_p],
    "pmg_dd_partition": [ctypes.POINTER(PmgConfig), ctypes.POINTER(c_int), ctypes.POINTER(c_int), c_int,
                         ctypes.POINTER(c_int), ctypes.POINTER(c_void_p), ctypes.POINTER(c_int)],
    "pmg_vv_dot_static": [c_void_p, c_void_p, c_int, c_int, c_int, c_void_p, ctypes.POINTER(c_double)],
    "pmg_profile": [c_void_p, c_int],
    "pmg_profile_read": [c_void_p, c_int, ctypes.POINTER(c_double), ctypes.POINTER(ctypes.c_longlong),
                         ctypes.POINTER(c_double)],
    "pmg_launch_count": [ctypes.POINTER(ctypes.c_longlong)],
    "pmg_selftest_convert": [c_void_p, c_void_p, c_void_p, c_void_p, c_int],
    "pmg_selftest_smooth32": [c_void_p, c_int, c_int, c_int, c_int, c_int, c_double, c_void_p, c_void_p,
                              c_void_p],
    "pmg_selftest_wait_timeout": [c_void_p, c_int],
    "pmg_set_abort": [c_void_p, c_int],
    "pmg_inject_alloc_failure": [ctypes.c_longlong],
    "pmg_sync": [c_void_p],
    "pmg_last_error": [],
    "pmg_status_string": [c_int],
}

EXPORTED = tuple(_SIGS)

_lib = None


class PmgError(RuntimeError):
    """Raised where the reference would print an error and stop."""

    def __init__(self, status, where, detail=""):
        self.status = status
        super().__init__("%s failed: %s%s" % (where, STATUS_NAMES.get(status, str(status)),
                                               (" (%s)" % detail) if detail else ""))


STATUS_NAMES = {PMG_OK: "ok", PMG_EINVAL: "invalid argument", PMG_ENOMEM: "out of memory",
                PMG_EDIVERGED: "diverged", PMG_ETIMEOUT: "timeout", PMG_ECUDA: "cuda error"}


def load(path=LIB_PATH):
    """Load the shared library (once).  Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libpeps_mg.so not found at %s: build it with "
                           "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)" % path)
    lib = ctypes.CDLL(path)
    for name, argtypes in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = argtypes
        fn.restype = ctypes.c_char_p if name in ("pmg_last_error", "pmg_status_string") else c_int
    _lib = lib
    return lib


def check(rc, where):
    if rc != PMG_OK:
        detail = load().pmg_last_error()
        raise PmgError(rc, where, detail.decode() if detail else "")
    return rc
