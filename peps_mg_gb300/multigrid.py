"""Python host mirror of the reference's `multigrid` module over the C-ABI.

    mg = Multigrid(mesh, number_of_levels, number_of_vcycles, aggregation_method,
                   cga_level, cgpsa_level)                    # multigrid_create
    report = mg.solve_vcycle(sol, rsd, rhs, maxiteration, tolerance, omega_sor)
    mg.destroy()                                             # multigrid_destroy

`mesh` is the caller's subdomain mesh: three (dm, dg, xg) triples (see geometry.py).
Grid arrays are (nx+2)(ny+2)(nz+2) float64 values in Fortran order: either CUDA
tensors (torch, any shape with that element count, contiguous) or host numpy arrays
(solve_vcycle only; they are staged through the device).  Errors raise PmgError where
the reference prints and stops.

The lower-level methods mirror rbgs_poisson_matrix, cg_poisson_matrix,
poisson_matrix_operator and the restriction / prolongation / residual routines of
multigrid.f90 on one level of the hierarchy (level 0 = the caller's grid).
"""
import ctypes
from dataclasses import dataclass, field as dfield

import numpy as np

from . import _lib
from ._lib import PmgConfig, PmgReport, check

_METHODS = {"cgs": 0, "cga": 1, "cgpsa": 2}
_COARSE = {"rbgs": 0, "cg": 1}
_PREC = {"fp64": 0, "mixed": 1, "fp64_fast": 2}


def _code(table, v):
    """Name -> C-ABI code; integers pass through (the library validates them)."""
    if isinstance(v, str):
        if v.lower() not in table:
            raise ValueError("unknown option %r (expected one of %s)" % (v, sorted(table)))
        return table[v.lower()]
    return int(v)


@dataclass
class SolveReport:
    cycles: int
    converged: bool
    res0: float
    final_ratio: float
    history: np.ndarray = dfield(repr=False)      # (cycles, 3): sqrt(rsd), sqrt(res0), ratio
    coarse_iterations: np.ndarray = dfield(repr=False)
    elapsed_ms: float = 0.0
    inner_cycles: int = 0

    def log_lines(self):
        """The reference's per-cycle log lines (src/multigrid.f90:1972)."""
        return ["[MG] cycle = %4d, Error:%15.7E %15.7E %15.7E" % (c + 1, h[0], h[1], h[2])
                for c, h in enumerate(self.history)]


def _ptr(a):
    """Data pointer and element count of a torch tensor or numpy array."""
    if isinstance(a, np.ndarray):
        if a.dtype != np.float64 or not (a.flags.f_contiguous or a.flags.c_contiguous):
            raise TypeError("numpy grid arrays must be contiguous float64")
        return a.ctypes.data, a.size, False
    try:
        import torch
    except ImportError:  # pragma: no cover
        raise TypeError("unsupported array type %r" % type(a))
    if isinstance(a, torch.Tensor):
        if a.dtype != torch.float64 or not a.is_contiguous():
            raise TypeError("tensor grid arrays must be contiguous float64")
        return a.data_ptr(), a.numel(), a.is_cuda
    raise TypeError("unsupported array type %r" % type(a))


def _default_stream():
    try:
        import torch
        if torch.cuda.is_available() and torch.cuda.is_initialized():
            return torch.cuda.current_stream().cuda_stream
    except Exception:
        pass
    return None


class Multigrid:
    def __init__(self, mesh, number_of_levels, number_of_vcycles, aggregation_method="cgs", cga_level=0,
                 cgpsa_level=(0, 0, 0), coarse_solver="rbgs", precision="fp64", mixed_inner_cycles=0,
                 stream=None):
        self._lib = _lib.load()
        (dxm, dxg, xg), (dym, dyg, yg), (dzm, dzg, zg) = [tuple(np.ascontiguousarray(a, dtype=np.float64)
                                                               for a in m) for m in mesh]
        self._keep = (dxm, dxg, xg, dym, dyg, yg, dzm, dzg, zg)
        self.n = (dxm.size - 2, dym.size - 2, dzm.size - 2)
        cfg = PmgConfig()
        cfg.nx, cfg.ny, cfg.nz = self.n
        for name, arr in zip(("dxm", "dxg", "xg", "dym", "dyg", "yg", "dzm", "dzg", "zg"), self._keep):
            setattr(cfg, name, arr.ctypes.data)
        cfg.number_of_levels = int(number_of_levels)
        cfg.number_of_vcycles = int(number_of_vcycles)
        cfg.aggregation_method = _code(_METHODS, aggregation_method)
        cfg.cga_level = int(cga_level)
        cfg.cgpsa_level[:] = [int(v) for v in cgpsa_level]
        cfg.coarse_solver = _code(_COARSE, coarse_solver)
        cfg.precision = _code(_PREC, precision)
        cfg.mixed_inner_cycles = int(mixed_inner_cycles)
        self.number_of_levels = cfg.number_of_levels
        self.number_of_vcycles = cfg.number_of_vcycles
        self.precision = cfg.precision
        self.stream = _default_stream() if stream is None else stream
        h = ctypes.c_void_p()
        check(self._lib.pmg_create(ctypes.byref(h), ctypes.byref(cfg), self.stream), "multigrid_create")
        self._h = h

    # -- life cycle -------------------------------------------------------------------
    def destroy(self):
        if getattr(self, "_h", None):
            self._lib.pmg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.destroy()

    # -- hierarchy ----------------------------------------------------------------------
    def level_dims(self, level):
        d = (ctypes.c_int * 3)()
        check(self._lib.pmg_level_dims(self._h, level, d), "level_dims")
        return tuple(d)

    def level_mesh(self, level, axis):
        n = self.level_dims(level)[axis]
        dm, dg, xg = np.zeros(n + 2), np.zeros(n + 2), np.zeros(n + 2)
        check(self._lib.pmg_level_mesh(self._h, level, axis, dm.ctypes.data, dg.ctypes.data, xg.ctypes.data),
              "level_mesh")
        return dm, dg, xg

    def coarsest_levels(self):
        d = (ctypes.c_int * 3)()
        check(self._lib.pmg_coarsest_levels(self._h, d), "coarsest_levels")
        return tuple(d)

    def _size(self, level):
        nx, ny, nz = self.level_dims(level)
        return (nx + 2) * (ny + 2) * (nz + 2)

    def _dev(self, a, level, what):
        p, n, is_dev = _ptr(a)
        if n != self._size(level):
            raise ValueError("%s has %d elements, level %d needs %d" % (what, n, level, self._size(level)))
        if not is_dev:
            raise TypeError("%s must be a CUDA tensor for the level operations" % what)
        return p

    # -- the solve ----------------------------------------------------------------------
    def solve_vcycle(self, sol, rsd, rhs, maxiteration, tolerance, omega_sor):
        """multigrid_solve_vcycle (src/multigrid.f90:1864)."""
        ps, ns, ds = _ptr(sol)
        pr, nr, dr = _ptr(rsd)
        pb, nb, db = _ptr(rhs)
        need = self._size(0)
        if not (ns == nr == nb == need):
            raise ValueError("sol, rsd and rhs must have %d elements" % need)
        hist = np.zeros(3 * max(self.number_of_vcycles, 1))
        citers = np.zeros(max(self.number_of_vcycles, 1), dtype=np.int32)
        rep = PmgReport()
        rep.history = hist.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        rep.coarse_iterations = citers.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        rc = self._lib.pmg_solve_vcycle(self._h, ps, pr, pb, int(maxiteration), float(tolerance),
                                        float(omega_sor), ctypes.byref(rep))
        out = SolveReport(rep.cycles, bool(rep.converged), rep.res0, rep.final_ratio,
                          hist[:3 * rep.cycles].reshape(rep.cycles, 3).copy(), citers[:rep.cycles].copy(),
                          rep.elapsed_ms, rep.inner_cycles)
        if rc == _lib.PMG_EDIVERGED:
            err = _lib.PmgError(rc, "multigrid_solve_vcycle")
            err.report = out
            raise err
        check(rc, "multigrid_solve_vcycle")
        return out

    # -- level operations (device arrays) ---------------------------------------------------
    def mv_mul(self, level, y, x):
        check(self._lib.pmg_mv_mul(self._h, level, self._dev(y, level, "y"), self._dev(x, level, "x")), "mv_mul")

    def vv_dot(self, level, x, y):
        r = ctypes.c_double()
        check(self._lib.pmg_vv_dot(self._h, level, self._dev(x, level, "x"), self._dev(y, level, "y"),
                                   ctypes.byref(r)), "vv_dot")
        return r.value

    def residual(self, level, r, x, b):
        check(self._lib.pmg_residual(self._h, level, self._dev(r, level, "r"), self._dev(x, level, "x"),
                                     self._dev(b, level, "b")), "residual")

    def rbgs_iterator(self, level, x, b, maxiteration, omega):
        check(self._lib.pmg_rbgs_iterator(self._h, level, self._dev(x, level, "x"), self._dev(b, level, "b"),
                                          int(maxiteration), float(omega)), "rbgs_iterator")

    def rbgs_solver(self, level, x, b, maxiteration, tolerance, omega):
        it, ratio = ctypes.c_int(), ctypes.c_double()
        check(self._lib.pmg_rbgs_solver(self._h, level, self._dev(x, level, "x"), self._dev(b, level, "b"),
                                        int(maxiteration), float(tolerance), float(omega), ctypes.byref(it),
                                        ctypes.byref(ratio)), "rbgs_solver")
        return it.value, ratio.value

    def cg_iterator(self, level, x, b, maxiteration):
        check(self._lib.pmg_cg_iterator(self._h, level, self._dev(x, level, "x"), self._dev(b, level, "b"),
                                        int(maxiteration)), "cg_iterator")

    def cg_solver(self, level, x, b, maxiteration, tolerance):
        it, ratio = ctypes.c_int(), ctypes.c_double()
        check(self._lib.pmg_cg_solver(self._h, level, self._dev(x, level, "x"), self._dev(b, level, "b"),
                                      int(maxiteration), float(tolerance), ctypes.byref(it), ctypes.byref(ratio)),
              "cg_solver")
        return it.value, ratio.value

    def restriction(self, level, val_c, val_f):
        check(self._lib.pmg_restriction(self._h, level, self._dev(val_c, level + 1, "val_c"),
                                        self._dev(val_f, level, "val_f")), "restriction")

    def prolongation(self, level, val_f, val_c):
        check(self._lib.pmg_prolongation(self._h, level, self._dev(val_f, level, "val_f"),
                                         self._dev(val_c, level + 1, "val_c")), "prolongation")

    def prolong_add(self, level, x_f, x_c):
        check(self._lib.pmg_prolong_add(self._h, level, self._dev(x_f, level, "x_f"),
                                        self._dev(x_c, level + 1, "x_c")), "prolong_add")

    def sync(self):
        check(self._lib.pmg_sync(self._h), "sync")

    # -- adjoint --------------------------------------------------------------------------
    def adjoint(self, dLdu, dLdb, maxiteration, tolerance, omega_sor):
        """Gradients of a loss of the solution (pmg_adjoint): fills dLdb (device array of
        the finest level) and returns (SolveReport of the transposed solve, dL/dg[6])."""
        g = (ctypes.c_double * 6)()
        hist = np.zeros(3 * max(self.number_of_vcycles, 1))
        citers = np.zeros(max(self.number_of_vcycles, 1), dtype=np.int32)
        rep = PmgReport()
        rep.history = hist.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        rep.coarse_iterations = citers.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        rc = self._lib.pmg_adjoint(self._h, self._dev(dLdu, 0, "dLdu"), self._dev(dLdb, 0, "dLdb"), g,
                                   int(maxiteration), float(tolerance), float(omega_sor), ctypes.byref(rep))
        check(rc, "adjoint")
        out = SolveReport(rep.cycles, bool(rep.converged), rep.res0, rep.final_ratio,
                          hist[:3 * rep.cycles].reshape(rep.cycles, 3).copy(), citers[:rep.cycles].copy(),
                          rep.elapsed_ms, rep.inner_cycles)
        return out, np.array(g[:])

    # -- telemetry ----------------------------------------------------------------------------
    def profile(self, enable=True):
        """Enable (and reset) or disable CUDA-event timing of the finest-level launches."""
        check(self._lib.pmg_profile(self._h, 1 if enable else 0), "profile")

    def profile_read(self, kernel_class):
        """(total_ms, launches, algorithmic bytes per launch) of a PROF_* kernel class."""
        t, n, b = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_double()
        check(self._lib.pmg_profile_read(self._h, int(kernel_class), ctypes.byref(t), ctypes.byref(n),
                                         ctypes.byref(b)), "profile_read")
        return t.value, n.value, b.value


PROF_CLASSES = {0: "smooth32", 1: "outer_residual64", 2: "resrestrict32", 3: "prolong32", 4: "add_correction64",
                5: "tail32", 6: "smooth64", 7: "residual64", 8: "restrict64", 9: "prolong64", 10: "tail64",
                11: "update_residual", 12: "coarse_levels32", 13: "coarse_levels64"}


def launch_count():
    """Kernels launched by the library in this process so far."""
    n = ctypes.c_longlong()
    check(_lib.load().pmg_launch_count(ctypes.byref(n)), "launch_count")
    return n.value


def level_sizes(n, number_of_levels, aggregation_method="cgs", cga_level=0):
    """Level sizes of the hierarchy (host only).  Returns (sizes[(L+1),3], lv_coarsest[3]);
    raises PmgError where the reference stops with an error."""
    lib = _lib.load()
    L = int(number_of_levels)
    sizes = (ctypes.c_int * (3 * (max(L, 0) + 1)))()
    co = (ctypes.c_int * 3)()
    check(lib.pmg_level_sizes(int(n[0]), int(n[1]), int(n[2]), L, _code(_METHODS, aggregation_method), int(cga_level),
                              sizes, co), "level_sizes")
    return np.array(sizes, dtype=np.int64).reshape(-1, 3), tuple(co)


def multigrid_create(mesh, nlevel, ncycle, aggr_method, single_aggr_level=0, adaptive_aggr_level=(0, 0, 0), **kw):
    """multigrid_create(sdm, nlevel, ncycle, aggr_method, single_aggr_level,
    adaptive_aggr_level) -- src/multigrid.f90:75."""
    return Multigrid(mesh, nlevel, ncycle, aggr_method, single_aggr_level, adaptive_aggr_level, **kw)


def multigrid_solve_vcycle(mg, sol, rsd, rhs, maxiteration, tolerance, omega_sor):
    """multigrid_solve_vcycle -- src/multigrid.f90:1864."""
    return mg.solve_vcycle(sol, rsd, rhs, maxiteration, tolerance, omega_sor)


def multigrid_destroy(mg):
    """multigrid_destroy -- src/multigrid.f90:1320."""
    mg.destroy()


def _config(mesh, number_of_levels, number_of_vcycles, keep):
    """A PmgConfig of the plain FP64 CGS path for a global mesh (keep holds the arrays)."""
    arrs = [tuple(np.ascontiguousarray(a, dtype=np.float64) for a in m) for m in mesh]
    keep.extend(arrs)
    cfg = PmgConfig()
    cfg.nx, cfg.ny, cfg.nz = (arrs[d][0].size - 2 for d in range(3))
    for d, a in enumerate("xyz"):
        setattr(cfg, "d%sm" % a, arrs[d][0].ctypes.data)
        setattr(cfg, "d%sg" % a, arrs[d][1].ctypes.data)
        setattr(cfg, "%sg" % a, arrs[d][2].ctypes.data)
    cfg.number_of_levels = int(number_of_levels)
    cfg.number_of_vcycles = int(number_of_vcycles)
    cfg.aggregation_method = 0
    cfg.coarse_solver = 0
    cfg.precision = 0
    return cfg


class DecomposedMultigrid:
    """The reference's multi-rank CGS V-cycle on a procs[0] x procs[1] x procs[2]
    decomposition of one grid, every subdomain on this process's GPU (pmg_dd_*): the
    subdomains exchange ghost layers where the reference's MPI code does, and the solution
    equals the one-grid solution bit for bit.  mesh is the GLOBAL mesh; solve_vcycle takes
    the global (nx+2)(ny+2)(nz+2) CUDA tensors."""

    def __init__(self, mesh, procs, number_of_levels, number_of_vcycles, stream=None):
        self._lib = _lib.load()
        self._keep = []
        cfg = _config(mesh, number_of_levels, number_of_vcycles, self._keep)
        self.n = (cfg.nx, cfg.ny, cfg.nz)
        self.number_of_vcycles = cfg.number_of_vcycles
        p = (ctypes.c_int * 3)(*[int(v) for v in procs])
        self.stream = _default_stream() if stream is None else stream
        h = ctypes.c_void_p()
        check(self._lib.pmg_dd_create(ctypes.byref(h), ctypes.byref(cfg), p, self.stream), "pmg_dd_create")
        self._h = h

    def destroy(self):
        if getattr(self, "_h", None):
            self._lib.pmg_dd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.destroy()

    def solve_vcycle(self, sol, rsd, rhs, maxiteration, tolerance, omega_sor):
        need = (self.n[0] + 2) * (self.n[1] + 2) * (self.n[2] + 2)
        ptrs = []
        for a, what in ((sol, "sol"), (rsd, "rsd"), (rhs, "rhs")):
            p, n, dev = _ptr(a)
            if n != need or not dev:
                raise ValueError("%s must be a CUDA tensor of %d elements" % (what, need))
            ptrs.append(p)
        hist = np.zeros(3 * max(self.number_of_vcycles, 1))
        citers = np.zeros(max(self.number_of_vcycles, 1), dtype=np.int32)
        rep = PmgReport()
        rep.history = hist.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        rep.coarse_iterations = citers.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        check(self._lib.pmg_dd_solve(self._h, ptrs[0], ptrs[1], ptrs[2], int(maxiteration), float(tolerance),
                                     float(omega_sor), ctypes.byref(rep)), "pmg_dd_solve")
        return SolveReport(rep.cycles, bool(rep.converged), rep.res0, rep.final_ratio,
                           hist[:3 * rep.cycles].reshape(rep.cycles, 3).copy(), citers[:rep.cycles].copy(),
                           rep.elapsed_ms, rep.inner_cycles)


def dd_partition(mesh, procs, coords, level, number_of_levels):
    """The subdomain of the rank at `coords` in a procs decomposition of the global mesh
    (host only): (dims, [(dm, dg, xg) per axis], colour offset) on `level`."""
    lib = _lib.load()
    keep = []
    cfg = _config(mesh, number_of_levels, 1, keep)
    p = (ctypes.c_int * 3)(*[int(v) for v in procs])
    c = (ctypes.c_int * 3)(*[int(v) for v in coords])
    dims = (ctypes.c_int * 3)()
    off = ctypes.c_int()
    check(lib.pmg_dd_partition(ctypes.byref(cfg), p, c, int(level), dims, None, ctypes.byref(off)), "pmg_dd_partition")
    d = tuple(dims)
    bufs = [np.zeros(d[a] + 2) for a in range(3) for _ in range(3)]
    ptrs = (ctypes.c_void_p * 9)(*[b.ctypes.data for b in bufs])
    check(lib.pmg_dd_partition(ctypes.byref(cfg), p, c, int(level), dims, ptrs, ctypes.byref(off)),
          "pmg_dd_partition")
    return d, [tuple(bufs[3 * a:3 * a + 3]) for a in range(3)], off.value
