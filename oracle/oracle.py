"""ctypes wrapper of the CPU oracle (oracle/pmg_oracle.c) -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py (its cpu_baseline leg and the
``--impl reference`` arm) import this module.  The product path in peps_mg_gb300 never
does.  Arrays are numpy float64, Fortran-ordered with one ghost layer, shape
(nx+2, ny+2, nz+2) in ``order="F"``.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS = {}

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build():
    """Compile the oracle shared libraries in place (plain and OpenMP variants)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def _lib(omp=False):
    name = "libpmg_oracle_omp.so" if omp else "libpmg_oracle.so"
    if name not in _LIBS:
        path = os.path.join(_HERE, name)
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(
                os.path.join(_HERE, "pmg_oracle.c")):
            build()
        lib = ctypes.CDLL(path)
        lib.orc_vv_dot.restype = ctypes.c_double
        lib.orc_mg_create.restype = ctypes.c_void_p
        lib.orc_mg_level_coeff.restype = _dp
        lib.orc_mg_destroy.argtypes = [ctypes.c_void_p]
        lib.orc_dd_create.restype = ctypes.c_void_p
        lib.orc_dd_destroy.argtypes = [ctypes.c_void_p]
        for fn in ("orc_mg_solve", "orc_mg_level_dims", "orc_mg_coarsest", "orc_mg_level_mesh",
                   "orc_mg_level_coeff", "orc_dd_solve", "orc_dd_offset", "orc_dd_level_dims"):
            getattr(lib, fn).argtypes = None
        _LIBS[name] = lib
    return _LIBS[name]


def P(a):
    """Pointer to a Fortran-ordered (column-major) contiguous float64 numpy array."""
    assert a.dtype == np.float64 and a.flags.f_contiguous, "oracle arrays must be float64 in Fortran order"
    return a.ctypes.data_as(_dp)


def field(nx, ny, nz, fill=0.0):
    return np.full((nx + 2, ny + 2, nz + 2), fill, dtype=np.float64, order="F")


def set_threads(n, omp=True):
    _lib(omp).orc_set_threads(ctypes.c_int(n))


def max_threads(omp=True):
    return _lib(omp).orc_max_threads()


def mesh_axis(n, o, length, a):
    """geometry_domain_create along one axis: returns (dxm, dxg, xg), each length n+2."""
    dm = np.zeros(n + 2); dg = np.zeros(n + 2); xg = np.zeros(n + 2)
    _lib().orc_mesh_axis(ctypes.c_int(n), ctypes.c_double(o), ctypes.c_double(length),
                         ctypes.c_double(a), P(dm), P(dg), P(xg))
    return dm, dg, xg


def level_sizes(nx, ny, nz, n_levels, method, cga_level=0):
    """Level-size rules; returns (rc, sizes[(n_levels+1),3], coarsest[3])."""
    sizes = np.zeros((n_levels + 1) * 3, dtype=np.int32)
    co = np.zeros(3, dtype=np.int32)
    rc = _lib().orc_level_sizes(ctypes.c_int(nx), ctypes.c_int(ny), ctypes.c_int(nz),
                                ctypes.c_int(n_levels), ctypes.c_int(method), ctypes.c_int(cga_level),
                                sizes.ctypes.data_as(_ip), co.ctypes.data_as(_ip))
    return rc, sizes.reshape(-1, 3), co


def matrix_create(mesh):
    (dxm, dxg, _), (dym, dyg, _), (dzm, dzg, _) = mesh
    nx, ny, nz = len(dxm) - 2, len(dym) - 2, len(dzm) - 2
    coeff = np.zeros((7, nx, ny, nz), order="F")
    _lib().orc_matrix_create(nx, ny, nz, P(dxm), P(dxg), P(dym), P(dyg), P(dzm), P(dzg), P(coeff))
    return coeff


def dims_of(x):
    return x.shape[0] - 2, x.shape[1] - 2, x.shape[2] - 2


def mv_mul(coeff, x, omp=False):
    y = np.empty_like(x, order="F")
    _lib(omp).orc_mv_mul(*dims_of(x), P(coeff), P(x), P(y))
    return y


def vv_dot(x, y, omp=False):
    return _lib(omp).orc_vv_dot(*dims_of(x), P(x), P(y))


def residual(coeff, x, b, omp=False):
    r = np.empty_like(x, order="F")
    _lib(omp).orc_residual(*dims_of(x), P(coeff), P(x), P(b), P(r))
    return r


def rbgs_iterator(coeff, x, b, maxiteration, omega, omp=False):
    """In place on x."""
    _lib(omp).orc_rbgs_iterator(*dims_of(x), P(coeff), P(x), P(b), ctypes.c_int(maxiteration),
                                ctypes.c_double(omega))


def rbgs_solver(coeff, x, b, maxiteration, tolerance, omega, omp=False):
    """In place on x; returns (iterations, ||r||^2, ||r0||^2)."""
    rsd = np.zeros_like(x, order="F")
    n2 = ctypes.c_double(); n02 = ctypes.c_double()
    it = _lib(omp).orc_rbgs_solver(*dims_of(x), P(coeff), P(x), P(b), ctypes.c_int(maxiteration),
                                   ctypes.c_double(tolerance), ctypes.c_double(omega), P(rsd),
                                   ctypes.byref(n2), ctypes.byref(n02))
    return it, n2.value, n02.value


def cg(coeff, x, b, maxiteration, tolerance, check_tol=True, omp=False):
    """CG solver (check_tol) or iterator, in place on x; returns (iters, ||r||^2, ||r0||^2)."""
    work = np.zeros(4 * x.size)
    n2 = ctypes.c_double(); n02 = ctypes.c_double()
    it = _lib(omp).orc_cg(*dims_of(x), P(coeff), P(x), P(b), ctypes.c_int(maxiteration),
                          ctypes.c_double(tolerance), ctypes.c_int(1 if check_tol else 0), P(work),
                          ctypes.byref(n2), ctypes.byref(n02))
    return it, n2.value, n02.value


def rbgs_colour(coeff, x, b, omega, colour, offset):
    """One RBGS colour (0 first, 1 second) with a rank's start offset, in place on x."""
    _lib().orc_rbgs_colour(*dims_of(x), P(coeff), P(x), P(b), ctypes.c_double(omega), ctypes.c_int(colour),
                           ctypes.c_int(offset))


def restriction(mesh_c, mesh_f, level, coarsest, val_f, val_c):
    """multigrid_restriction of val_f into val_c (meshes: (dm, dg, xg) per axis)."""
    ci = (ctypes.c_int * 3)(*coarsest)
    _lib().orc_restriction(*dims_of(val_c), P(mesh_c[0][0]), P(mesh_c[1][0]), P(mesh_c[2][0]), *dims_of(val_f),
                           P(mesh_f[0][0]), P(mesh_f[1][0]), P(mesh_f[2][0]), ctypes.c_int(level), ci, P(val_f),
                           P(val_c))


def prolongation(mesh_c, mesh_f, level, coarsest, val_c, val_f):
    """multigrid_prolongation_linear_on_nonuniform_grid of val_c into val_f."""
    ci = (ctypes.c_int * 3)(*coarsest)
    _lib().orc_prolongation(*dims_of(val_c), P(mesh_c[0][0]), P(mesh_c[1][0]), P(mesh_c[2][0]), *dims_of(val_f),
                            P(mesh_f[0][0]), P(mesh_f[1][0]), P(mesh_f[2][0]), ctypes.c_int(level), ci, P(val_c),
                            P(val_f))


class OracleMG:
    """multigrid_create / multigrid_solve_vcycle / multigrid_destroy on the CPU."""

    def __init__(self, mesh, n_levels, n_vcycles, method=0, cga_level=0, coarse_solver=0, omp=False):
        self._lib = _lib(omp)
        (dxm, dxg, xg), (dym, dyg, yg), (dzm, dzg, zg) = mesh
        self.mesh = mesh
        self.n = (len(dxm) - 2, len(dym) - 2, len(dzm) - 2)
        self.n_levels = n_levels
        self.n_vcycles = n_vcycles
        err = ctypes.c_int()
        h = self._lib.orc_mg_create(ctypes.c_int(self.n[0]), ctypes.c_int(self.n[1]), ctypes.c_int(self.n[2]),
                                    P(dxm), P(dxg), P(xg), P(dym), P(dyg), P(yg), P(dzm), P(dzg), P(zg),
                                    ctypes.c_int(n_levels), ctypes.c_int(n_vcycles), ctypes.c_int(method),
                                    ctypes.c_int(cga_level), ctypes.c_int(coarse_solver), ctypes.byref(err))
        if not h:
            raise ValueError("oracle multigrid_create rejected the configuration (code %d)" % err.value)
        self._h = ctypes.c_void_p(h)

    def close(self):
        if self._h:
            self._lib.orc_mg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def level_dims(self, l):
        d = np.zeros(3, dtype=np.int32)
        self._lib.orc_mg_level_dims(self._h, ctypes.c_int(l), d.ctypes.data_as(_ip))
        return tuple(int(v) for v in d)

    def coarsest(self):
        c = np.zeros(3, dtype=np.int32)
        self._lib.orc_mg_coarsest(self._h, c.ctypes.data_as(_ip))
        return tuple(int(v) for v in c)

    def level_mesh(self, l, axis):
        n = self.level_dims(l)[axis]
        dm = np.zeros(n + 2); dg = np.zeros(n + 2); xg = np.zeros(n + 2)
        self._lib.orc_mg_level_mesh(self._h, ctypes.c_int(l), ctypes.c_int(axis), P(dm), P(dg), P(xg))
        return dm, dg, xg

    def level_coeff(self, l):
        nx, ny, nz = self.level_dims(l)
        ptr = self._lib.orc_mg_level_coeff(self._h, ctypes.c_int(l))
        return np.ctypeslib.as_array(ptr, shape=(7 * nx * ny * nz,)).reshape((7, nx, ny, nz), order="F").copy()

    def solve(self, sol, rsd, rhs, maxiteration, tolerance, omega):
        """In place on sol and rsd; returns (cycles, hist[cycles,3], coarse_iters[cycles])."""
        hist = np.zeros(3 * self.n_vcycles)
        ci = np.zeros(self.n_vcycles, dtype=np.int32)
        ncyc = self._lib.orc_mg_solve(self._h, P(sol), P(rsd), P(rhs), ctypes.c_int(maxiteration),
                                      ctypes.c_double(tolerance), ctypes.c_double(omega), P(hist),
                                      ci.ctypes.data_as(_ip))
        return ncyc, hist[:3 * ncyc].reshape(ncyc, 3), ci[:ncyc]


class OracleDD:
    """The CGS V-cycle on a px x py x pz decomposition of the global problem, every rank
    simulated in this process (halo exchanges, rank-parity colour offsets and rank-ordered
    all-reduces as the reference's MPI code has them).  solve() takes and returns global
    arrays."""

    def __init__(self, mesh, procs, n_levels, n_vcycles, coarse_solver=0, omp=False):
        self._lib = _lib(omp)
        (dxm, dxg, xg), (dym, dyg, yg), (dzm, dzg, zg) = mesh
        self.n = (len(dxm) - 2, len(dym) - 2, len(dzm) - 2)
        self.procs = tuple(int(p) for p in procs)
        self.n_levels = n_levels
        self.n_vcycles = n_vcycles
        err = ctypes.c_int()
        h = self._lib.orc_dd_create(ctypes.c_int(self.n[0]), ctypes.c_int(self.n[1]), ctypes.c_int(self.n[2]),
                                    P(dxm), P(dxg), P(xg), P(dym), P(dyg), P(yg), P(dzm), P(dzg), P(zg),
                                    ctypes.c_int(self.procs[0]), ctypes.c_int(self.procs[1]),
                                    ctypes.c_int(self.procs[2]), ctypes.c_int(n_levels), ctypes.c_int(n_vcycles),
                                    ctypes.c_int(coarse_solver), ctypes.byref(err))
        if not h:
            raise ValueError("oracle multigrid_create on %s ranks rejected the configuration" % (self.procs,))
        self._h = ctypes.c_void_p(h)

    def close(self):
        if self._h:
            self._lib.orc_dd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def offset(self, coords, level):
        return self._lib.orc_dd_offset(self._h, *(ctypes.c_int(c) for c in coords), ctypes.c_int(level))

    def level_dims(self, level):
        d = np.zeros(3, dtype=np.int32)
        self._lib.orc_dd_level_dims(self._h, ctypes.c_int(level), d.ctypes.data_as(_ip))
        return tuple(int(v) for v in d)

    def solve(self, sol, rsd, rhs, maxiteration, tolerance, omega):
        """In place on the global sol and rsd; returns (cycles, hist[cycles,3], coarse_iters)."""
        hist = np.zeros(3 * self.n_vcycles)
        ci = np.zeros(self.n_vcycles, dtype=np.int32)
        ncyc = self._lib.orc_dd_solve(self._h, P(sol), P(rsd), P(rhs), ctypes.c_int(maxiteration),
                                      ctypes.c_double(tolerance), ctypes.c_double(omega), P(hist),
                                      ci.ctypes.data_as(_ip))
        return ncyc, hist[:3 * ncyc].reshape(ncyc, 3), ci[:ncyc]
