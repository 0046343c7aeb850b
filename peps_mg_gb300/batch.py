"""Batched solver: many independent problems of uneven sizes in one set of launches.

    bs = BatchSolver(dims)                      # dims: (n, 3) sizes; uniform meshes of cubic cells
    sol, rhs = bs.field(), bs.field()           # packed CUDA arrays
    bs.view(rhs, p)[...] = ...                  # problem p as a (nz+2, ny+2, nx+2) view
    cycles, ratio, ms = bs.solve(sol, rhs, 2, 1e-10, 1.0, max_cycles=50)

Every problem is solved in mixed precision (FP32 V-cycles in FP64 defect correction) on
its own hierarchy; see include/peps_mg.h (pmg_batch_*).
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check


class BatchSolver:
    def __init__(self, dims, meshes=None, mixed_inner_cycles=2, stream=None):
        self._lib = _lib.load()
        d = np.ascontiguousarray(np.asarray(dims, dtype=np.int32).reshape(-1, 3))
        self.dims = d
        self.n = d.shape[0]
        mp = None
        self._keep = []
        if meshes is not None:
            arr = (ctypes.c_void_p * (6 * self.n))()
            for p, m in enumerate(meshes):
                if m is None:
                    continue
                for ax in range(3):
                    dm = np.ascontiguousarray(m[ax][0], dtype=np.float64)
                    dg = np.ascontiguousarray(m[ax][1], dtype=np.float64)
                    self._keep += [dm, dg]
                    arr[6 * p + 2 * ax] = dm.ctypes.data
                    arr[6 * p + 2 * ax + 1] = dg.ctypes.data
            mp = arr
        h = ctypes.c_void_p()
        check(self._lib.pmg_batch_create(ctypes.byref(h), self.n, d.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                         mp, int(mixed_inner_cycles), stream), "batch_create")
        self._h = h
        off = (ctypes.c_longlong * (self.n + 1))()
        lev = (ctypes.c_int * self.n)()
        check(self._lib.pmg_batch_layout(self._h, off, lev), "batch_layout")
        self.offsets = np.array(off[:], dtype=np.int64)
        self.levels = np.array(lev[:], dtype=np.int32)

    def mesh(self, p):
        """The default mesh of problem p (no meshes given): cubic cells of width
        1/max(nx, ny, nz), the same values the library builds."""
        from . import geometry as G
        d = [int(v) for v in self.dims[p]]
        h = 1.0 / float(max(d))
        return [G.mesh_from_widths(np.full(m, h)) for m in d]

    @property
    def total(self):
        return int(self.offsets[-1])

    def field(self, device="cuda"):
        import torch
        return torch.zeros(self.total, dtype=torch.float64, device=device)

    def view(self, packed, p):
        nx, ny, nz = (int(v) for v in self.dims[p])
        return packed[self.offsets[p]:self.offsets[p + 1]].view(nz + 2, ny + 2, nx + 2)

    def solve(self, sol, rhs, maxiteration=2, tolerance=1e-10, omega=1.0, max_cycles=100):
        cyc = (ctypes.c_int * self.n)()
        rat = (ctypes.c_double * self.n)()
        ms = ctypes.c_float()
        check(self._lib.pmg_batch_solve(self._h, sol.data_ptr(), rhs.data_ptr(), int(maxiteration), float(tolerance),
                                        float(omega), int(max_cycles), cyc, rat, ctypes.byref(ms)), "batch_solve")
        return np.array(cyc[:]), np.array(rat[:]), ms.value

    def destroy(self):
        if getattr(self, "_h", None):
            self._lib.pmg_batch_destroy(self._h)
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
