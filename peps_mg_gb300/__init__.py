"""peps_mg_gb300 -- GB300 (sm_103a) multigrid V-cycle solver for the 3-D Poisson
equation on cell-centred, non-uniform Cartesian grids; a drop-in for the solve path of
PEPS_MG (multigrid_create / multigrid_solve_vcycle / multigrid_destroy).
"""
from . import geometry  # noqa: F401
from .autograd import PoissonSolve  # noqa: F401
from .batch import BatchSolver  # noqa: F401
from ._lib import (PMG_CGA, PMG_CGPSA, PMG_CGS, PMG_COARSE_CG, PMG_COARSE_RBGS, PMG_FP64,  # noqa: F401
                   PMG_FP64_FAST, PMG_MIXED, PmgError, load)
from .multigrid import (PROF_CLASSES, DecomposedMultigrid, Multigrid, SolveReport, dd_partition,  # noqa: F401
                        launch_count, level_sizes, multigrid_create, multigrid_destroy, multigrid_solve_vcycle)

__all__ = ["Multigrid", "SolveReport", "PmgError", "multigrid_create", "multigrid_solve_vcycle",
           "multigrid_destroy", "level_sizes", "geometry", "load", "BatchSolver", "PoissonSolve",
           "DecomposedMultigrid", "dd_partition"]
