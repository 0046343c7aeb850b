"""The 512^3 mixed-precision workload at full size, pinned against the oracle.

Problem: the seeded Gaussian-blob right-hand side (8 Gaussians, sigma 0.05, amplitudes
U[-10,10], plus 1e-3 U[-1,1] noise, PCG64(3)) on the unit cube, zero Dirichlet ghosts,
8 levels down to 2^3, V(2,2) RBGS with omega 1, tolerance 1e-10 -- the CGS cycle of
src/multigrid.f90:1907-1976 from x0 = 0.

(a) The plain FP64 GPU solve against the oracle's FP64 solve (OpenMP over the host
    cores): the solution and residual arrays bit for bit, the residual-ratio history
    within 1e-12 relative (the norms are sums in another order), the coarsest-level
    iteration counts equal.
(b) The mixed solve (FP32 V-cycles inside FP64 defect correction) against the oracle's
    solution: max-abs error within 1e-8 of max |u| and relative L2 error within 1e-8;
    the returned residual is the FP64 b - A x of the returned solution (to within a few
    ulps of |c0| |x|: the mixed path evaluates it with FMA).
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import peps_mg_gb300 as pmg  # noqa: E402
from oracle import oracle as O  # noqa: E402
from peps_mg_gb300 import problems  # noqa: E402
from tests.helpers import from_dev, rel, to_dev  # noqa: E402

N = 512
LEVELS = 8
HIST_TOL = 1e-12
MIXED_TOL = 1e-8


@pytest.fixture(scope="module")
def oracle_512():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    mesh, rhs = problems.gaussian_blobs(N)
    rhs = np.asfortranarray(rhs)
    O.set_threads(os.cpu_count() or 1)
    omg = O.OracleMG(mesh, LEVELS, 40, 0, omp=True)
    osol, orsd = O.field(N, N, N), O.field(N, N, N)
    ncyc, hist, ci = omg.solve(osol, orsd, rhs, 2, 1e-10, 1.0)
    omg.close()
    return mesh, rhs, osol, orsd, ncyc, hist, ci


def test_fp64_512_equals_oracle(oracle_512):
    mesh, rhs, osol, orsd, ncyc, hist, ci = oracle_512
    with pmg.Multigrid(mesh, LEVELS, 40, "cgs", precision="fp64") as mg:
        b = to_dev(rhs)
        sol = torch.zeros_like(b)
        rsd = torch.zeros_like(b)
        rep = mg.solve_vcycle(sol, rsd, b, 2, 1e-10, 1.0)
        torch.cuda.synchronize()
    assert rep.converged and rep.cycles == ncyc
    assert rel(rep.history, hist) < HIST_TOL
    assert np.array_equal(rep.coarse_iterations, ci)
    assert np.array_equal(from_dev(sol), osol), "FP64 solution differs from the oracle's bits"
    assert np.array_equal(from_dev(rsd), orsd), "FP64 residual differs from the oracle's bits"


def test_mixed_512_against_oracle(oracle_512):
    mesh, rhs, osol, _, _, _, _ = oracle_512
    with pmg.Multigrid(mesh, LEVELS, 40, "cgs", precision="mixed", mixed_inner_cycles=4) as mg:
        b = to_dev(rhs)
        sol = torch.zeros_like(b)
        rsd = torch.zeros_like(b)
        rep = mg.solve_vcycle(sol, rsd, b, 2, 1e-10, 1.0)
        torch.cuda.synchronize()
        # the returned residual is the FP64 b - A x of the returned solution
        r_check = torch.zeros_like(b)
        mg.residual(0, r_check, sol, b)
        torch.cuda.synchronize()
        r_diff = (r_check - rsd).abs().max().item()
        x_max = sol.abs().max().item()
    assert rep.converged and rep.final_ratio < 1e-10
    s = from_dev(sol)[1:-1, 1:-1, 1:-1]
    o = osol[1:-1, 1:-1, 1:-1]
    max_abs = np.abs(s - o).max() / np.abs(o).max()
    l2 = np.linalg.norm(s - o) / np.linalg.norm(o)
    assert max_abs < MIXED_TOL, max_abs
    assert l2 < MIXED_TOL, l2
    # FMA vs non-FMA rounding of the same FP64 residual formula only: a few ulps of the
    # largest term, |c0| |x| with |c0| = 6 / h^2 on the uniform 512^3 mesh
    c0 = 6.0 * N * N
    assert r_diff <= 8 * np.finfo(np.float64).eps * c0 * x_max, (r_diff, x_max)
