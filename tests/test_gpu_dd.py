"""The decomposed solve (pmg_dd_*, the reference's multi-rank CGS execution with every
subdomain on one GPU) against the one-grid solve and the oracle's multi-rank restatement.

The subdomains exchange ghost layers by device-side packing, cudaMemcpyAsync and unpacking
where the reference's MPI code exchanges them, and start their RBGS colours at the
rank-parity offset.  So the solution and the residual must equal, bit for bit, those of a
single context on the whole grid and those of the oracle's px x py x pz restatement (which
equal the oracle's one-rank solve); residual histories agree to 1e-12 (the norms are sums
over the subdomains), coarsest iteration counts are equal.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import peps_mg_gb300 as pmg  # noqa: E402
from oracle import oracle as O  # noqa: E402
from peps_mg_gb300 import geometry as G  # noqa: E402
from peps_mg_gb300 import problems  # noqa: E402
from tests.helpers import from_dev, to_dev  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()


def random_rhs(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    rhs = G.field(*n)
    rhs[1:-1, 1:-1, 1:-1] = rng.uniform(-1.0, 1.0, size=n)
    return np.asfortranarray(rhs)


def problem(case):
    if case == "blobs48":
        mesh, rhs = problems.gaussian_blobs(48)
        return mesh, np.asfortranarray(rhs)
    if case == "odd24":
        ax = G.uniform_axis(24, 0.0, 1.0)
        return [ax, ax, ax], random_rhs((24, 24, 24), 5)
    mesh = [G.stretched_axis(40, 0.0, 1.0, 1.1), G.uniform_axis(24, 0.0, 2.0), G.tanh_axis(32, 0.0, 1.0, 1.3)]
    return mesh, random_rhs((40, 24, 32), 6)


@pytest.mark.parametrize("case,procs,nl", [("blobs48", (2, 1, 1), 3), ("blobs48", (1, 2, 2), 3),
                                           ("blobs48", (2, 2, 2), 3), ("blobs48", (4, 1, 1), 2),
                                           ("odd24", (2, 2, 2), 2), ("stretched", (2, 2, 2), 2),
                                           ("stretched", (1, 3, 1), 2)])
def test_decomposed_equals_one_grid(case, procs, nl):
    mesh, rhs = problem(case)
    n = tuple(len(m[0]) - 2 for m in mesh)
    # a non-zero Dirichlet face: the global ghost values reach the boundary subdomains
    sol0 = G.field(*n)
    sol0[:, :, -1] = 0.25
    with pmg.Multigrid(mesh, nl, 60, "cgs") as mg:
        s1, r1 = to_dev(sol0), torch.zeros_like(to_dev(rhs))
        rep1 = mg.solve_vcycle(s1, r1, to_dev(rhs), 2, 1e-10, 1.0)
    with pmg.DecomposedMultigrid(mesh, procs, nl, 60) as dd:
        s2, r2 = to_dev(sol0), torch.zeros_like(to_dev(rhs))
        rep2 = dd.solve_vcycle(s2, r2, to_dev(rhs), 2, 1e-10, 1.0)
    torch.cuda.synchronize()
    assert rep2.converged and rep2.cycles == rep1.cycles
    assert torch.equal(s1, s2), "decomposed solution differs from the one-grid solution"
    assert torch.equal(r1, r2), "decomposed residual differs from the one-grid residual"
    assert np.abs(rep1.history[:, 2] - rep2.history[:, 2]).max() <= 1e-12 * np.abs(rep1.history[:, 2]).max()
    assert np.array_equal(rep1.coarse_iterations, rep2.coarse_iterations)
    # the oracle's multi-rank restatement
    od = O.OracleDD(mesh, procs, nl, 60)
    osol, orsd = np.asfortranarray(sol0.copy()), O.field(*n)
    ocyc, _, ci = od.solve(osol, orsd, rhs, 2, 1e-10, 1.0)
    od.close()
    assert ocyc == rep2.cycles
    assert np.array_equal(from_dev(s2), osol)
    assert np.array_equal(from_dev(r2), orsd)


def test_decomposition_rejects_what_the_reference_rejects():
    ax = G.uniform_axis(24, 0.0, 1.0)
    with pytest.raises(pmg.PmgError):
        pmg.DecomposedMultigrid([ax, ax, ax], (2, 1, 1), 3, 10)    # 12, 6, 3: cannot halve again
    with pytest.raises(pmg.PmgError):
        pmg.DecomposedMultigrid([ax, ax, ax], (5, 1, 1), 2, 10)    # 24 not divisible by 5
