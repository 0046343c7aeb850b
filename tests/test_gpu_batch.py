"""Batched solver: every problem of an uneven batch converges, agrees with the single-
problem mixed solver, and (for a sample) with the FP64 oracle."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import peps_mg_gb300 as pmg  # noqa: E402
from oracle import oracle as O  # noqa: E402
from peps_mg_gb300.batch import BatchSolver  # noqa: E402
from tests.helpers import from_dev, rel, to_dev  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def batch_dims(count, sizes, seed=4):
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.choice(sizes, size=(count, 3))


def fill(bs, seed=4):
    rng = np.random.Generator(np.random.PCG64(seed + 100))
    rhs = bs.field()
    for p in range(bs.n):
        v = bs.view(rhs, p)
        nz, ny, nx = (s - 2 for s in v.shape)
        v[1:-1, 1:-1, 1:-1] = torch.from_numpy(rng.uniform(-1, 1, (nz, ny, nx))).cuda()
    return rhs


def test_batch_matches_single_problem_solves():
    dims = batch_dims(12, [8, 12, 16, 24, 32, 48])
    with BatchSolver(dims) as bs:
        rhs = fill(bs)
        sol = bs.field()
        cycles, ratio, ms = bs.solve(sol, rhs, 2, 1e-10, 1.0, max_cycles=60)
        assert np.all(ratio < 1e-10), ratio
        for p in range(bs.n):
            nx, ny, nz = (int(v) for v in dims[p])
            mesh = bs.mesh(p)
            with pmg.Multigrid(mesh, int(bs.levels[p]), 60, "cgs", precision="mixed") as mg:
                s1 = torch.zeros_like(bs.view(rhs, p))
                r1 = torch.zeros_like(s1)
                rep = mg.solve_vcycle(s1, r1, bs.view(rhs, p).contiguous(), 2, 1e-10, 1.0)
            assert abs(rep.cycles - cycles[p]) <= 1
            assert rel(from_dev(bs.view(sol, p)), from_dev(s1)) < 1e-8


def test_batch_nonzero_initial_guess():
    """Problems whose initial guess is not zero (interior values, or a Dirichlet ghost face)
    next to problems that start from zero: the first residual takes the full FP64 stencil
    only for the former, and every problem matches its single-problem solve."""
    dims = batch_dims(6, [16, 24, 32], seed=7)
    with BatchSolver(dims) as bs:
        rhs = fill(bs, seed=7)
        sol = bs.field()
        rng = np.random.default_rng(3)
        starts = []
        for p in range(bs.n):
            v = bs.view(sol, p)
            if p % 3 == 1:
                v[1:-1, 1:-1, 1:-1] = torch.from_numpy(rng.uniform(-0.1, 0.1, tuple(s - 2 for s in v.shape))).cuda()
            elif p % 3 == 2:
                v[:, :, 0] = 0.25
            starts.append(v.clone())
        cycles, ratio, _ = bs.solve(sol, rhs, 2, 1e-10, 1.0, max_cycles=60)
        assert np.all(ratio < 1e-10), ratio
        for p in range(bs.n):
            with pmg.Multigrid(bs.mesh(p), int(bs.levels[p]), 60, "cgs", precision="mixed") as mg:
                s1 = starts[p].clone()
                r1 = torch.zeros_like(s1)
                mg.solve_vcycle(s1, r1, bs.view(rhs, p).contiguous(), 2, 1e-10, 1.0)
            assert rel(from_dev(bs.view(sol, p)), from_dev(s1)) < 1e-8, p


def test_batch_against_fp64_oracle_sample():
    dims = batch_dims(6, [16, 24, 32], seed=11)
    with BatchSolver(dims) as bs:
        rhs = fill(bs, seed=11)
        sol = bs.field()
        cycles, ratio, _ = bs.solve(sol, rhs, 2, 1e-10, 1.0, max_cycles=60)
        assert np.all(ratio < 1e-10)
        for p in (0, 3, 5):
            nx, ny, nz = (int(v) for v in dims[p])
            mesh = bs.mesh(p)
            omg = O.OracleMG(mesh, int(bs.levels[p]), 100, 0)
            ref, rr = O.field(nx, ny, nz), O.field(nx, ny, nz)
            omg.solve(ref, rr, from_dev(bs.view(rhs, p)), 2, 1e-10, 1.0)
            assert rel(from_dev(bs.view(sol, p)), ref) < 1e-8


def test_batch_rejects_bad_sizes():
    with pytest.raises(pmg.PmgError):
        BatchSolver([[9, 9, 9]])


def test_batch_128_problems_full_size():
    """The batched workload at full size: 128 problems, axis sizes from {32..192}
    (PCG64(4)), rhs U[-1,1]; every problem converges, and a sample matches single-problem
    mixed solves and the FP64 oracle."""
    from peps_mg_gb300 import problems
    dims = problems.batch_dims(128)
    with BatchSolver(dims, mixed_inner_cycles=4) as bs:
        rhs = bs.field()
        for p, vals in enumerate(problems.batch_rhs(dims)):
            bs.view(rhs, p)[1:-1, 1:-1, 1:-1] = torch.from_numpy(vals).cuda()
        sol = bs.field()
        cycles, ratio, ms = bs.solve(sol, rhs, 2, 1e-10, 1.0, max_cycles=60)
        assert np.all(ratio < 1e-10), ratio.max()
        order = np.argsort(np.prod(dims, axis=1))
        for p in (int(order[0]), int(order[len(order) // 2]), int(order[-1])):
            nx, ny, nz = (int(v) for v in dims[p])
            mesh = bs.mesh(p)
            with pmg.Multigrid(mesh, int(bs.levels[p]), 60, "cgs", precision="mixed", mixed_inner_cycles=4) as mg:
                s1 = torch.zeros_like(bs.view(rhs, p))
                r1 = torch.zeros_like(s1)
                mg.solve_vcycle(s1, r1, bs.view(rhs, p).contiguous(), 2, 1e-10, 1.0)
            assert rel(from_dev(bs.view(sol, p)), from_dev(s1)) < 1e-8
            omg = O.OracleMG(mesh, int(bs.levels[p]), 100, 0, omp=True)
            ref, rr = O.field(nx, ny, nz), O.field(nx, ny, nz)
            omg.solve(ref, rr, from_dev(bs.view(rhs, p)), 2, 1e-10, 1.0)
            omg.close()
            assert rel(from_dev(bs.view(sol, p)), ref) < 1e-8


def test_batch_random_sizes_and_stretched_meshes():
    """24 problems with random sizes (odd counts that stop coarsening, axes of 6 to 100
    cells) and, for two thirds of them, geometrically stretched meshes: every problem that
    its single-problem mixed solve converges on matches it (cycle count within one,
    solution within 1e-7 of max |u|)."""
    from peps_mg_gb300 import geometry as G
    rng = np.random.default_rng(3)
    dims = rng.choice([6, 8, 10, 12, 16, 20, 24, 30, 32, 40, 48, 64, 72, 96, 100], size=(24, 3))
    meshes = [None if p % 3 == 0 else
              [G.stretched_axis(int(dims[p][d]), 0.0, 1.0, float(rng.uniform(0.97, 1.03))) for d in range(3)]
              for p in range(len(dims))]
    with BatchSolver(dims, meshes=meshes, mixed_inner_cycles=4) as bs:
        rhs = bs.field()
        for p in range(bs.n):
            v = bs.view(rhs, p)
            nz, ny, nx = (s - 2 for s in v.shape)
            v[1:-1, 1:-1, 1:-1] = torch.from_numpy(rng.uniform(-1, 1, (nz, ny, nx))).cuda()
        sol = bs.field()
        cycles, ratio, _ = bs.solve(sol, rhs, 2, 1e-10, 1.0, max_cycles=60)
        checked = 0
        for p in range(bs.n):
            mesh = bs.mesh(p) if meshes[p] is None else meshes[p]
            with pmg.Multigrid(mesh, int(bs.levels[p]), 60, "cgs", precision="mixed", mixed_inner_cycles=4) as mg:
                s1 = torch.zeros_like(bs.view(rhs, p))
                r1 = torch.zeros_like(s1)
                try:
                    rep = mg.solve_vcycle(s1, r1, bs.view(rhs, p).contiguous(), 2, 1e-10, 1.0)
                except pmg.PmgError:
                    continue
            if not rep.converged:
                continue
            checked += 1
            assert ratio[p] < 1e-10, (p, ratio[p])
            assert abs(rep.cycles - cycles[p]) <= 1, (p, rep.cycles, cycles[p])
            assert rel(from_dev(bs.view(sol, p)), from_dev(s1)) < 1e-7, p
        assert checked >= 18
