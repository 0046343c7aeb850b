"""The oracle's multi-rank restatement (px x py x pz ranks simulated in one process) against
its one-rank solve.

With a red-black smoother whose colours follow the global cell parity (the rank-parity offset
of src/rbgs_poisson_matrix.f90:230-232), halo exchanges before every colour and every
mv_mul, and coarse meshes whose ghost widths come from the neighbours, the reference's CGS
V-cycle on several ranks performs exactly the one-rank arithmetic on every cell; only the
order of the dot products' sums differs.  So the multi-rank solution and residual must equal
the one-rank ones bit for bit (RBGS coarsest solver), the residual history agree to 1e-12
and the coarsest-solver iteration counts match.  Odd local sizes (offset 1 on odd ranks)
are included, and so is the reference's error for a split axis that cannot halve.
"""
import numpy as np
import pytest

from oracle import oracle as O
from peps_mg_gb300 import geometry as G
from peps_mg_gb300 import problems


def random_rhs(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    rhs = G.field(*n)
    rhs[1:-1, 1:-1, 1:-1] = rng.uniform(-1.0, 1.0, size=n)
    return np.asfortranarray(rhs)


def solve_both(mesh, rhs, procs, nl, coarse=0):
    n = tuple(len(m[0]) - 2 for m in mesh)
    one = O.OracleMG(mesh, nl, 60, 0, 0, coarse)
    s1, r1 = O.field(*n), O.field(*n)
    c1, h1, ci1 = one.solve(s1, r1, rhs, 2, 1e-10, 1.0)
    one.close()
    dd = O.OracleDD(mesh, procs, nl, 60, coarse)
    s2, r2 = O.field(*n), O.field(*n)
    c2, h2, ci2 = dd.solve(s2, r2, rhs, 2, 1e-10, 1.0)
    return (s1, r1, c1, h1, ci1), (s2, r2, c2, h2, ci2), dd


CASES = [
    ("blobs32", (2, 1, 1), 3), ("blobs32", (1, 2, 1), 3), ("blobs32", (1, 1, 2), 3),
    ("blobs32", (2, 2, 2), 3), ("blobs32", (4, 1, 1), 3), ("odd24", (2, 1, 1), 2), ("odd24", (2, 2, 2), 2),
    ("stretched", (2, 2, 2), 2), ("stretched", (1, 1, 2), 3),
]


@pytest.mark.parametrize("case,procs,nl", CASES)
def test_multi_rank_equals_one_rank(case, procs, nl):
    if case == "blobs32":
        mesh, rhs = problems.gaussian_blobs(32)
        rhs = np.asfortranarray(rhs)
    elif case == "odd24":
        ax = G.uniform_axis(24, 0.0, 1.0)
        mesh, rhs = [ax, ax, ax], random_rhs((24, 24, 24), 5)
    else:
        mesh = [G.stretched_axis(40, 0.0, 1.0, 1.1), G.uniform_axis(24, 0.0, 2.0), G.tanh_axis(32, 0.0, 1.0, 1.3)]
        rhs = random_rhs((40, 24, 32), 6)
    (s1, r1, c1, h1, ci1), (s2, r2, c2, h2, ci2), dd = solve_both(mesh, rhs, procs, nl)
    assert c1 == c2
    assert np.array_equal(s1, s2)
    assert np.array_equal(r1, r2)
    assert np.abs(h1[:, 2] - h2[:, 2]).max() <= 1e-12 * np.abs(h1[:, 2]).max() + 1e-300
    assert np.array_equal(ci1, ci2)
    if case == "odd24":
        # the coarsest level has 3 cells along x per rank: odd ranks start their colours
        # one cell later
        assert dd.level_dims(nl)[0] == 3
        assert [dd.offset((cx, 0, 0), nl) for cx in range(procs[0])] == [0, 1]


def test_multi_rank_cg_coarse_solver():
    """With the CG coarsest solver the iterates depend on the dot products, whose sums the
    ranks split differently: the solutions agree to rounding."""
    mesh, rhs = problems.gaussian_blobs(32)
    (s1, _, c1, _, _), (s2, _, c2, _, _), _ = solve_both(mesh, np.asfortranarray(rhs), (2, 2, 1), 3, coarse=1)
    assert c1 == c2
    assert np.abs(s1 - s2).max() <= 1e-12 * np.abs(s1).max()


def test_split_axis_that_cannot_halve_is_rejected():
    # 24 cells on 2 ranks: 12, 6, 3 -- a third level would halve 3 (src/multigrid.f90:226-246)
    ax = G.uniform_axis(24, 0.0, 1.0)
    with pytest.raises(ValueError):
        O.OracleDD([ax, ax, ax], (2, 1, 1), 3, 10)
    # sizes not divisible by the rank count
    with pytest.raises(ValueError):
        O.OracleDD([ax, ax, ax], (5, 1, 1), 2, 10)


@pytest.mark.parametrize("procs", [(2, 1, 1), (2, 2, 2), (1, 3, 1)])
def test_library_partition_matches_the_oracle(procs):
    """pmg_dd_partition (host only): each rank's level sizes and colour offsets are the
    oracle's, and its meshes are the global hierarchy's meshes restricted to its cells and
    ghost cells."""
    import peps_mg_gb300 as pmg
    mesh = [G.stretched_axis(24, 0.0, 1.0, 1.1), G.uniform_axis(24, 0.0, 2.0), G.tanh_axis(24, 0.0, 1.0, 1.3)]
    nl = 2
    dd = O.OracleDD(mesh, procs, nl, 1)
    glob = O.OracleMG(mesh, nl, 1, 0)
    for cz in range(procs[2]):
        for cy in range(procs[1]):
            for cx in range(procs[0]):
                co = (cx, cy, cz)
                for lev in range(nl + 1):
                    dims, m, off = pmg.dd_partition(mesh, procs, co, lev, nl)
                    assert dims == dd.level_dims(lev)
                    assert off == dd.offset(co, lev)
                    for a in range(3):
                        o = co[a] * dims[a]
                        gdm, gdg, _ = glob.level_mesh(lev, a)
                        assert np.array_equal(m[a][0], gdm[o:o + dims[a] + 2])
                        assert np.array_equal(m[a][1], gdg[o:o + dims[a] + 2])
    with pytest.raises(pmg.PmgError):
        pmg.dd_partition(mesh, (2, 1, 1), (0, 0, 0), 0, 4)     # 24/2 = 12, 6, 3: cannot halve again
