"""Device-side hierarchy set-up: the coarse meshes, coefficient tables and transfer weights
that pmg_create builds on the GPU (one launch) equal the host computation of the same
expressions bit for bit (src/multigrid.f90:419-495, src/matrix.f90:67-92).

PEPS_MG_HOST_SETUP=1 makes a context compute the coarse meshes on the host and check the
device-built tables against host-built ones inside pmg_create (a mismatch fails the
create); without it the meshes come from the device too, and they must equal the host's
and the oracle's.  A batch (whose problems' hierarchies come from one device arena) is
created and destroyed twice in a row.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import peps_mg_gb300 as pmg  # noqa: E402
from oracle import oracle as O  # noqa: E402
from peps_mg_gb300 import geometry as G  # noqa: E402
from peps_mg_gb300 import problems  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()


CASES = [
    ("cgs", 0, (0, 0, 0), [G.stretched_axis(48, 0.0, 1.0, 1.1), G.uniform_axis(40, -1.0, 2.0),
                           G.tanh_axis(36, 0.0, 1.5, 1.3)], 4),
    ("cga", 2, (0, 0, 0), [G.uniform_axis(64, 0.0, 1.0), G.tanh_axis(32, 0.0, 1.0, 1.5),
                           G.stretched_axis(32, 0.0, 2.0, 0.95)], 5),
    ("cgpsa", 0, (1, 2, 3), [G.uniform_axis(16, 0.0, 1.0), G.uniform_axis(32, 0.0, 1.0),
                             G.uniform_axis(64, 0.0, 1.0)], 6),
]


def levels(mg, nl):
    return [[mg.level_mesh(l, a) for a in range(3)] for l in range(nl + 1)]


@pytest.mark.parametrize("method,cga,cg3,mesh,nl", CASES)
def test_device_setup_equals_host(method, cga, cg3, mesh, nl):
    os.environ["PEPS_MG_HOST_SETUP"] = "1"
    try:
        # host meshes; the create itself checks the device tables against host tables
        with pmg.Multigrid(mesh, nl, 10, method, cga, cg3) as mg:
            host = levels(mg, nl)
    finally:
        del os.environ["PEPS_MG_HOST_SETUP"]
    n = tuple(len(m[0]) - 2 for m in mesh)
    rng = np.random.Generator(np.random.PCG64(3))
    rhs = G.field(*n)
    rhs[1:-1, 1:-1, 1:-1] = rng.uniform(-1.0, 1.0, size=n)
    with pmg.Multigrid(mesh, nl, 10, method, cga, cg3) as mg:
        dev = levels(mg, nl)
        b = torch.from_numpy(np.ascontiguousarray(rhs.T)).cuda()
        sol = torch.zeros_like(b)
        rep = mg.solve_vcycle(sol, torch.zeros_like(b), b, 2, 1e-10, 1.0)
        torch.cuda.synchronize()
    for l in range(nl + 1):
        for a in range(3):
            for q in range(3):
                assert np.array_equal(host[l][a][q], dev[l][a][q]), (l, a, q)
    # and the oracle's one-rank hierarchy and solve
    omg = O.OracleMG(mesh, nl, 10, {"cgs": 0, "cga": 1, "cgpsa": 2}[method], cga)
    for l in range(nl + 1):
        for a in range(3):
            om = omg.level_mesh(l, a)
            assert np.array_equal(om[0], dev[l][a][0]) and np.array_equal(om[1], dev[l][a][1]), (l, a)
    osol, orsd = O.field(*n), O.field(*n)
    ocyc, _, _ = omg.solve(osol, orsd, np.asfortranarray(rhs), 2, 1e-10, 1.0)
    omg.close()
    assert rep.cycles == ocyc
    assert np.array_equal(np.asfortranarray(sol.cpu().numpy().T), osol)


def test_batch_arena_create_destroy_twice():
    dims = problems.batch_dims(16)
    res = []
    for _ in range(2):
        with pmg.BatchSolver(dims, mixed_inner_cycles=4) as bs:
            rhs = bs.field()
            for p, vals in enumerate(problems.batch_rhs(dims)):
                bs.view(rhs, p)[1:-1, 1:-1, 1:-1] = torch.from_numpy(vals).cuda()
            sol = bs.field()
            cycles, ratio, _ = bs.solve(sol, rhs, 2, 1e-10, 1.0, max_cycles=50)
            torch.cuda.synchronize()
            assert np.all(ratio < 1e-10)
            res.append(sol.cpu())
    assert torch.equal(res[0], res[1])
