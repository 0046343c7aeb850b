"""Seeded random configurations against the oracle: sizes from 8 to 96 per axis (odd counts
that stop coarsening included), uniform, geometrically stretched and tanh meshes, CGS / CGA /
CGPSA with random levels, RBGS or CG coarsest solver, omega 1 or 1.2, zero, Dirichlet-face
or interior initial guesses, host or device arrays.

* FP64 with the RBGS coarsest solver: solution bit for bit, the same cycle count.
* FP64 with CG: the multi-CTA CG sums its dots in another order than the oracle, so the
  solution within 1e-10 of max |u| and the cycle count within one.
* Mixed: converged, and the oracle's own FP64 residual of the returned solution reaches the
  tolerance (ratio to the initial residual below 2e-10: the solver's FMA-form residual and
  the oracle's differ by rounding); the solution within 1e-6 of the oracle's (two solves that
  each reach a 1e-10 ratio differ by up to the condition number times that).
Cases whose oracle needs the whole cycle budget are skipped (no converged reference)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import peps_mg_gb300 as pmg  # noqa: E402
from oracle import oracle as O  # noqa: E402
from peps_mg_gb300 import geometry as G  # noqa: E402
from tests.helpers import from_dev, rel, to_dev  # noqa: E402

MAX_CYCLES = 60


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()


def draw(seed):
    rng = np.random.default_rng(seed)
    n = [int(rng.choice([8, 12, 16, 20, 24, 32, 40, 48, 64, 72, 96])) for _ in range(3)]
    axes = []
    for d in range(3):
        kind = int(rng.integers(3))
        axes.append(G.uniform_axis(n[d], 0.0, 1.0) if kind == 0 else
                    G.stretched_axis(n[d], 0.0, 1.0, float(rng.uniform(0.95, 1.05))) if kind == 1 else
                    G.tanh_axis(n[d], 0.0, 1.0, float(rng.uniform(0.5, 1.5))))
    method = str(rng.choice(["cgs", "cga", "cgpsa"]))
    nl = int(rng.integers(2, 6))
    cga = int(rng.integers(1, nl + 1)) if method == "cga" else 0
    cg3 = tuple(int(v) for v in rng.integers(1, nl + 1, size=3)) if method == "cgpsa" else (0, 0, 0)
    prec = str(rng.choice(["fp64", "mixed"]))
    coarse = str(rng.choice(["rbgs", "cg"]))
    host = bool(rng.integers(2))
    x0kind = int(rng.integers(3))
    omega = float(rng.choice([1.0, 1.2]))
    rhs = G.field(*n)
    rhs[1:-1, 1:-1, 1:-1] = rng.uniform(-1, 1, size=n)
    x0 = G.field(*n)
    if x0kind == 1:
        x0[:, :, 0] = 0.3
    elif x0kind == 2:
        x0[1:-1, 1:-1, 1:-1] = rng.uniform(-0.1, 0.1, size=n)
    return n, axes, method, nl, cga, cg3, prec, coarse, host, x0, omega, rhs


@pytest.mark.parametrize("seed", range(40))
def test_random_configuration(seed):
    n, axes, method, nl, cga, cg3, prec, coarse, host, x0, omega, rhs = draw(1000 + seed)
    try:
        mg = pmg.Multigrid(axes, nl, MAX_CYCLES, method, cga, cg3, coarse_solver=coarse, precision=prec,
                           mixed_inner_cycles=4 if prec == "mixed" else 0)
    except pmg.PmgError:
        pytest.skip("not a valid hierarchy for these sizes")
    with mg:
        omg = O.OracleMG(axes, nl, MAX_CYCLES, {"cgs": 0, "cga": 1, "cgpsa": 2}[method], cga,
                         {"rbgs": 0, "cg": 1}[coarse])
        osol, orsd = np.asfortranarray(x0.copy()), O.field(*n)
        ocyc, _, _ = omg.solve(osol, orsd, np.asfortranarray(rhs), 2, 1e-10, omega)
        omg.close()
        if ocyc >= MAX_CYCLES:
            pytest.skip("the oracle does not converge within the cycle budget")
        if host:
            s = np.ascontiguousarray(np.asfortranarray(x0).T).copy()
            r = np.zeros_like(s)
            rep = mg.solve_vcycle(s, r, np.ascontiguousarray(np.asfortranarray(rhs).T), 2, 1e-10, omega)
            sol = np.asfortranarray(s.T)
        else:
            sd = to_dev(x0)
            rep = mg.solve_vcycle(sd, torch.zeros_like(sd), to_dev(rhs), 2, 1e-10, omega)
            torch.cuda.synchronize()
            sol = from_dev(sd)
    if prec == "fp64" and coarse == "rbgs":
        assert rep.cycles == ocyc
        assert np.array_equal(sol, osol)
    elif prec == "fp64":
        assert abs(rep.cycles - ocyc) <= 1
        assert rel(sol, osol) < 1e-10
    else:
        assert rep.converged and rep.final_ratio < 1e-10
        coeff = O.matrix_create(axes)
        r0 = O.residual(coeff, np.asfortranarray(x0), np.asfortranarray(rhs))
        r = O.residual(coeff, np.asfortranarray(sol), np.asfortranarray(rhs))
        assert np.linalg.norm(r) < 2e-10 * np.linalg.norm(r0)
        assert rel(sol, osol) < 1e-6
