"""The FP64 performance mode (PMG_FP64_FAST) against the oracle.

It runs the plain path's V-cycle with FMA chains, a stored omega/c0 per cell and per-axis
normalised transfer weights, so it is not bit-identical to the reference; it must
converge like the plain path (the same cycle count, or one more) to the oracle's solution
within rounding: max-abs difference below 1e-9 of max |u| (the solutions of two solves that
each reach a 1e-10 relative residual), with the returned residual the FP64 b - A x of the
returned solution within a few ulps of |c0| |x|.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import peps_mg_gb300 as pmg  # noqa: E402
from oracle import oracle as O  # noqa: E402
from tests.helpers import from_dev, rel, sine_problem, tanh_z_problem, to_dev  # noqa: E402

SOL_TOL = 1e-9
EPS = np.finfo(np.float64).eps


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()


def F(a):
    return np.asfortranarray(np.array(a, dtype=np.float64))


def check_against_oracle(mesh, rhs, levels, method="cgs", cga=0, cgpsa=(0, 0, 0), coarse="rbgs", omega=1.0,
                         maxit=2, tol=1e-10, omp=False):
    nx, ny, nz = (len(m[0]) - 2 for m in mesh)
    omg = O.OracleMG(mesh, levels, 60, {"cgs": 0, "cga": 1, "cgpsa": 2}[method], cga,
                     {"rbgs": 0, "cg": 1}[coarse], omp=omp)
    osol, orsd = O.field(nx, ny, nz), O.field(nx, ny, nz)
    ocyc, _, _ = omg.solve(osol, orsd, F(rhs), maxit, tol, omega)
    omg.close()
    with pmg.Multigrid(mesh, levels, 60, method, cga, cgpsa, coarse_solver=coarse, precision="fp64_fast") as mg:
        b = to_dev(rhs)
        sol = torch.zeros_like(b)
        rsd = torch.zeros_like(b)
        rep = mg.solve_vcycle(sol, rsd, b, maxit, tol, omega)
        r_check = torch.zeros_like(b)
        mg.residual(0, r_check, sol, b)           # the bitwise residual of the returned solution
        torch.cuda.synchronize()
        r_diff = (r_check - rsd).abs().max().item()
    s = from_dev(sol)
    assert rep.converged and rep.final_ratio < tol
    assert ocyc <= rep.cycles <= ocyc + 1, (rep.cycles, ocyc)
    err = rel(s[1:-1, 1:-1, 1:-1], osol[1:-1, 1:-1, 1:-1])
    assert err < SOL_TOL, err
    # |c0| <= sum over the axes of max(1/(dm dg) + 1/(dm dg(+1))) (src/matrix.f90:75-82)
    c0 = sum((1.0 / (m[0][1:-1] * m[1][1:-1]) + 1.0 / (m[0][1:-1] * m[1][2:])).max() for m in mesh)
    assert r_diff <= 16 * EPS * c0 * np.abs(s).max(), r_diff
    # the ghost layers (zero Dirichlet values) are untouched
    for g in (s[0], s[-1], s[:, 0], s[:, -1], s[:, :, 0], s[:, :, -1]):
        assert not g.any()
    return rep, s


@pytest.mark.parametrize("coarse", ["rbgs", "cg"])
def test_fast_sine_64(coarse):
    mesh, rhs, _ = sine_problem(64)
    check_against_oracle(mesh, rhs, 4, coarse=coarse)


def test_fast_omega_sor():
    mesh, rhs, _ = sine_problem(32)
    check_against_oracle(mesh, rhs, 3, omega=1.3)


def test_fast_uneven_strides():
    """Axes that stop coarsening (stride-1 transfers) on a stretched mesh."""
    ax = pmg.geometry.stretched_axis(48, 0.0, 1.0, 1.05)
    ay = pmg.geometry.uniform_axis(40, 0.0, 2.0)
    az = pmg.geometry.tanh_axis(36, 0.0, 1.5, 1.3)
    rng = np.random.Generator(np.random.PCG64(21))
    rhs = pmg.geometry.field(48, 40, 36)
    rhs[1:-1, 1:-1, 1:-1] = rng.uniform(-1.0, 1.0, size=(48, 40, 36))
    check_against_oracle([ax, ay, az], rhs, 4)


@pytest.mark.parametrize("method,cga,cg3", [("cgs", 0, (0, 0, 0)), ("cga", 4, (0, 0, 0)), ("cgpsa", 0, (4, 5, 6))])
def test_fast_tanh_256(method, cga, cg3):
    """The 256^3 tanh-z workload with each aggregation mapping.  (The mappings move
    different levels into the single-CTA tail, which keeps the bitwise arithmetic, so in
    this mode they agree with the oracle, not bit for bit with each other.)"""
    mesh, rhs = tanh_z_problem(256)
    check_against_oracle(mesh, rhs, 7, method=method, cga=cga, cgpsa=cg3, omp=True)


def test_fast_nonzero_dirichlet_faces():
    mesh, rhs, _ = sine_problem(32)
    rhs = rhs.copy()
    rhs[0, :, :] = 0.0
    sol0 = pmg.geometry.field(32, 32, 32)
    sol0[:, :, -1] = 0.5          # a Dirichlet face value in the ghost layer
    omg = O.OracleMG(mesh, 3, 60, 0)
    osol, orsd = F(sol0).copy(order="F"), O.field(32, 32, 32)
    omg.solve(osol, orsd, F(rhs), 2, 1e-10, 1.0)
    omg.close()
    with pmg.Multigrid(mesh, 3, 60, "cgs", precision="fp64_fast") as mg:
        sol = to_dev(sol0)
        b = to_dev(rhs)
        rep = mg.solve_vcycle(sol, torch.zeros_like(b), b, 2, 1e-10, 1.0)
        torch.cuda.synchronize()
    s = from_dev(sol)
    assert rep.converged
    assert rel(s, osol) < SOL_TOL
    assert np.array_equal(s[:, :, -1], sol0[:, :, -1])
