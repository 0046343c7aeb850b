"""Hand-written adjoint: against a direct solve of the transposed system (scipy, from the
oracle's coefficient matrix), and through torch.autograd against central finite
differences of L = 1/2 |u - u_t|^2 (interior) with respect to b and the six face values."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
sp = pytest.importorskip("scipy.sparse")
spla = pytest.importorskip("scipy.sparse.linalg")
pytestmark = pytest.mark.gpu

import peps_mg_gb300 as pmg  # noqa: E402
from oracle import oracle as O  # noqa: E402
from peps_mg_gb300.autograd import PoissonSolve  # noqa: E402
from tests.helpers import from_dev, rel, to_dev  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def assemble(mesh):
    """Interior operator A (CSR, Fortran cell order) and the per-face ghost couplings."""
    c = O.matrix_create(mesh)
    nx, ny, nz = c.shape[1:]
    N = nx * ny * nz
    idx = np.arange(N).reshape((nx, ny, nz), order="F")
    rows, cols, vals = [idx.ravel(order="F")], [idx.ravel(order="F")], [c[0].ravel(order="F")]
    shifts = [(-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)]
    face = []
    for q, (di, dj, dk) in enumerate(shifts, start=1):
        I, J, K = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
        I2, J2, K2 = I + di, J + dj, K + dk
        ok = (I2 >= 0) & (I2 < nx) & (J2 >= 0) & (J2 < ny) & (K2 >= 0) & (K2 < nz)
        rows.append(idx[ok]); cols.append(idx[I2[ok], J2[ok], K2[ok]]); vals.append(c[q][ok])
        f = np.zeros((nx, ny, nz))
        f[~ok] = c[q][~ok]
        face.append(f)
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(N, N))
    return A, face


@pytest.mark.parametrize("stretched,precision", [(False, "fp64"), (True, "fp64"), (True, "mixed")])
def test_adjoint_matches_transposed_solve(stretched, precision):
    rng = np.random.default_rng(3)
    n = (16, 12, 20)
    if stretched:
        mesh = [pmg.geometry.mesh_from_widths(rng.uniform(0.6, 1.4, m) / m) for m in n]
    else:
        mesh = [pmg.geometry.uniform_axis(m, 0.0, 1.0) for m in n]
    A, face = assemble(mesh)
    w = pmg.geometry.field(*n)
    w[1:-1, 1:-1, 1:-1] = rng.uniform(-1, 1, n)
    lam = spla.spsolve(A.T.tocsc(), w[1:-1, 1:-1, 1:-1].ravel(order="F")).reshape(n, order="F")
    with pmg.Multigrid(mesh, 2, 100, "cgs", precision=precision) as mg:
        dldb = torch.zeros((n[2] + 2, n[1] + 2, n[0] + 2), dtype=torch.float64, device="cuda")
        rep, dldg = mg.adjoint(to_dev(w), dldb, 2, 1e-13, 1.0)
    got = from_dev(dldb)
    assert rep.converged
    assert rel(got[1:-1, 1:-1, 1:-1], lam) < 1e-9
    assert np.all(got[0] == 0) and np.all(got[:, :, -1] == 0)
    ref_g = np.array([-(f * lam).sum() for f in face])
    # face order of the coupling list: x-, x+, y-, y+, z-, z+
    assert np.allclose(dldg, ref_g, rtol=1e-9, atol=1e-12 * np.abs(ref_g).max())


def sine_target(n, seed=5, modes=16):
    rng = np.random.Generator(np.random.PCG64(seed))
    xc = (np.arange(n) + 0.5) / n
    u = np.zeros((n, n, n))
    pqr = rng.integers(1, 5, size=(modes, 3))
    amp = rng.uniform(-1, 1, modes)
    for (p, q, r), a in zip(pqr, amp):
        u += a * np.sin(p * np.pi * xc)[:, None, None] * np.sin(q * np.pi * xc)[None, :, None] * \
            np.sin(r * np.pi * xc)[None, None, :]
    return u


def test_autograd_against_finite_differences():
    n = 16
    ax = pmg.geometry.uniform_axis(n, 0.0, 1.0)
    mesh = [ax, ax, ax]
    rng = np.random.default_rng(9)
    ut = torch.from_numpy(np.ascontiguousarray(sine_target(n).T)).cuda()
    b0 = torch.zeros((n + 2,) * 3, dtype=torch.float64, device="cuda")
    b0[1:-1, 1:-1, 1:-1] = torch.from_numpy(rng.uniform(-1, 1, (n, n, n))).cuda()
    g0 = torch.tensor(rng.uniform(-0.5, 0.5, 6), dtype=torch.float64)
    mg = pmg.Multigrid(mesh, 3, 200, "cgs")
    args = (mg, 2, 1e-14, 1.0)

    def loss(b, g):
        u = PoissonSolve.apply(b, g, *args)
        return 0.5 * ((u[1:-1, 1:-1, 1:-1] - ut) ** 2).sum()

    def central_difference(bp, gp, bm, gm, h):
        # (L(+) - L(-)) / 2h, summed as 1/2 (u+ - u-)(u+ + u- - 2 u_t) so that the two
        # losses' rounding does not cancel
        up = PoissonSolve.apply(bp, gp, *args)[1:-1, 1:-1, 1:-1]
        um = PoissonSolve.apply(bm, gm, *args)[1:-1, 1:-1, 1:-1]
        return 0.5 * float(((up - um) * (up + um - 2 * ut)).sum()) / (2 * h)

    b = b0.clone().requires_grad_(True)
    g = g0.clone().requires_grad_(True)
    L = loss(b, g)
    L.backward()
    gb, gg = b.grad.detach().cpu().numpy(), g.grad.detach().numpy()
    with torch.no_grad():
        # h = 1e-2 is exact for this quadratic loss up to the solves' rounding; at h = 1e-6
        # the signal 2 h dL/db(cell) is ~1e-10 against ~1e-14 of FP64 rounding in u+ - u-
        for h, rtol in ((1e-2, 1e-7), (1e-6, 2e-3)):
            for (k, j, i) in [(1, 1, 1), (8, 8, 8), (3, 12, 15), (16, 2, 9), (10, 16, 4)]:
                bp, bm = b0.clone(), b0.clone()
                bp[k, j, i] += h
                bm[k, j, i] -= h
                fd = central_difference(bp, g0, bm, g0, h)
                assert abs(fd - gb[k, j, i]) <= rtol * max(abs(gb[k, j, i]), 1e-3 * np.abs(gb).max()), (h, k, j, i)
            for f in range(6):
                gp, gm = g0.clone(), g0.clone()
                gp[f] += h
                gm[f] -= h
                fd = central_difference(b0, gp, b0, gm, h)
                assert abs(fd - gg[f]) <= rtol * max(abs(gg[f]), 1e-3 * np.abs(gg).max()), (h, f)
    mg.destroy()


def test_adjoint_256_finite_differences_and_oracle():
    """The adjoint workload at full size: 256^3 uniform grid, b ~ U[-1,1] (PCG64(6)), zero
    faces, L = 1/2 |u - u_t|^2 with u_t a 16-mode sine sum.  Gradients from autograd are
    checked against central differences (h = 1e-6, FP64 solves) along a smooth direction
    in b and along each face value, and dL/db against the oracle's FP64 V-cycle applied
    to the adjoint right-hand side."""
    n = 256
    ax = pmg.geometry.uniform_axis(n, 0.0, 1.0)
    mesh = [ax, ax, ax]
    rng = np.random.Generator(np.random.PCG64(6))
    ut = torch.from_numpy(np.ascontiguousarray(sine_target(n).T)).cuda()
    b0 = torch.zeros((n + 2,) * 3, dtype=torch.float64, device="cuda")
    b0[1:-1, 1:-1, 1:-1] = torch.from_numpy(rng.uniform(-1, 1, (n, n, n))).cuda()
    g0 = torch.zeros(6, dtype=torch.float64, device="cuda")
    mg = pmg.Multigrid(mesh, 7, 100, "cgs")
    args = (mg, 2, 1e-12, 1.0)

    def loss(b, g):
        u = PoissonSolve.apply(b, g, *args)
        return 0.5 * ((u[1:-1, 1:-1, 1:-1] - ut) ** 2).sum()

    b = b0.clone().requires_grad_(True)
    g = g0.clone().requires_grad_(True)
    loss(b, g).backward()
    gb, gg = b.grad.detach(), g.grad.detach()
    h = 1e-6

    def central_difference(bp, gp, bm, gm):
        up = PoissonSolve.apply(bp, gp, *args)[1:-1, 1:-1, 1:-1]
        um = PoissonSolve.apply(bm, gm, *args)[1:-1, 1:-1, 1:-1]
        return 0.5 * float(((up - um) * (up + um - 2 * ut)).sum()) / (2 * h)

    with torch.no_grad():
        v = torch.zeros_like(b0)
        v[1:-1, 1:-1, 1:-1] = torch.from_numpy(np.ascontiguousarray(sine_target(n, seed=8, modes=4).T)).cuda()
        fd = central_difference(b0 + h * v, g0, b0 - h * v, g0)
        an = float((gb * v).sum())
        assert abs(fd - an) <= 1e-6 * abs(an), (fd, an)
        for f in range(6):
            e = torch.zeros(6, dtype=torch.float64, device="cuda")
            e[f] = h
            fd = central_difference(b0, g0 + e, b0, g0 - e)
            assert abs(fd - float(gg[f])) <= 1e-6 * float(gg.abs().max()), (f, fd, float(gg[f]))
        # the oracle on the adjoint right-hand side: A^T lam = u - u_t, with A^T = A here
        u = PoissonSolve.apply(b0, g0, *args)
        w = O.field(n, n, n)
        w[1:-1, 1:-1, 1:-1] = from_dev(u)[1:-1, 1:-1, 1:-1] - sine_target(n)
    mg.destroy()
    omg = O.OracleMG(mesh, 7, 100, 0, omp=True)
    lam, rr = O.field(n, n, n), O.field(n, n, n)
    omg.solve(lam, rr, w, 2, 1e-12, 1.0)
    omg.close()
    assert rel(from_dev(gb)[1:-1, 1:-1, 1:-1], lam[1:-1, 1:-1, 1:-1]) < 1e-9
