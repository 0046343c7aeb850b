"""Mixed precision (FP32 V-cycles inside FP64 defect correction) against the FP64 oracle.

Both solvers stop at a relative residual of 1e-10 (FP64 norms), so their solutions
agree to about that level times the conditioning of the discrete problem; the test
bound on the solution is 1e-8 relative to max|u|, and the final FP64 residual ratio
must be below the tolerance.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import peps_mg_gb300 as pmg  # noqa: E402
from oracle import oracle as O  # noqa: E402
from peps_mg_gb300 import problems  # noqa: E402
from tests.helpers import from_dev, rel, to_dev  # noqa: E402

SOL_TOL = 1e-8


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def oracle_solution(mesh, rhs, n_levels, method=0, cga=0, cs=0, maxit=2, omega=1.0, tol=1e-10):
    n = tuple(len(m[0]) - 2 for m in mesh)
    omg = O.OracleMG(mesh, n_levels, 100, method, cga, cs)
    sol, rsd = O.field(*n), O.field(*n)
    ncyc, hist, _ = omg.solve(sol, rsd, np.asfortranarray(rhs), maxit, tol, omega)
    return sol, ncyc


def mixed_solve(mesh, rhs, n_levels, inner=2, **kw):
    with pmg.Multigrid(mesh, n_levels, 100, precision="mixed", mixed_inner_cycles=inner, **kw) as mg:
        sol = torch.zeros(tuple(reversed(rhs.shape)), dtype=torch.float64, device="cuda")
        rsd = torch.zeros_like(sol)
        rep = mg.solve_vcycle(sol, rsd, to_dev(rhs), 2, 1e-10, 1.0)
    return from_dev(sol), from_dev(rsd), rep


@pytest.mark.parametrize("inner", [1, 2, 3])
def test_mixed_sine_64(inner):
    mesh, rhs, u = problems.sine(64)
    ref, _ = oracle_solution(mesh, rhs, 4)
    sol, rsd, rep = mixed_solve(mesh, rhs, 4, inner=inner)
    assert rep.converged and rep.final_ratio < 1e-10
    # every correction runs `inner` FP32 cycles, except that the last may stop early once
    # the residual it leaves is below the tolerance
    assert inner * (rep.cycles - 1) < rep.inner_cycles <= inner * rep.cycles
    assert rel(sol, ref) < SOL_TOL
    # the returned residual is the FP64 residual of the returned solution; at a 1e-10
    # relative residual both evaluations carry rounding noise of order 1e-13 |b|, so the
    # comparison is relative to the right-hand side
    c = O.matrix_create(mesh)
    r = O.residual(c, np.asfortranarray(sol), np.asfortranarray(rhs))
    assert np.max(np.abs(rsd - r)) < 1e-12 * np.max(np.abs(rhs))
    assert np.sqrt(O.vv_dot(r, r)) / rep.res0 < 1.1e-10


def test_mixed_gaussian_blobs_96():
    mesh, rhs = problems.gaussian_blobs(96)
    ref, _ = oracle_solution(mesh, rhs, 5)
    sol, _, rep = mixed_solve(mesh, rhs, 5)
    assert rep.converged
    assert rel(sol, ref) < SOL_TOL


@pytest.mark.parametrize("method,cga,cg3,cs", [("cga", 2, (0, 0, 0), "rbgs"), ("cgpsa", 0, (1, 2, 3), "rbgs"),
                                               ("cgs", 0, (0, 0, 0), "cg")])
def test_mixed_tanh_z(method, cga, cg3, cs):
    mesh, rhs = problems.tanh_z(64)
    ref, _ = oracle_solution(mesh, rhs, 5, cs=1 if cs == "cg" else 0)
    sol, _, rep = mixed_solve(mesh, rhs, 5, aggregation_method=method, cga_level=cga, cgpsa_level=cg3,
                              coarse_solver=cs)
    assert rep.converged
    assert rel(sol, ref) < SOL_TOL


def test_mixed_host_buffers():
    mesh, rhs, _ = problems.sine(32)
    with pmg.Multigrid(mesh, 3, 50, precision="mixed") as mg:
        hs, hr = pmg.geometry.field(32, 32, 32), pmg.geometry.field(32, 32, 32)
        rep = mg.solve_vcycle(hs, hr, np.asfortranarray(rhs), 2, 1e-10, 1.0)
        ds = torch.zeros((34,) * 3, dtype=torch.float64, device="cuda")
        dr = torch.zeros_like(ds)
        rep2 = mg.solve_vcycle(ds, dr, to_dev(rhs), 2, 1e-10, 1.0)
    assert rep.converged and np.array_equal(hs, from_dev(ds)) and np.array_equal(rep.history, rep2.history)


def test_mixed_faster_cycles_than_fp64_history():
    """The mixed solver reaches the tolerance in no more FP64 residual evaluations than
    the plain FP64 solver needs V-cycles (two FP32 cycles per correction)."""
    mesh, rhs, _ = problems.sine(64)
    _, ncyc = oracle_solution(mesh, rhs, 4)
    _, _, rep = mixed_solve(mesh, rhs, 4, inner=2)
    assert rep.cycles <= (ncyc + 1) // 2 + 1


@pytest.mark.parametrize("n3,levels", [((100, 36, 20), 2), ((72, 40, 24), 3), ((130, 68, 36), 2)])
def test_mixed_uneven_tiles(n3, levels):
    """Sizes that are not multiples of the fused smoother's 64 x 16 tile, odd sizes at the
    coarse levels, a stretched mesh and a non-zero Dirichlet face."""
    rng = np.random.default_rng(sum(n3))
    mesh = [pmg.geometry.mesh_from_widths(rng.uniform(0.7, 1.3, n) / n) for n in n3]
    nx, ny, nz = n3
    rhs = pmg.geometry.field(nx, ny, nz)
    rhs[1:-1, 1:-1, 1:-1] = rng.uniform(-1, 1, (nx, ny, nz))
    sol0 = pmg.geometry.field(nx, ny, nz)
    sol0[:, 0, :] = 0.5
    omg = O.OracleMG(mesh, levels, 200, 0, 0, 0)
    ref, rr = np.asfortranarray(sol0.copy()), O.field(nx, ny, nz)
    omg.solve(ref, rr, np.asfortranarray(rhs), 2, 1e-10, 1.0)
    with pmg.Multigrid(mesh, levels, 200, precision="mixed") as mg:
        sol = to_dev(sol0)
        rsd = torch.zeros_like(sol)
        rep = mg.solve_vcycle(sol, rsd, to_dev(rhs), 2, 1e-10, 1.0)
    assert rep.converged
    s = from_dev(sol)
    assert rel(s, ref) < SOL_TOL
    assert np.array_equal(s[:, 0, :], sol0[:, 0, :])


def test_conversion_selftest():
    """The integer-pipe double->float (round to nearest even) and float->double
    conversions of the outer kernels agree with the hardware conversions."""
    lib = pmg.load()
    rng = np.random.default_rng(7)
    n = 1 << 20
    a = rng.standard_normal(n) * np.exp2(rng.integers(-140, 140, n))
    # values exactly halfway between floats, and near the overflow/underflow limits
    f = rng.standard_normal(n // 8).astype(np.float32).astype(np.float64)
    a[: n // 8] = f + np.ldexp(np.abs(f), -24) * np.sign(f)
    a[-8:] = [0.0, -0.0, 3.4028235677973366e38, 3.4028235e38 * 1.0000001, 1.1754943508222875e-38,
              1e-39, np.inf, np.nan]
    d64 = torch.from_numpy(a).cuda()
    f32 = torch.from_numpy((rng.standard_normal(n) * np.exp2(rng.integers(-140, 120, n))).astype(np.float32)).cuda()
    o32 = torch.empty(n, dtype=torch.float32, device="cuda")
    o64 = torch.empty(n, dtype=torch.float64, device="cuda")
    assert lib.pmg_selftest_convert(d64.data_ptr(), o32.data_ptr(), f32.data_ptr(), o64.data_ptr(), n) == 0
    ref32 = d64.float()
    same = (o32 == ref32) | (torch.isnan(o32) & torch.isnan(ref32))
    assert bool(same.all())
    assert torch.equal(torch.signbit(o32[~torch.isnan(o32)]), torch.signbit(ref32[~torch.isnan(ref32)]))
    assert torch.equal(o64, f32.double())


def test_residual_update_matches_recomputed(tmp_path):
    """After a correction the residual is updated as r -= A e (compensated FP32 products)
    instead of recomputed as b - A x in FP64.  On a stretched mesh with a non-zero
    Dirichlet face both variants take the same corrections; the updated residual norms
    agree with the recomputed ones far below the tolerance, the solve still ends on a
    recomputed residual, and the solutions agree to the solver's accuracy."""
    import os
    import subprocess
    import sys
    code = r'''
import sys, numpy as np, torch, peps_mg_gb300 as pmg
from tests.helpers import to_dev, from_dev
n = (80, 72, 64)
rng = np.random.default_rng(11)
mesh = [pmg.geometry.mesh_from_widths(rng.uniform(0.7, 1.3, m) / m) for m in n]
rhs = pmg.geometry.field(*n); rhs[1:-1, 1:-1, 1:-1] = rng.uniform(-1, 1, n)
sol0 = pmg.geometry.field(*n); sol0[0, :, :] = 0.25
with pmg.Multigrid(mesh, 4, 50, "cgs", precision="mixed", mixed_inner_cycles=2) as mg:
    sol = to_dev(sol0)
    rsd = torch.zeros_like(sol)
    rep = mg.solve_vcycle(sol, rsd, to_dev(rhs), 2, 1e-10, 1.0)
np.savez(sys.argv[1], sol=from_dev(sol), rsd=from_dev(rsd), hist=rep.history, conv=rep.converged)
'''
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    res = {}
    for mode in ("update", "recompute"):
        env = dict(os.environ, PEPS_MG_OUTER=mode, PYTHONPATH=root)
        path = str(tmp_path / (mode + ".npz"))
        r = subprocess.run([sys.executable, "-c", code, path], cwd=root, env=env, capture_output=True, text=True,
                           timeout=300)
        assert r.returncode == 0, r.stderr[-2000:]
        res[mode] = np.load(path)
    u, c = res["update"], res["recompute"]
    assert bool(u["conv"]) and bool(c["conv"])
    hu, hc = u["hist"], c["hist"]
    m = min(len(hu), len(hc))
    assert m >= 2
    # ratio after each correction (column 2): identical corrections until the last one;
    # the updated residual's norm is summed in FP32 (it only decides when to recompute)
    np.testing.assert_allclose(hu[:m - 1, 2], hc[:m - 1, 2], rtol=1e-5, atol=1e-11)
    assert hu[-1, 2] < 1e-10
    scale = np.abs(c["sol"]).max()
    assert np.abs(u["sol"] - c["sol"]).max() / scale < 1e-9
    # the returned residual is recomputed b - A x in both
    mesh_rng = np.random.default_rng(11)
    n = (80, 72, 64)
    mesh = [pmg.geometry.mesh_from_widths(mesh_rng.uniform(0.7, 1.3, k) / k) for k in n]
    rhs = pmg.geometry.field(*n)
    rhs[1:-1, 1:-1, 1:-1] = mesh_rng.uniform(-1, 1, n)
    coeff = O.matrix_create(mesh)
    r = O.residual(coeff, np.asfortranarray(u["sol"]), np.asfortranarray(rhs))
    # FMA form against the reference's left-to-right form: rounding noise of order
    # eps |c0| |x| (the Dirichlet face makes |x| large here)
    noise = 8 * np.finfo(np.float64).eps * np.abs(coeff[0]).max() * np.abs(u["sol"]).max()
    assert np.max(np.abs(u["rsd"] - r)) < noise


def test_residual_update_stash_same_bits(tmp_path):
    """The residual update leaves x alone and keeps the corrections in two stash arrays; x
    gets them, one at a time in the order they were made, where it is needed (the FP64
    residual, the third correction in a row, the end of the solve).  The solution, the
    residual and every residual norm have the same bits as with each correction added at
    once (PEPS_MG_STASH=off).  One FP32 cycle per correction gives runs of updates longer
    than the stash; the Dirichlet face and stretched mesh give a non-zero x0 and
    corrections of every size."""
    import os
    import subprocess
    import sys
    code = r'''
import sys, numpy as np, torch, peps_mg_gb300 as pmg
from tests.helpers import to_dev, from_dev
n = (72, 64, 56)
rng = np.random.default_rng(5)
mesh = [pmg.geometry.mesh_from_widths(rng.uniform(0.7, 1.3, m) / m) for m in n]
rhs = pmg.geometry.field(*n); rhs[1:-1, 1:-1, 1:-1] = rng.uniform(-1, 1, n)
sol0 = pmg.geometry.field(*n); sol0[0, :, :] = 0.5
out = {}
for inner in (1, 2, 4):
    with pmg.Multigrid(mesh, 4, 50, "cgs", precision="mixed", mixed_inner_cycles=inner) as mg:
        sol = to_dev(sol0)
        rsd = torch.zeros_like(sol)
        rep = mg.solve_vcycle(sol, rsd, to_dev(rhs), 2, 1e-10, 1.0)
    out["sol%d" % inner] = from_dev(sol)
    out["rsd%d" % inner] = from_dev(rsd)
    out["hist%d" % inner] = rep.history
    out["n%d" % inner] = np.array([rep.cycles, rep.inner_cycles, rep.converged])
np.savez(sys.argv[1], **out)
'''
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    res = {}
    for mode in ("on", "off"):
        env = dict(os.environ, PEPS_MG_STASH=mode, PYTHONPATH=root)
        path = str(tmp_path / (mode + ".npz"))
        r = subprocess.run([sys.executable, "-c", code, path], cwd=root, env=env, capture_output=True, text=True,
                           timeout=300)
        assert r.returncode == 0, r.stderr[-2000:]
        res[mode] = np.load(path)
    a, b = res["on"], res["off"]
    for inner in (1, 2, 4):
        assert a["n%d" % inner][2] == 1
        assert np.array_equal(a["n%d" % inner], b["n%d" % inner])
        # one FP32 cycle per correction: more updates in a row than stash arrays
        if inner == 1:
            assert a["n1"][0] >= 4
        for key in ("sol", "rsd", "hist"):
            assert np.array_equal(a["%s%d" % (key, inner)].view(np.uint64), b["%s%d" % (key, inner)].view(np.uint64)), \
                (key, inner)


def test_mixed_pinned_host_buffers():
    """Pinned host buffers: the solution's copy back starts while the final residual is
    computed; the results equal those of device buffers."""
    mesh, rhs, _ = problems.sine(48)
    n = 48
    with pmg.Multigrid(mesh, 4, 50, precision="mixed") as mg:
        shape = (n + 2,) * 3
        h_rhs = torch.from_numpy(np.ascontiguousarray(np.asfortranarray(rhs).T)).pin_memory()
        h_sol = torch.zeros(shape, dtype=torch.float64).pin_memory()
        h_rsd = torch.zeros(shape, dtype=torch.float64).pin_memory()
        rep = mg.solve_vcycle(h_sol.numpy(), h_rsd.numpy(), h_rhs.numpy(), 2, 1e-10, 1.0)
        ds = torch.zeros(shape, dtype=torch.float64, device="cuda")
        dr = torch.zeros_like(ds)
        rep2 = mg.solve_vcycle(ds, dr, to_dev(rhs), 2, 1e-10, 1.0)
    assert rep.converged and np.array_equal(rep.history, rep2.history)
    assert torch.equal(h_sol, ds.cpu()) and torch.equal(h_rsd, dr.cpu())


def test_mixed_nan_rhs_reports_divergence():
    """A NaN in the right-hand side: the mixed solver (zero-guess first residual, residual
    update, FP64 recompute) reports divergence instead of looping or returning success."""
    mesh, rhs, _ = problems.sine(32)
    rhs[7, 9, 11] = np.nan
    with pmg.Multigrid(mesh, 3, 5, "cgs", precision="mixed") as mg:
        sol = torch.zeros((34,) * 3, dtype=torch.float64, device="cuda")
        with pytest.raises(pmg.PmgError) as e:
            mg.solve_vcycle(sol, torch.zeros_like(sol), to_dev(rhs), 1, 1e-10, 1.0)
        assert e.value.status == 3


def test_mixed_pageable_host_buffers_registered_or_not(monkeypatch):
    """Pageable host buffers are page-locked for the call (cudaHostRegister) and released
    after it; with PEPS_MG_NO_HOST_REGISTER=1 they are copied as pageable memory, and three
    buffers carved from one allocation (sharing pages, so not all can be registered) fall
    back to pageable copies.  All three give the device-buffer result bit for bit, and the
    arrays are not left page-locked."""
    mesh, rhs, _ = problems.sine(48)
    n = 48
    shape = (n + 2,) * 3
    size = (n + 2) ** 3
    with pmg.Multigrid(mesh, 4, 50, precision="mixed") as mg:
        ds = torch.zeros(shape, dtype=torch.float64, device="cuda")
        dr = torch.zeros_like(ds)
        rep_d = mg.solve_vcycle(ds, dr, to_dev(rhs), 2, 1e-10, 1.0)
        ref_s, ref_r = ds.cpu().numpy(), dr.cpu().numpy()
        b = np.ascontiguousarray(np.asfortranarray(rhs).T)
        for env in ("0", "1"):
            monkeypatch.setenv("PEPS_MG_NO_HOST_REGISTER", env)
            hs, hr = np.zeros(shape), np.zeros(shape)
            rep = mg.solve_vcycle(hs, hr, b, 2, 1e-10, 1.0)
            assert np.array_equal(rep.history, rep_d.history)
            assert np.array_equal(hs, ref_s) and np.array_equal(hr, ref_r)
            for a in (hs, hr, b):       # released: a new registration of the same range works
                assert int(torch.cuda.cudart().cudaHostRegister(a.ctypes.data, a.nbytes, 0)) == 0
                assert int(torch.cuda.cudart().cudaHostUnregister(a.ctypes.data)) == 0
        monkeypatch.setenv("PEPS_MG_NO_HOST_REGISTER", "0")
        one = np.zeros(3 * size + 7)
        hs, hr, hb = (one[1 + q * size:1 + (q + 1) * size].reshape(shape) for q in range(3))
        hb[...] = b
        rep = mg.solve_vcycle(hs, hr, hb, 2, 1e-10, 1.0)
        assert np.array_equal(rep.history, rep_d.history)
        assert np.array_equal(hs, ref_s) and np.array_equal(hr, ref_r)


@pytest.mark.parametrize("start", ["zero", "ghost_face", "interior"])
def test_mixed_host_initial_guess(start):
    """Host arrays: an all-zero initial guess is not copied (the host scans it while the
    right-hand side is on its way; the staging buffer is cleared on the device), any other
    is -- a Dirichlet value on one ghost face, or a non-zero interior.  Every case equals
    the device-buffer solve bit for bit."""
    mesh, rhs, _ = problems.sine(48)
    shape = (50,) * 3
    x0 = np.zeros(shape)
    if start == "ghost_face":
        x0[:, :, 0] = 0.25
    elif start == "interior":
        x0[1:-1, 1:-1, 1:-1] = np.random.default_rng(5).uniform(-0.1, 0.1, (48, 48, 48))
    b = np.ascontiguousarray(np.asfortranarray(rhs).T)
    with pmg.Multigrid(mesh, 4, 50, precision="mixed") as mg:
        ds = torch.from_numpy(x0.copy()).cuda()
        dr = torch.zeros_like(ds)
        rep_d = mg.solve_vcycle(ds, dr, torch.from_numpy(b).cuda(), 2, 1e-10, 1.0)
        hs, hr = x0.copy(), np.zeros(shape)
        rep = mg.solve_vcycle(hs, hr, b, 2, 1e-10, 1.0)
    assert rep.converged and np.array_equal(rep.history, rep_d.history)
    assert np.array_equal(hs, ds.cpu().numpy()) and np.array_equal(hr, dr.cpu().numpy())
