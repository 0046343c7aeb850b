"""Failure detection without a GPU fault.

* The abort flag (pmg_set_abort): set before a solve, the solve returns PMG_ETIMEOUT
  before its first cycle; set from another host thread during a long solve, the solve
  stops within a bounded time; cleared, the same context solves again with the bits of a
  fresh context.
* The timeout path of the TMA-fed smoother (pmg_selftest_wait_timeout): its bounded
  waits run out with no copy in flight, the error flag becomes PMG_ETIMEOUT, and the
  context then solves normally.
* Host-side injection of device-allocation failures (pmg_inject_alloc_failure): every
  allocation of pmg_create, of the first mixed solve and of a staged host solve can fail
  with PMG_ENOMEM without leaking or poisoning later calls.
* An exactly zero initial residual (rhs = 0, sol = 0) returns at once: sol stays 0,
  rsd = 0, no cycles, converged.
"""
import ctypes
import threading
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import peps_mg_gb300 as pmg  # noqa: E402
from peps_mg_gb300 import _lib  # noqa: E402
from peps_mg_gb300 import problems  # noqa: E402
from tests.helpers import from_dev, to_dev  # noqa: E402

ETIMEOUT, ENOMEM = _lib.PMG_ETIMEOUT, _lib.PMG_ENOMEM


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    yield
    _lib.load().pmg_inject_alloc_failure(-1)


def set_abort(mg, flag):
    _lib.check(_lib.load().pmg_set_abort(mg._h, int(flag)), "pmg_set_abort")


def solve(mg, rhs, tol=1e-10, maxit=2):
    b = to_dev(rhs)
    sol = torch.zeros_like(b)
    rsd = torch.zeros_like(b)
    rep = mg.solve_vcycle(sol, rsd, b, maxit, tol, 1.0)
    torch.cuda.synchronize()
    return from_dev(sol), from_dev(rsd), rep


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_abort_before_solve_then_clear(precision):
    mesh, rhs = problems.gaussian_blobs(64)
    with pmg.Multigrid(mesh, 4, 40, "cgs", precision=precision) as fresh:
        ref_sol, _, ref_rep = solve(fresh, rhs)
    with pmg.Multigrid(mesh, 4, 40, "cgs", precision=precision) as mg:
        set_abort(mg, 1)
        t0 = time.perf_counter()
        with pytest.raises(pmg.PmgError) as e:
            solve(mg, rhs)
        assert e.value.status == ETIMEOUT
        assert "abort" in _lib.load().pmg_last_error().decode()
        assert time.perf_counter() - t0 < 5.0
        set_abort(mg, 0)
        sol, _, rep = solve(mg, rhs)
    assert rep.cycles == ref_rep.cycles and rep.converged
    assert np.array_equal(sol, ref_sol)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_abort_from_another_thread(precision):
    """A solve that would run for minutes (tolerance 0 is never reached, and each coarsest
    solve runs its 1000 RBGS iterations) stops soon after another thread sets the flag.
    (With the CG coarse solver a zero tolerance breaks CG down to NaN once the coarsest
    residual vanishes, as in the reference, so that solver is not used here.)"""
    coarse = "rbgs"
    mesh, rhs = problems.gaussian_blobs(96)
    with pmg.Multigrid(mesh, 5, 100000, "cgs", coarse_solver=coarse, precision=precision) as mg:
        solve(mg, rhs)                     # set-up (autotuning, graphs) outside the timing
        b = to_dev(rhs)
        sol, rsd = torch.zeros_like(b), torch.zeros_like(b)
        torch.cuda.synchronize()
        out = {}

        def run():
            try:
                out["rep"] = mg.solve_vcycle(sol, rsd, b, 2, 0.0, 1.0)
            except pmg.PmgError as exc:
                out["err"] = exc

        th = threading.Thread(target=run)
        th.start()
        time.sleep(0.5)
        t0 = time.perf_counter()
        set_abort(mg, 1)
        th.join(timeout=60.0)
        assert not th.is_alive(), "the solve did not stop after the abort flag was set"
        assert time.perf_counter() - t0 < 10.0
        assert "err" in out and out["err"].status == ETIMEOUT, out
        set_abort(mg, 0)
        # usable afterwards
        s2, _, rep = solve(mg, rhs)
        assert rep.converged


def test_wait_timeout_selftest_then_solve():
    mesh, rhs = problems.gaussian_blobs(64)
    with pmg.Multigrid(mesh, 4, 40, "cgs", precision="mixed", mixed_inner_cycles=2) as fresh:
        ref_sol, _, ref_rep = solve(fresh, rhs)
    with pmg.Multigrid(mesh, 4, 40, "cgs", precision="mixed", mixed_inner_cycles=2) as mg:
        solve(mg, rhs)
        lib = _lib.load()
        for _ in range(2):
            rc = lib.pmg_selftest_wait_timeout(mg._h, 0)
            assert rc == ETIMEOUT, rc
            assert "timed out" in lib.pmg_last_error().decode()
        sol, _, rep = solve(mg, rhs)
    assert rep.cycles == ref_rep.cycles
    assert np.array_equal(sol, ref_sol)


def test_wait_timeout_selftest_rejects_levels_without_tma():
    mesh, _ = problems.gaussian_blobs(32)
    with pmg.Multigrid(mesh, 3, 10, "cgs", precision="mixed") as mg:
        assert _lib.load().pmg_selftest_wait_timeout(mg._h, 99) == _lib.PMG_EINVAL


def test_allocation_failures_are_reported_and_recoverable():
    lib = _lib.load()
    mesh, rhs = problems.gaussian_blobs(48)
    # every allocation of multigrid_create, one at a time
    k, failures = 0, 0
    while True:
        lib.pmg_inject_alloc_failure(k)
        try:
            mg = pmg.Multigrid(mesh, 4, 40, "cgs", precision="mixed", mixed_inner_cycles=2)
        except pmg.PmgError as e:
            assert e.status == ENOMEM, e
            failures += 1
            k += 1
            assert k < 200
            continue
        lib.pmg_inject_alloc_failure(-1)
        break
    assert failures >= 5
    # the first mixed solve allocates the FP32 state: each of its allocations can fail
    with mg:
        k = 0
        while True:
            lib.pmg_inject_alloc_failure(k)
            try:
                solve(mg, rhs)
            except pmg.PmgError as e:
                assert e.status == ENOMEM, e
                k += 1
                assert k < 200
                continue
            lib.pmg_inject_alloc_failure(-1)
            break
        sol, _, rep = solve(mg, rhs)
        assert rep.converged
    with pmg.Multigrid(mesh, 4, 40, "cgs", precision="mixed", mixed_inner_cycles=2) as fresh:
        ref_sol, _, _ = solve(fresh, rhs)
    assert np.array_equal(sol, ref_sol)
    # a staged solve from host arrays allocates its staging buffers
    with pmg.Multigrid(mesh, 4, 40, "cgs") as mg:
        h_rhs = np.ascontiguousarray(rhs.T)
        h_sol, h_rsd = np.zeros_like(h_rhs), np.zeros_like(h_rhs)
        lib.pmg_inject_alloc_failure(0)
        with pytest.raises(pmg.PmgError) as e:
            mg.solve_vcycle(h_sol, h_rsd, h_rhs, 2, 1e-10, 1.0)
        assert e.value.status == ENOMEM
        lib.pmg_inject_alloc_failure(-1)
        rep = mg.solve_vcycle(h_sol, h_rsd, h_rhs, 2, 1e-10, 1.0)
        assert rep.converged


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_zero_rhs_and_zero_guess(precision):
    mesh, rhs = problems.gaussian_blobs(32)
    rhs[...] = 0.0
    with pmg.Multigrid(mesh, 3, 20, "cgs", precision=precision) as mg:
        b = to_dev(rhs)
        sol = torch.zeros_like(b)
        rsd = torch.full_like(b, 7.0)
        rep = mg.solve_vcycle(sol, rsd, b, 2, 1e-10, 1.0)
        torch.cuda.synchronize()
        assert rep.cycles == 0 and rep.converged and rep.final_ratio == 0.0 and rep.res0 == 0.0
        assert not sol.any()
        assert not rsd.any()
