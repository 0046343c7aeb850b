"""pmg_vv_dot_static: the interior dot product for callers that cannot allocate device
memory, checked against pmg_vv_dot (a context's dot product) through the C-ABI.

Collected last so that it also runs after every other test in one process; it passes
alone in a fresh process too (the first call does the per-device set-up).
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import peps_mg_gb300 as pmg  # noqa: E402
from peps_mg_gb300 import _lib  # noqa: E402
from peps_mg_gb300 import geometry as G  # noqa: E402

REL_TOL = 1e-12   # FP64 sums of the same products in another order


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def static_dot(x, y, nx, ny, nz, stream=None):
    out = ctypes.c_double(np.nan)
    rc = _lib.load().pmg_vv_dot_static(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), nx, ny, nz,
                                       stream, ctypes.byref(out))
    _lib.check(rc, "pmg_vv_dot_static")
    return out.value


def fields(nx, ny, nz, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    shape = (nz + 2, ny + 2, nx + 2)
    return (torch.rand(shape, dtype=torch.float64, device="cuda", generator=g) * 2 - 1,
            torch.rand(shape, dtype=torch.float64, device="cuda", generator=g) * 2 - 1)


# (nx, ny, nz, levels): one grid whose z extent fits the scratch uncapped (same order
# of operations as pmg_vv_dot), two whose CTA grid is capped in z, one odd-sized
@pytest.mark.parametrize("nx,ny,nz,levels", [(64, 48, 40, 3), (256, 256, 96, 4), (512, 128, 512, 5),
                                             (100, 36, 20, 2)])
def test_static_dot_matches_vv_dot_twice(nx, ny, nz, levels):
    x, y = fields(nx, ny, nz, seed=nx + ny + nz)
    mesh = [G.uniform_axis(n, 0.0, 1.0) for n in (nx, ny, nz)]
    with pmg.Multigrid(mesh, levels, 1, "cgs") as mg:
        ref = mg.vv_dot(0, x, y)
    torch.cuda.synchronize()
    first = static_dot(x, y, nx, ny, nz)
    second = static_dot(x, y, nx, ny, nz)
    assert abs(first - ref) <= REL_TOL * abs(ref), (first, ref)
    assert abs(second - ref) <= REL_TOL * abs(ref), (second, ref)
    assert first == second
    gx, gy = -(-nx // 32), -(-ny // 8)
    if gx * gy * nz <= 16384:
        assert first == ref   # uncapped grid: same partials, same order


def test_static_dot_on_a_caller_stream():
    nx, ny, nz = 96, 64, 48
    x, y = fields(nx, ny, nz, seed=7)
    ref = float((x[1:-1, 1:-1, 1:-1] * y[1:-1, 1:-1, 1:-1]).sum())
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    for _ in range(2):
        v = static_dot(x, y, nx, ny, nz, stream=ctypes.c_void_p(s.cuda_stream))
        assert abs(v - ref) <= REL_TOL * abs(ref)


def test_static_dot_rejects_planes_beyond_the_scratch():
    x, y = fields(8, 8, 8, seed=1)
    # ceil(6400/32) * ceil(800/8) = 20000 partial sums > 16384; rejected before any access
    rc = _lib.load().pmg_vv_dot_static(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), 6400, 800, 4,
                                       None, ctypes.byref(ctypes.c_double()))
    assert rc == 1
    msg = _lib.load().pmg_last_error().decode()
    assert "static scratch holds 16384" in msg
    with pytest.raises(pmg.PmgError):
        _lib.check(rc, "pmg_vv_dot_static")
