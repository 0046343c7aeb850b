"""The fused FP32 red-black smoother, one iteration at a time, against the oracle's FP64
rbgs_iterator (src/rbgs_poisson_matrix.f90:191) on stretched meshes whose tiles and
plane chunks end part-way through the grid; the TMA-fed, register-window and one-launch
cell-pair kernels must agree bit for bit."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import peps_mg_gb300 as pmg  # noqa: E402
from oracle import oracle as O  # noqa: E402
from peps_mg_gb300 import _lib  # noqa: E402

FP32_TOL = 2e-6   # max |e32 - e64| / max |e64| after one iteration


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def stretched_mesh(n, seed):
    rng = np.random.default_rng(seed)
    return [pmg.geometry.mesh_from_widths(rng.uniform(0.7, 1.3, m) / m) for m in n]


def run_selftest(mg, impl, variant, kchunk, zero_in, omega, e_in, b):
    out = pmg.geometry.field(*(s - 2 for s in e_in.shape))
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    rc = _lib.load().pmg_selftest_smooth32(mg._h, 0, impl, variant, kchunk, int(zero_in), float(omega), P(e_in), P(b),
                                          P(out))
    _lib.check(rc, "pmg_selftest_smooth32")
    return out


# (nx, ny, nz): 200 x 92 x 40 ends part-way through 60-column tiles and 14/10/22-row
# tiles; 124 x 132 x 68 leaves 4 columns in its last tile and 4 planes in its last chunk
@pytest.mark.parametrize("n", [(200, 92, 40), (124, 132, 68)])
def test_one_iteration_against_oracle(n):
    mesh = stretched_mesh(n, seed=sum(n))
    coeff = O.matrix_create(mesh)
    rng = np.random.default_rng(7)
    e0 = pmg.geometry.field(*n)
    e0[1:-1, 1:-1, 1:-1] = rng.uniform(-1, 1, n)
    b = pmg.geometry.field(*n)
    b[1:-1, 1:-1, 1:-1] = rng.uniform(-1, 1, n) * np.abs(coeff[0]).max()
    with pmg.Multigrid(mesh, 2, 1, "cgs", precision="mixed") as mg:
        for omega in (1.0, 1.3):
            for zero_in in (False, True):
                ref = e0.copy(order="F") if not zero_in else pmg.geometry.field(*n)
                O.rbgs_iterator(coeff, ref, b, 1, omega)
                scale = np.abs(ref).max()
                # variant 3 (60 x 22 tiles) exists for the TMA-fed kernel only
                for variant in (0, 1, 2, 3):
                    for kchunk in (0, 16, 7):
                        outs = []
                        for impl in ((0,) if variant == 3 else (0, 1)):
                            got = run_selftest(mg, impl, variant, kchunk, zero_in, omega, e0, b)
                            err = np.abs(got - ref).max() / scale
                            assert err < FP32_TOL, (impl, variant, kchunk, zero_in, omega, err)
                            outs.append(got)
                        assert all(np.array_equal(outs[0], o) for o in outs[1:]), (variant, kchunk, zero_in, omega)
                # the cell-pair kernel (no tiles, no chunks) against the tiled kernels' bits
                got = run_selftest(mg, 2, 0, 0, zero_in, omega, e0, b)
                assert np.array_equal(got, outs[0]), (zero_in, omega)


def test_kernel_variants_give_identical_solves(tmp_path):
    """A whole mixed-precision solve gives the same bits with any smoother kernel (TMA-fed,
    register-window or one-launch cell-pair, or the autotuner's mix of them), with
    either kind of transfer kernel (marching or one thread per cell), and with the FP32
    V-cycles replayed as CUDA graphs or launched kernel by kernel."""
    import os
    import subprocess
    import sys
    code = r'''
import numpy as np, torch, peps_mg_gb300 as pmg
from tests.helpers import to_dev, from_dev
n = (96, 80, 64)
rng = np.random.default_rng(5)
mesh = [pmg.geometry.uniform_axis(m, 0.0, 1.0) for m in n]
rhs = pmg.geometry.field(*n); rhs[1:-1, 1:-1, 1:-1] = rng.uniform(-1, 1, n)
with pmg.Multigrid(mesh, 4, 50, "cgs", precision="mixed") as mg:
    sol = torch.zeros((n[2] + 2, n[1] + 2, n[0] + 2), dtype=torch.float64, device="cuda")
    rsd = torch.zeros_like(sol)
    rep = mg.solve_vcycle(sol, rsd, to_dev(rhs), 2, 1e-10, 1.0)
np.save(__import__("sys").argv[1], from_dev(sol))
print(rep.cycles)
'''
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    outs = []
    for sm, tr, gr in (("tma", "march", "1"), ("window", "march", "1"), ("tma", "cell", "1"), ("tma", "march", "0"),
                       ("cell", "march", "1")):
        env = dict(os.environ, PEPS_MG_SMOOTHER=sm, PEPS_MG_TRANSFER=tr, PEPS_MG_GRAPHS=gr, PYTHONPATH=root)
        path = str(tmp_path / ("%s_%s_%s.npy" % (sm, tr, gr)))
        r = subprocess.run([sys.executable, "-c", code, path], cwd=root, env=env, capture_output=True, text=True,
                           timeout=300)
        assert r.returncode == 0, r.stderr[-2000:]
        outs.append(np.load(path))
    assert np.array_equal(outs[0], outs[1])
    assert np.array_equal(outs[0], outs[2])
    assert np.array_equal(outs[0], outs[3])
    assert np.array_equal(outs[0], outs[4])
