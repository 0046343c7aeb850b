"""The PARA_INPUT.inp driver on the GPU: the reference's problem 1 on a stretched mesh
with each aggregation method, against the oracle (bit for bit in FP64), plus the
written solution files."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import oracle as O  # noqa: E402
from peps_mg_gb300 import driver  # noqa: E402
from peps_mg_gb300 import io as pio  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def para_input(method, cga, cgpsa, n=(32, 24, 40), levels=3, stretch=1.05, procs=(1, 1, 1)):
    return """&meshes
nx = %d
ny = %d
nz = %d
/
&origin
ox = -0.5d0
oy = -0.5d0
oz = -0.5d0
/
&length
lx = 1.0d0
ly = 1.0d0
lz = 1.0d0
/
&mesh_stretch
ax = %sd0
ay = 1.0d0
az = 1.0d0
/
&procs
npx = %d
npy = %d
npz = %d
/
&control
maxiteration = 2
tolerance = 1.0d-10
number_of_vcycles = 60
number_of_levels = %d
aggregation_method = %d
CGA_level = %d
CGPSA_level = %d, %d, %d
omega_sor = 1.0d0
/
&coefficients
alpha_x = 1.0d0
alpha_y = 1.0d0
alpha_z = 1.0d0
/
""" % (n + (repr(stretch),) + procs + (levels, method, cga) + tuple(cgpsa))


@pytest.mark.parametrize("method,cga,cgpsa", [(0, 0, (0, 0, 0)), (1, 2, (0, 0, 0)), (2, 0, (1, 2, 3))])
def test_driver_matches_oracle(tmp_path, method, cga, cgpsa):
    p = tmp_path / "PARA_INPUT.inp"
    p.write_text(para_input(method, cga, cgpsa))
    lines = []
    res = driver.run(str(p), write_dir=str(tmp_path / "out"), log=lines.append)
    rep = res["report"]
    assert rep.converged
    assert any(ln.startswith("[Poisson] RMS = ") for ln in lines)
    assert sum(ln.startswith("[MG] cycle =") for ln in lines) == rep.cycles
    assert res["rms"] < 1e-5
    # the oracle on the same mesh and right-hand side
    mesh = res["mesh"]
    rhs, _ = driver.cosine_problem(mesh, (1.0, 1.0, 1.0))
    omg = O.OracleMG(mesh, 3, 60, method, cga)
    n = tuple(len(m[0]) - 2 for m in mesh)
    osol, orsd = O.field(*n), O.field(*n)
    ncyc, hist, ci = omg.solve(osol, orsd, np.asfortranarray(rhs), 2, 1e-10, 1.0)
    omg.close()
    assert rep.cycles == ncyc
    assert np.array_equal(res["sol"], osol)
    inner = res["sol"][1:-1, 1:-1, 1:-1]
    assert np.array_equal(pio.read_fortran_record(str(tmp_path / "out" / "solution_all.bin"), n), inner)
    assert np.array_equal(pio.read_raw(str(tmp_path / "out" / "solution_all_MPI_IO.bin"), n), inner)
    x, y, z, u = pio.read_ascii(str(tmp_path / "out" / "solution_all.dat"))
    assert np.allclose(u, inner.ravel(order="F"), rtol=1e-19, atol=1e-300)


def test_driver_mixed_precision_and_ranks_note(tmp_path):
    p = tmp_path / "PARA_INPUT.inp"
    p.write_text(para_input(0, 0, (0, 0, 0), n=(64, 64, 64), levels=4, stretch=1.0, procs=(2, 2, 1)))
    lines = []
    res = driver.run(str(p), precision="mixed", log=lines.append)
    assert res["report"].converged
    assert any("one GPU solves the whole domain" in ln for ln in lines)
    assert res["rms"] < 1e-6
