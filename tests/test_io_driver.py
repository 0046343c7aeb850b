"""The reference's input/output formats and the driver's host-side setup (no GPU)."""
import struct

import numpy as np
import pytest

from oracle import oracle as O
from peps_mg_gb300 import driver
from peps_mg_gb300 import io as pio

SAMPLE = """! a driver input in the reference's namelist format
&meshes
nx = 24, ny = 16
nz = 20   ! trailing comment
/
&origin
ox = -0.5d0 oy=-0.5D0
oz = -5.0E-1
/
&length
lx = 1.0d0
ly = 1.0d0
lz = 1.0d0
/
&mesh_stretch
ax = 1.05d0
ay = 1.0d0
az = 1.0d0
/
&procs
npx = 1
npy = 1
npz = 1
/
&control
maxiteration = 2
tolerance = 1.0d-10
number_of_vcycles = 40
number_of_levels = 3
aggregation_method = 2
CGA_level = 0
CGPSA_level(1) = 1, CGPSA_level(2) = 2
CGPSA_level(3) = 3
omega_sor = 1.0d0
/
&coefficients
alpha_x = 1.0d0
alpha_y = 1.0d0
alpha_z = 1.0d0
/
"""


def test_namelist_parsing():
    nl = pio.parse_namelists(SAMPLE)
    assert nl["meshes"] == {"nx": 24, "ny": 16, "nz": 20}
    assert nl["origin"] == {"ox": -0.5, "oy": -0.5, "oz": -0.5}
    assert nl["control"]["tolerance"] == 1e-10
    assert nl["control"]["cgpsa_level"] == [1, 2, 3]
    assert nl["control"]["aggregation_method"] == 2
    assert nl["mesh_stretch"]["ax"] == 1.05
    nl2 = pio.parse_namelists("&control\n CGPSA_level = 9, 6, 8\n flag = .true.\n name = 'abc'\n/\n")
    assert nl2["control"] == {"cgpsa_level": [9, 6, 8], "flag": True, "name": "abc"}


def test_read_config_checks(tmp_path):
    p = tmp_path / "PARA_INPUT.inp"
    p.write_text(SAMPLE)
    cfg = driver.read_config(str(p))
    assert cfg["control"]["cgpsa_level"] == [1, 2, 3]
    p.write_text(SAMPLE.replace("aggregation_method = 2", "aggregation_method = 7"))
    with pytest.raises(ValueError, match="Aggregation method"):
        driver.read_config(str(p))
    p.write_text(SAMPLE.replace("&length", "&lengths"))
    with pytest.raises(ValueError, match="&length"):
        driver.read_config(str(p))


@pytest.mark.parametrize("value,d20,e30", [
    (0.5, "    0.5000000000D+00", "    0.50000000000000000000E+00"),
    (-0.5, "   -0.5000000000D+00", "   -0.50000000000000000000E+00"),
    (1.0, "    0.1000000000D+01", "    0.10000000000000000000E+01"),
    (0.0, "    0.0000000000D+00", "    0.00000000000000000000E+00"),
    (1e-5, "    0.1000000000D-04", "    0.10000000000000000818E-04"),
    (9.99999999999e9, "    0.1000000000D+11", "    0.99999999999899997711E+10"),
    (-2.5e-120, "   -0.2500000000-119", "   -0.25000000000000000325-119"),
])
def test_fortran_edit_descriptors(value, d20, e30):
    assert pio.fortran_exp(value, 20, 10, "D") == d20
    assert pio.fortran_exp(value, 30, 20, "E") == e30


def test_binary_formats_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    u = np.asfortranarray(rng.standard_normal((5, 4, 3)))
    pio.write_fortran_record(str(tmp_path / "a.bin"), u)
    raw = (tmp_path / "a.bin").read_bytes()
    assert len(raw) == 8 + 8 * u.size
    assert struct.unpack("<i", raw[:4])[0] == 8 * u.size == struct.unpack("<i", raw[-4:])[0]
    assert np.array_equal(np.frombuffer(raw[4:-4], "<f8"), u.ravel(order="F"))
    assert np.array_equal(pio.read_fortran_record(str(tmp_path / "a.bin"), u.shape), u)
    pio.write_raw(str(tmp_path / "b.bin"), u)
    assert (tmp_path / "b.bin").read_bytes() == raw[4:-4]
    assert np.array_equal(pio.read_raw(str(tmp_path / "b.bin"), u.shape), u)


def test_ascii_format(tmp_path):
    rng = np.random.default_rng(2)
    xg, yg, zg = np.linspace(-0.4, 0.4, 3), np.linspace(0.1, 0.2, 2), np.array([1.5])
    u = np.asfortranarray(rng.standard_normal((3, 2, 1)))
    field = np.zeros((5, 4, 3), order="F")
    field[1:-1, 1:-1, 1:-1] = u
    pio.write_ascii(str(tmp_path / "s.dat"), xg, yg, zg, field)
    lines = (tmp_path / "s.dat").read_text().splitlines()
    assert len(lines) == 6 and all(len(ln) == 90 for ln in lines)
    x, y, z, v = pio.read_ascii(str(tmp_path / "s.dat"))
    assert np.allclose(x, np.tile(xg, 2), rtol=1e-10) and np.allclose(y, np.repeat(yg, 3), rtol=1e-10)
    assert np.allclose(v, u.ravel(order="F"), rtol=1e-19, atol=0)


def test_driver_mesh_and_problem_match_the_oracle():
    """The driver's global mesh is the oracle's geometry_domain_create bit for bit, and its
    right-hand side is the reference's problem 1."""
    nl = pio.parse_namelists(SAMPLE)
    m, o, ln, st = nl["meshes"], nl["origin"], nl["length"], nl["mesh_stretch"]
    for a in "xyz":
        ours = driver.domain_mesh(m["n" + a], o["o" + a], ln["l" + a], st["a" + a])
        ref = O.mesh_axis(m["n" + a], o["o" + a], ln["l" + a], st["a" + a])
        for u, v in zip(ours, ref):
            assert np.array_equal(u, v), a
    mesh = [driver.domain_mesh(m["n" + a], o["o" + a], ln["l" + a], st["a" + a]) for a in "xyz"]
    b, exact = driver.cosine_problem(mesh, (1.0, 1.0, 1.0))
    i, j, k = 3, 5, 7
    x, y, z = mesh[0][2][i], mesh[1][2][j], mesh[2][2][k]
    want = -np.cos(x * np.pi) * np.cos(y * np.pi) * np.cos(z * np.pi) * np.pi ** 2 * 3.0
    assert abs(b[i, j, k] - want) <= 1e-14 * abs(want)
    assert abs(exact[i - 1, j - 1, k - 1] - np.cos(x * np.pi) * np.cos(y * np.pi) * np.cos(z * np.pi)) < 1e-15
    assert np.all(b[0] == 0) and np.all(b[:, :, -1] == 0)
