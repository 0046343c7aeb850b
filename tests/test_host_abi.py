"""CPU-only checks of the C-ABI library: it loads, exports every symbol declared in
include/peps_mg.h, and its host-side hierarchy rules agree with the oracle."""
import os
import re

import numpy as np
import pytest

import peps_mg_gb300 as pmg
from oracle import oracle as O
from peps_mg_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "peps_mg.h")).read()
    return sorted(set(re.findall(r"^(?:int|const char \*)\s*(pmg_\w+)\s*\(", txt, re.M)))


def test_library_exports_header_symbols():
    lib = pmg.load()
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(_lib.EXPORTED)


def test_status_strings():
    lib = pmg.load()
    assert lib.pmg_status_string(0) == b"ok"
    assert lib.pmg_status_string(3) == b"diverged"


def test_level_size_rules_match_oracle(golden):
    for row in golden["D_table"]:
        n = tuple(int(v) for v in row[:3])
        nl, meth, cga, ok = (int(v) for v in row[3:7])
        if ok:
            sizes, co = pmg.level_sizes(n, nl, meth, cga)
            assert tuple(co) == tuple(row[7:10])
            assert np.array_equal(sizes.ravel(), row[10:10 + sizes.size])
        else:
            with pytest.raises(pmg.PmgError):
                pmg.level_sizes(n, nl, meth, cga)


@pytest.mark.parametrize("n,nl,meth,cga", [((512, 512, 512), 8, 0, 0), ((256, 256, 256), 7, 1, 4),
                                           ((256, 256, 256), 7, 2, 0), ((96, 48, 192), 5, 0, 0),
                                           ((192, 32, 128), 5, 0, 0), ((7, 9, 11), 2, 0, 0)])
def test_level_sizes_random_agree(n, nl, meth, cga):
    rc, sizes, co = O.level_sizes(*n, nl, meth, cga)
    if rc != 0:
        with pytest.raises(pmg.PmgError):
            pmg.level_sizes(n, nl, meth, cga)
        return
    s2, c2 = pmg.level_sizes(n, nl, meth, cga)
    assert np.array_equal(s2, sizes) and tuple(c2) == tuple(co)


def test_create_rejects_bad_config_without_gpu():
    mesh = [pmg.geometry.uniform_axis(16, 0.0, 1.0)] * 3
    with pytest.raises(pmg.PmgError) as e:
        pmg.Multigrid(mesh, 9, 10, "cgs")
    assert e.value.status == _lib.PMG_EINVAL
    with pytest.raises(pmg.PmgError):
        pmg.Multigrid(mesh, 3, 10, "cgs", coarse_solver=5)


def test_geometry_matches_oracle_mesh():
    for n, a in ((16, 1.0), (32, 1.1), (10, 0.9)):
        ref = O.mesh_axis(n, -0.5, 2.0, a)
        got = pmg.geometry.stretched_axis(n, -0.5, 2.0, a)
        for r, g_ in zip(ref, got):
            assert np.array_equal(r, g_)
