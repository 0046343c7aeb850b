"""The C oracle reproduces the independent numpy restatement's golden fixtures bit for bit."""
import numpy as np
import pytest

from oracle import oracle as O


def mesh_of(g, p):
    return [(g[p + "d%sm" % a], g[p + "d%sg" % a], g[p + "%sg" % a]) for a in "xyz"]


def F(a):
    return np.asfortranarray(a.copy())


def test_coefficients(golden):
    g = golden
    c = O.matrix_create(mesh_of(g, "A_"))
    assert np.array_equal(c, np.asfortranarray(g["A_coeff"]))


def test_operator_kernels(golden):
    g = golden
    c = O.matrix_create(mesh_of(g, "A_"))
    x, b, y = F(g["A_x"]), F(g["A_b"]), F(g["A_y"])
    assert np.array_equal(O.mv_mul(c, x), g["A_mv"])
    assert np.array_equal(O.residual(c, x, b), g["A_res"])
    assert O.vv_dot(x, y) == g["A_dot"][0]


@pytest.mark.parametrize("tag,omega,it", [("w16", 1.6, 2), ("w10", 1.0, 3)])
def test_rbgs_iterator(golden, tag, omega, it):
    g = golden
    c = O.matrix_create(mesh_of(g, "A_"))
    x = F(g["A_x"])
    O.rbgs_iterator(c, x, F(g["A_b"]), it, omega)
    assert np.array_equal(x, g["A_rbgs_" + tag])


def test_rbgs_and_cg_solvers(golden):
    g = golden
    c = O.matrix_create(mesh_of(g, "A_"))
    x = F(g["A_x"])
    it, _, _ = O.rbgs_solver(c, x, F(g["A_b"]), 50, 1e-6, 1.3)
    assert it == g["A_rbgs_solver_iters"][0]
    assert np.array_equal(x, g["A_rbgs_solver_x"])
    x = F(g["A_x"])
    it, _, _ = O.cg(c, x, F(g["A_b"]), 200, 1e-9)
    assert it == g["A_cg_solver_iters"][0]
    assert np.array_equal(x, g["A_cg_solver_x"])
    x = F(g["A_x"])
    O.cg(c, x, F(g["A_b"]), 5, 0.0, check_tol=False)
    assert np.array_equal(x, g["A_cg_iter5_x"])


def test_hierarchy_mesh_and_transfer(golden):
    g = golden
    mesh = mesh_of(g, "B_")
    mg = O.OracleMG(mesh, 3, 1)
    for l in range(4):
        assert mg.level_dims(l) == tuple(g["B_sizes"][l])
    assert mg.coarsest() == tuple(g["B_lvc"])
    for l in range(1, 4):
        for d, a in enumerate("xyz"):
            dm, dg, _ = mg.level_mesh(l, d)
            assert np.array_equal(dm, g["B_L%d_d%sm" % (l, a)])
            assert np.array_equal(dg, g["B_L%d_d%sg" % (l, a)])
    lib = O._lib()
    for l in range(3):
        nf, nc = mg.level_dims(l), mg.level_dims(l + 1)
        mf = [mg.level_mesh(l, d)[0] for d in range(3)]
        mc = [mg.level_mesh(l + 1, d)[0] for d in range(3)]
        co = np.array(mg.coarsest(), dtype=np.int32)
        vf = F(g["B_R%d_in" % l])
        out = O.field(*nc)
        lib.orc_restriction(*nc, O.P(mc[0]), O.P(mc[1]), O.P(mc[2]), *nf, O.P(mf[0]), O.P(mf[1]), O.P(mf[2]),
                            l, co.ctypes.data_as(O._ip), O.P(vf), O.P(out))
        assert np.array_equal(out, g["B_R%d_out" % l]), l
        vc = F(g["B_P%d_in" % l])
        base = F(g["B_P%d_base" % l])
        lib.orc_prolongation(*nc, O.P(mc[0]), O.P(mc[1]), O.P(mc[2]), *nf, O.P(mf[0]), O.P(mf[1]), O.P(mf[2]),
                             l, co.ctypes.data_as(O._ip), O.P(vc), O.P(base))
        assert np.array_equal(base, g["B_P%d_out" % l]), l


@pytest.mark.parametrize("tag,method,cga,cs", [("cgs_rbgs", 0, 0, 0), ("cgs_cg", 0, 0, 1),
                                               ("cga_rbgs", 1, 2, 0), ("cgpsa_rbgs", 2, 0, 0)])
def test_vcycle_solve(golden, tag, method, cga, cs):
    g = golden
    mg = O.OracleMG(mesh_of(g, "B_"), 3, 40, method=method, cga_level=cga, coarse_solver=cs)
    sol = F(g["C_sol0"])
    rsd = O.field(*mg.level_dims(0))
    ncyc, hist, ci = mg.solve(sol, rsd, F(g["C_rhs"]), 2, 1e-9, 1.2)
    assert ncyc == len(g["C_%s_hist" % tag])
    assert np.array_equal(ci, g["C_%s_citers" % tag])
    assert np.array_equal(hist, g["C_%s_hist" % tag])
    assert np.array_equal(sol, g["C_%s_sol" % tag])
    assert np.array_equal(rsd, g["C_%s_rsd" % tag])


def test_level_size_rules(golden):
    for row in golden["D_table"]:
        n = tuple(int(v) for v in row[:3])
        nl, meth, cga, ok = (int(v) for v in row[3:7])
        rc, sizes, co = O.level_sizes(*n, nl, meth, cga) if nl >= 1 else (1, None, None)
        assert (rc == 0) == bool(ok), row
        if ok:
            assert tuple(co) == tuple(row[7:10])
            flat = sizes.ravel()
            assert np.array_equal(flat, row[10:10 + len(flat)]), row


def test_unit_cube_sine_problem(golden):
    g = golden
    mg = O.OracleMG(mesh_of(g, "E_"), 2, 60, method=0, coarse_solver=1)
    rhs = F(g["E_rhs"])
    sol = O.field(16, 16, 16)
    rsd = O.field(16, 16, 16)
    ncyc, hist, ci = mg.solve(sol, rsd, rhs, 2, 1e-10, 1.0)
    assert np.array_equal(hist, g["E_hist"])
    assert np.array_equal(sol, g["E_sol"])
    assert hist[-1, 2] < 1e-10


def test_known_answers():
    """Hand-derived values of the reference formulas on a uniform 4^3 unit cube."""
    m = O.mesh_axis(4, 0.0, 1.0, 1.0)
    assert np.array_equal(m[0], [0.0, 0.25, 0.25, 0.25, 0.25, 0.0])
    assert np.array_equal(m[1], [0.0, 0.125, 0.25, 0.25, 0.25, 0.125])
    c = O.matrix_create([m, m, m])
    # boundary cell (1,1,1): c1 = 1/(0.25*0.125) = 32, c2 = 1/(0.25*0.25) = 16
    assert c[1, 0, 0, 0] == 32.0 and c[2, 0, 0, 0] == 16.0
    assert c[0, 0, 0, 0] == -(32.0 + 16.0) * 3
    assert c[0, 1, 1, 1] == -96.0
    # restriction of a constant is that constant (volume-weighted mean)
    mg = O.OracleMG([m, m, m], 2, 1)
    assert mg.level_dims(1) == (2, 2, 2)
    assert np.array_equal(mg.level_mesh(1, 0)[0], [0.0, 0.5, 0.5, 0.0])
    # one-cell coarsest level solves x = b / c0 exactly
    rc, sizes, co = O.level_sizes(4, 4, 4, 2, 0, 0)
    assert rc == 0 and tuple(sizes[2]) == (1, 1, 1) and tuple(co) == (2, 2, 2)
