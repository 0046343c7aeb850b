"""Generate tests/golden/golden.npz from the independent numpy restatement.

Run:  python tests/golden/make_golden.py
The fixtures pin the C oracle (oracle/pmg_oracle.c): tests/test_oracle_golden.py
requires bit-for-bit agreement.  All inputs are seeded synthetic data.
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import numpy_restatement as R  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz")


def stretched_mesh(n, rng, o=0.0):
    w = rng.uniform(0.5, 1.5, size=n)
    w = w / w.sum()
    return R.mesh_from_widths(w, o)


def field(shape, rng, ghosts=True):
    x = np.zeros(tuple(s + 2 for s in shape))
    if ghosts:
        x[...] = rng.uniform(-1.0, 1.0, size=x.shape)
    else:
        x[1:-1, 1:-1, 1:-1] = rng.uniform(-1.0, 1.0, size=shape)
    return x


def put_mesh(g, prefix, mesh):
    for d, ax in enumerate("xyz"):
        g[prefix + "d%sm" % ax] = mesh[d][0]
        g[prefix + "d%sg" % ax] = mesh[d][1]
        g[prefix + "%sg" % ax] = mesh[d][2]


def main():
    g = {}
    rng = np.random.default_rng(20210501)

    # A. operator kernels on a stretched 8x6x10 grid with non-zero ghost values
    shape = (8, 6, 10)
    mesh = [stretched_mesh(n, rng) for n in shape]
    put_mesh(g, "A_", mesh)
    c = R.coeff_fields(mesh)
    x = field(shape, rng)
    b = field(shape, rng)
    y = field(shape, rng)
    g["A_x"], g["A_b"], g["A_y"] = x, b, y
    g["A_coeff"] = np.stack(c)
    g["A_mv"] = R.mv_mul(c, x)
    g["A_res"] = R.residual(c, x, b)
    g["A_dot"] = np.array([R.vv_dot(x, y)])
    for tag, om, it in (("w16", 1.6, 2), ("w10", 1.0, 3)):
        xs = x.copy()
        R.rbgs_iterator(c, xs, b, it, om)
        g["A_rbgs_" + tag] = xs
    xs = x.copy()
    g["A_rbgs_solver_iters"] = np.array([R.rbgs_solver(c, xs, b, 50, 1e-6, 1.3)])
    g["A_rbgs_solver_x"] = xs
    xs = x.copy()
    g["A_cg_solver_iters"] = np.array([R.cg_solver(c, xs, b, 200, 1e-9)])
    g["A_cg_solver_x"] = xs
    xs = x.copy()
    R.cg_solver(c, xs, b, 5, 0.0, check=False)
    g["A_cg_iter5_x"] = xs

    # B. hierarchy with a stride-1 axis: 16x12x8, 3 levels -> 8x6x4, 4x3x2, 2x3x1
    shape = (16, 12, 8)
    mesh = [stretched_mesh(n, rng, o=-0.5) for n in shape]
    put_mesh(g, "B_", mesh)
    mg = R.NumpyMG(mesh, 3, 1)
    g["B_sizes"] = np.array(mg.sizes)
    g["B_lvc"] = np.array(mg.lvc)
    for l in range(1, 4):
        for d, ax in enumerate("xyz"):
            g["B_L%d_d%sm" % (l, ax)] = mg.meshes[l][d][0]
            g["B_L%d_d%sg" % (l, ax)] = mg.meshes[l][d][1]
    for l in range(0, 3):
        nf = mg.sizes[l]
        nc = mg.sizes[l + 1]
        vf = field(nf, rng)
        vc = field(nc, rng)
        g["B_R%d_in" % l] = vf
        g["B_R%d_out" % l] = mg._restrict(l, vf)
        g["B_P%d_in" % l] = vc
        base = field(nf, rng)
        g["B_P%d_base" % l] = base.copy()
        mg._prolong(l, vc, base)
        g["B_P%d_out" % l] = base

    # C. full V-cycle solves (RBGS and CG coarse solvers; CGS, CGA, CGPSA)
    rhs = field(shape, rng, ghosts=False)
    sol0 = np.zeros_like(rhs)
    sol0[0, :, :] = 0.25            # a Dirichlet value held in one ghost face
    g["C_rhs"], g["C_sol0"] = rhs, sol0
    runs = [("cgs_rbgs", 0, 0, 0), ("cgs_cg", 0, 0, 1), ("cga_rbgs", 1, 2, 0), ("cgpsa_rbgs", 2, 0, 0)]
    for tag, method, cga, cs in runs:
        mgc = R.NumpyMG(mesh, 3, 40, method=method, cga_level=cga, coarse_solver=cs)
        sol = sol0.copy()
        rsd = np.zeros_like(sol)
        ncyc, hist, citers = mgc.solve(sol, rsd, rhs, 2, 1e-9, 1.2)
        g["C_%s_sol" % tag] = sol
        g["C_%s_rsd" % tag] = rsd
        g["C_%s_hist" % tag] = hist
        g["C_%s_citers" % tag] = citers

    # D. level-size rules (sizes, or -1 for a configuration the reference rejects)
    cases = [((64, 64, 64), 4, 0, 0), ((64, 64, 64), 6, 0, 0), ((64, 64, 64), 7, 0, 0),
             ((48, 96, 32), 5, 0, 0), ((48, 96, 32), 6, 0, 0), ((256, 256, 256), 7, 1, 4),
             ((256, 256, 256), 7, 2, 0), ((256, 256, 256), 6, 2, 0), ((12, 12, 12), 3, 1, 3),
             ((12, 12, 12), 3, 1, 2), ((20, 8, 8), 3, 1, 1), ((6, 10, 14), 2, 2, 0),
             ((6, 10, 14), 3, 2, 0), ((64, 64, 64), 1, 0, 0), ((64, 64, 64), 4, 0, 2),
             ((64, 64, 64), 4, 1, 0), ((64, 64, 64), 4, 3, 0), ((2, 2, 2), 2, 0, 0),
             ((2, 2, 2), 1, 0, 0), ((4, 4, 4), 2, 0, 0), ((5, 8, 8), 3, 0, 0)]
    table = []
    for n, nl, meth, cga in cases:
        try:
            sizes, lvc = R.level_sizes(n, nl, meth, cga)
            ok = 1
        except ValueError:
            sizes, lvc, ok = [], [0, 0, 0], 0
        flat = [v for s in sizes for v in s]
        table.append([n[0], n[1], n[2], nl, meth, cga, ok] + list(lvc) + flat + [0] * (3 * 9 - len(flat)))
    g["D_table"] = np.array(table, dtype=np.int64)

    # E. 16^3 unit-cube problem of the 64^3 benchmark (sine right-hand side, zero ghosts)
    n = 16
    m = R.mesh_uniform(n, 0.0, 1.0)
    mesh = [m, m, m]
    put_mesh(g, "E_", mesh)
    X, Y, Z = np.meshgrid(m[2][1:-1], m[2][1:-1], m[2][1:-1], indexing="ij")
    rhs = np.zeros((n + 2,) * 3)
    rhs[1:-1, 1:-1, 1:-1] = -3.0 * np.pi ** 2 * np.sin(np.pi * X) * np.sin(np.pi * Y) * np.sin(np.pi * Z)
    g["E_rhs"] = rhs
    mge = R.NumpyMG(mesh, 2, 60, method=0, coarse_solver=1)
    sol = np.zeros_like(rhs)
    rsd = np.zeros_like(rhs)
    ncyc, hist, citers = mge.solve(sol, rsd, rhs, 2, 1e-10, 1.0)
    g["E_sol"], g["E_hist"], g["E_citers"] = sol, hist, citers

    np.savez_compressed(OUT, **g)
    print("wrote", OUT, "(%d arrays)" % len(g))


if __name__ == "__main__":
    main()
