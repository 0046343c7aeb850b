"""Independent vectorised numpy restatement of the PEPS_MG V-cycle hot path.

Test infrastructure.  It is written separately from the C oracle (oracle/pmg_oracle.c)
and is used to cross-check it bit for bit and to generate the committed golden
fixtures (tests/golden/make_golden.py).  Element-wise numpy ufuncs round every
operation, so keeping the reference's association order reproduces the reference's
non-FMA arithmetic exactly.  Reductions use ``np.add.accumulate`` (a sequential
left-to-right sum, i.e. the reference's loop order with one OpenMP thread).

Arrays: float64, shape (nx+2, ny+2, nz+2), index [i, j, k] = Fortran x(i, j, k).
References are to the reference project's files.
"""
import numpy as np


def seq_sum(v):
    """Left-to-right sum starting from 0.0 (Fortran DO-loop accumulation)."""
    v = np.ravel(v, order="F")
    if v.size == 0:
        return 0.0
    return float(np.add.accumulate(v)[-1])


# --- mesh ------------------------------------------------------------------------

def mesh_uniform(n, o, length):
    """src/geometry.f90:180-189"""
    dm = np.zeros(n + 2); dg = np.zeros(n + 2); xg = np.zeros(n + 2)
    xg[0] = o
    h = length / float(n)
    for i in range(1, n + 1):
        dm[i] = h
        dg[i] = 0.5 * (dm[i] + dm[i - 1])
        xg[i] = xg[i - 1] + dg[i]
    dg[n + 1] = 0.5 * (dm[n + 1] + dm[n])
    xg[n + 1] = xg[n] + dg[n + 1]
    return dm, dg, xg


def mesh_from_widths(widths, o):
    """A mesh from interior cell widths, ghosts of zero width (the reference's form)."""
    n = len(widths)
    dm = np.zeros(n + 2); dg = np.zeros(n + 2); xg = np.zeros(n + 2)
    dm[1:n + 1] = widths
    xg[0] = o
    for i in range(1, n + 1):
        dg[i] = 0.5 * (dm[i] + dm[i - 1])
        xg[i] = xg[i - 1] + dg[i]
    dg[n + 1] = 0.5 * (dm[n + 1] + dm[n])
    xg[n + 1] = xg[n] + dg[n + 1]
    return dm, dg, xg


# --- operator --------------------------------------------------------------------

def axis_coeffs(dm, dg):
    """1/(dm*dg) and 1/(dm*dg(+1)) for the interior cells (src/matrix.f90:67-77)."""
    cm = 1.0 / (dm[1:-1] * dg[1:-1])
    cp = 1.0 / (dm[1:-1] * dg[2:])
    return cm, cp


def coeff_fields(mesh):
    """The seven coefficient fields c[0..6] of shape (nx, ny, nz) (src/matrix.f90:82-88)."""
    (dxm, dxg, _), (dym, dyg, _), (dzm, dzg, _) = mesh
    cxm, cxp = axis_coeffs(dxm, dxg)
    cym, cyp = axis_coeffs(dym, dyg)
    czm, czp = axis_coeffs(dzm, dzg)
    nx, ny, nz = len(cxm), len(cym), len(czm)
    X = lambda a: np.broadcast_to(a[:, None, None], (nx, ny, nz))
    Y = lambda a: np.broadcast_to(a[None, :, None], (nx, ny, nz))
    Z = lambda a: np.broadcast_to(a[None, None, :], (nx, ny, nz))
    s = X(cxm) + X(cxp)
    s = s + Y(cym)
    s = s + Y(cyp)
    s = s + Z(czm)
    s = s + Z(czp)
    return [-s, X(cxm).copy(), X(cxp).copy(), Y(cym).copy(), Y(cyp).copy(), Z(czm).copy(), Z(czp).copy()]


def _nb(x):
    """Neighbour views of the interior: centre, i-1, i+1, j-1, j+1, k-1, k+1."""
    return (x[1:-1, 1:-1, 1:-1], x[:-2, 1:-1, 1:-1], x[2:, 1:-1, 1:-1], x[1:-1, :-2, 1:-1],
            x[1:-1, 2:, 1:-1], x[1:-1, 1:-1, :-2], x[1:-1, 1:-1, 2:])


def mv_mul(c, x):
    """src/poisson_matrix_operator.f90:136-159"""
    y = np.zeros_like(x)
    n = _nb(x)
    t = c[0] * n[0]
    for q in range(1, 7):
        t = t + c[q] * n[q]
    y[1:-1, 1:-1, 1:-1] = t
    return y


def residual(c, x, b):
    """src/multigrid.f90:1795-1805"""
    r = mv_mul(c, x)
    r[1:-1, 1:-1, 1:-1] = b[1:-1, 1:-1, 1:-1] - r[1:-1, 1:-1, 1:-1]
    return r


def vv_dot(x, y):
    """src/poisson_matrix_operator.f90:58-65"""
    return seq_sum(x[1:-1, 1:-1, 1:-1] * y[1:-1, 1:-1, 1:-1])


def colour_mask(shape, colour):
    """Cells updated by the first (colour 0) or second (colour 1) half-sweep:
    i starts at 1 + mod(j+k+colour, 2) (src/rbgs_poisson_matrix.f90:242,260), i.e.
    (i + j + k + colour) odd for 1-based indices."""
    nx, ny, nz = shape
    i = np.arange(1, nx + 1)[:, None, None]
    j = np.arange(1, ny + 1)[None, :, None]
    k = np.arange(1, nz + 1)[None, None, :]
    return ((i + j + k + colour) % 2) == 1


def rbgs_half(c, x, b, omega, colour):
    n = _nb(x)
    t = c[1] * n[1]
    for q in range(2, 7):
        t = t + c[q] * n[q]
    new = omega * (b[1:-1, 1:-1, 1:-1] - t) / c[0] + (1.0 - omega) * n[0]
    m = colour_mask(n[0].shape, colour)
    inner = x[1:-1, 1:-1, 1:-1]
    inner[m] = new[m]


def rbgs_iterator(c, x, b, maxiteration, omega):
    """src/rbgs_poisson_matrix.f90:235-273 (in place)."""
    for _ in range(maxiteration):
        rbgs_half(c, x, b, omega, 0)
        rbgs_half(c, x, b, omega, 1)


def rbgs_solver(c, x, b, maxiteration, tolerance, omega):
    """src/rbgs_poisson_matrix.f90:69-171 (in place); returns the iteration counter."""
    r = residual(c, x, b)
    r0 = vv_dot(r, r)
    it = 0
    for it in range(maxiteration):
        rbgs_half(c, x, b, omega, 0)
        rbgs_half(c, x, b, omega, 1)
        r = residual(c, x, b)
        rn = vv_dot(r, r)
        if np.sqrt(rn / r0) <= tolerance:
            return it
    return maxiteration


def cg_solver(c, x, b, maxiteration, tolerance, check=True):
    """src/cg_poisson_matrix.f90:80-138 (in place); returns the iteration counter."""
    ax = mv_mul(c, x)
    r = np.zeros_like(x); p = np.zeros_like(x)
    r[1:-1, 1:-1, 1:-1] = b[1:-1, 1:-1, 1:-1] - ax[1:-1, 1:-1, 1:-1]
    p[1:-1, 1:-1, 1:-1] = r[1:-1, 1:-1, 1:-1]
    r0 = vv_dot(r, r) if check else 0.0
    for it in range(maxiteration):
        t1 = vv_dot(r, r)
        ap = mv_mul(c, p)
        t2 = vv_dot(ap, p)
        alpha = t1 / t2
        x[1:-1, 1:-1, 1:-1] = x[1:-1, 1:-1, 1:-1] + alpha * p[1:-1, 1:-1, 1:-1]
        r[1:-1, 1:-1, 1:-1] = r[1:-1, 1:-1, 1:-1] - alpha * ap[1:-1, 1:-1, 1:-1]
        t2 = vv_dot(r, r)
        if check and np.sqrt(t2 / r0) < tolerance:
            return it
        beta = t2 / t1
        p[1:-1, 1:-1, 1:-1] = r[1:-1, 1:-1, 1:-1] + beta * p[1:-1, 1:-1, 1:-1]
    return maxiteration


# --- hierarchy -------------------------------------------------------------------

def level_sizes(n, n_levels, method, cga_level=0):
    """One-rank level sizes and last halving level per axis; raises ValueError where
    the reference stops with an error (src/multigrid.f90:101-107, 190-195, 302-309,
    530-553, 593-601, 732-740, 1193-1201)."""
    if n_levels <= 1:
        raise ValueError("n_levels must exceed 1")
    n = list(n)
    sizes = [tuple(n)]
    lvc = [0, 0, 0]
    if method == 0 and cga_level != 0:
        raise ValueError("CGS needs aggregation level 0")
    if method == 1 and cga_level == 0:
        raise ValueError("CGA needs aggregation level > 0")
    if method not in (0, 1, 2):
        raise ValueError("method")
    for l in range(1, n_levels + 1):
        new = []
        for d in range(3):
            if method == 1 and l <= cga_level:
                if n[d] % 2:
                    raise ValueError("odd size at or before the CGA level")
                new.append(n[d] // 2)
                if l == cga_level:
                    lvc[d] = l
            elif n[d] % 2 == 0:
                new.append(n[d] // 2)
                lvc[d] = l
            else:
                new.append(n[d])
        n = new
        sizes.append(tuple(n))
        if method in (1, 2) and (n[0] * n[1] * n[2]) % 2 == 1 and l < n_levels:
            break
    if method == 2:
        if n_levels != max(lvc):
            raise ValueError("CGPSA needs n_levels equal to the coarsest level")
    elif n_levels > max(lvc):
        raise ValueError("n_levels beyond the coarsest level")
    return sizes, lvc


def coarsen_mesh(mesh_f, nc, lv, lvc):
    """dxm/dxg of a coarse level (src/multigrid.f90:450-491); xg is not needed by the
    operator and is not restated here."""
    dm_f, dg_f, _ = mesh_f
    if lv > lvc:
        return dm_f.copy(), dg_f.copy(), None
    dm = np.zeros(nc + 2); dg = np.zeros(nc + 2)
    dm[1:nc + 1] = dm_f[1:2 * nc:2] + dm_f[2:2 * nc + 1:2]
    dm[0] = dm_f[0]
    dm[nc + 1] = dm_f[2 * nc + 1]
    dg[1:nc + 2] = 0.5 * (dm[1:nc + 2] + dm[0:nc + 1])
    return dm, dg, None


def restriction(dm_c, dm_f, nf, stride1, val_f, nc):
    """src/multigrid.f90:1366-1494.  dm_c/dm_f/nf/nc/stride1 are 3-tuples per axis."""
    dfs, idx = [], []
    for d in range(3):
        if stride1[d]:
            df = dm_f[d].copy()
            ip = np.arange(1, nc[d] + 1); iz = ip
        else:
            df = np.zeros(nf[d] + 2)
            i = np.arange(1, nf[d] + 1)
            df[1:nf[d] + 1] = dm_c[d][(i - 1) // 2 + 1] - dm_f[d][i]
            ip = 2 * np.arange(1, nc[d] + 1); iz = ip - 1
        dfs.append(df); idx.append((iz, ip))
    (iz, ip), (jz, jp), (kz, kp) = idx
    dxf, dyf, dzf = dfs
    X = lambda a: a[:, None, None]
    Y = lambda a: a[None, :, None]
    Z = lambda a: a[None, None, :]
    v111 = X(dxf[iz]) * Y(dyf[jz]) * Z(dzf[kz])
    v211 = X(dxf[ip]) * Y(dyf[jz]) * Z(dzf[kz])
    v121 = X(dxf[iz]) * Y(dyf[jp]) * Z(dzf[kz])
    v221 = X(dxf[ip]) * Y(dyf[jp]) * Z(dzf[kz])
    v112 = X(dxf[iz]) * Y(dyf[jz]) * Z(dzf[kp])
    v212 = X(dxf[ip]) * Y(dyf[jz]) * Z(dzf[kp])
    v122 = X(dxf[iz]) * Y(dyf[jp]) * Z(dzf[kp])
    v222 = X(dxf[ip]) * Y(dyf[jp]) * Z(dzf[kp])
    vols = [v111, v211, v121, v221, v112, v212, v122, v222]
    vol = vols[0]
    for v in vols[1:]:
        vol = vol + v
    F = lambda a, b, c: val_f[np.ix_(a, b, c)]
    terms = [F(ip, jp, kp), F(iz, jp, kp), F(ip, jz, kp), F(iz, jz, kp),
             F(ip, jp, kz), F(iz, jp, kz), F(ip, jz, kz), F(iz, jz, kz)]
    s = vols[0] * terms[0]
    for v, t in zip(vols[1:], terms[1:]):
        s = s + v * t
    out = np.zeros((nc[0] + 2, nc[1] + 2, nc[2] + 2))
    out[1:-1, 1:-1, 1:-1] = s / vol
    return out


def _pweights(dm_c, dm_f, nc, nf, stride1):
    dp = np.zeros(nf + 2); dn = np.zeros(nf + 2)
    if stride1:
        dp[:] = dm_c; dn[:] = dm_c
    else:
        i = np.arange(1, nc + 1); f = 2 * i
        dp[f - 1] = 1.0 * dm_f[f - 2] + 0.5 * dm_f[f - 1]
        dp[f] = 0.5 * dm_f[f - 1]
        dn[f - 1] = 0.5 * dm_f[f]
        dn[f] = 1.0 * dm_f[f + 1] + 0.5 * dm_f[f]
    return dp, dn


def prolongation(dm_c, dm_f, nf, stride1, val_c, nc, val_f):
    """src/multigrid.f90:1594-1758: writes the children of every coarse cell into
    val_f (in place), in the reference's write order."""
    W, I = [], []
    for d in range(3):
        W.append(_pweights(dm_c[d], dm_f[d], nc[d], nf[d], stride1[d]))
        c = np.arange(1, nc[d] + 1)
        if stride1[d]:
            I.append((c, c, c, c, c))              # z_f, p_f, m_c, p_c, centre
        else:
            I.append((2 * c - 1, 2 * c, c - 1, c + 1, c))
    (xp, xn), (yp, yn), (zp, zn) = W
    (iz, ip, im, iq, ic), (jz, jp, jm, jq, jc), (kz, kp, km, kq, kc) = I
    X = lambda a: a[:, None, None]
    Y = lambda a: a[None, :, None]
    Z = lambda a: a[None, None, :]
    V = lambda a, b, c: val_c[np.ix_(a, b, c)]

    def child(wx, wy, wz, xs, ys, zs):
        # wx = (weight at own-side index, weight at other-side index) for x, etc.
        # xs = (centre index, neighbour index) of the coarse cell in x, etc.
        ax, bx = wx; ay, by = wy; az, bz = wz
        cx, nx_ = xs; cy, ny_ = ys; cz, nz_ = zs
        t = X(ax) * Y(ay) * Z(az) * V(cx, cy, cz)
        t = t + X(bx) * Y(ay) * Z(az) * V(nx_, cy, cz)
        t = t + X(ax) * Y(by) * Z(az) * V(cx, ny_, cz)
        t = t + X(ax) * Y(ay) * Z(bz) * V(cx, cy, nz_)
        t = t + X(bx) * Y(by) * Z(az) * V(nx_, ny_, cz)
        t = t + X(bx) * Y(ay) * Z(bz) * V(nx_, cy, nz_)
        t = t + X(ax) * Y(by) * Z(bz) * V(cx, ny_, nz_)
        t = t + X(bx) * Y(by) * Z(bz) * V(nx_, ny_, nz_)
        return t / (X(ax + bx) * Y(ay + by) * Z(az + bz))

    # low child: weights (p(z_f), p(p_f)), neighbour m_c; high child: (n(p_f), n(z_f)), neighbour p_c
    lox = ((xp[iz], xp[ip]), (ic, im)); hix = ((xn[ip], xn[iz]), (ic, iq))
    loy = ((yp[jz], yp[jp]), (jc, jm)); hiy = ((yn[jp], yn[jz]), (jc, jq))
    loz = ((zp[kz], zp[kp]), (kc, km)); hiz = ((zn[kp], zn[kz]), (kc, kq))
    order = [((lox, iz), (loy, jz), (loz, kz)), ((hix, ip), (loy, jz), (loz, kz)),
             ((lox, iz), (hiy, jp), (loz, kz)), ((hix, ip), (hiy, jp), (loz, kz)),
             ((lox, iz), (loy, jz), (hiz, kp)), ((hix, ip), (loy, jz), (hiz, kp)),
             ((lox, iz), (hiy, jp), (hiz, kp)), ((hix, ip), (hiy, jp), (hiz, kp))]
    for (xw, xi), (yw, yi), (zw, zi) in order:
        val_f[np.ix_(xi, yi, zi)] = child(xw[0], yw[0], zw[0], xw[1], yw[1], zw[1])
    return val_f


class NumpyMG:
    """One-rank multigrid_create + multigrid_solve_vcycle restated in numpy."""

    def __init__(self, mesh, n_levels, n_vcycles, method=0, cga_level=0, coarse_solver=0):
        n = tuple(len(m[0]) - 2 for m in mesh)
        self.sizes, self.lvc = level_sizes(n, n_levels, method, cga_level)
        self.n_levels = n_levels
        self.n_vcycles = n_vcycles
        self.coarse_solver = coarse_solver
        self.meshes = [tuple(mesh)]
        for l in range(1, n_levels + 1):
            self.meshes.append(tuple(coarsen_mesh(self.meshes[l - 1][d], self.sizes[l][d], l, self.lvc[d])
                                     for d in range(3)))
        self.coeffs = [coeff_fields(m) for m in self.meshes]
        self.x = [None] + [np.zeros(tuple(s + 2 for s in self.sizes[l])) for l in range(1, n_levels + 1)]
        self.b = [None] + [np.zeros_like(self.x[l]) for l in range(1, n_levels + 1)]
        self.r = [None] + [np.zeros_like(self.x[l]) for l in range(1, n_levels + 1)]

    def _restrict(self, l, val_f):
        dm_c = [self.meshes[l + 1][d][0] for d in range(3)]
        dm_f = [self.meshes[l][d][0] for d in range(3)]
        s1 = [l >= self.lvc[d] for d in range(3)]
        return restriction(dm_c, dm_f, self.sizes[l], s1, val_f, self.sizes[l + 1])

    def _prolong(self, l, val_c, val_f):
        dm_c = [self.meshes[l + 1][d][0] for d in range(3)]
        dm_f = [self.meshes[l][d][0] for d in range(3)]
        s1 = [l >= self.lvc[d] for d in range(3)]
        prolongation(dm_c, dm_f, self.sizes[l], s1, val_c, self.sizes[l + 1], val_f)

    def solve(self, sol, rsd, rhs, maxiteration, tolerance, omega):
        c0 = self.coeffs[0]
        nl = self.n_levels
        rsd[...] = residual(c0, sol, rhs)
        res0 = vv_dot(rsd, rsd)
        hist, citers = [], []
        for _cyc in range(self.n_vcycles):
            rbgs_iterator(c0, sol, rhs, maxiteration, omega)
            rsd[...] = residual(c0, sol, rhs)
            self.b[1] = self._restrict(0, rsd)
            for l in range(1, nl):
                self.x[l][...] = 0.0
                rbgs_iterator(self.coeffs[l], self.x[l], self.b[l], maxiteration, omega)
                self.r[l] = residual(self.coeffs[l], self.x[l], self.b[l])
                self.b[l + 1] = self._restrict(l, self.r[l])
            xc = self.x[nl]
            xc[...] = 0.0
            if xc[1:-1, 1:-1, 1:-1].size == 1:
                xc[1, 1, 1] = self.b[nl][1, 1, 1] / self.coeffs[nl][0][0, 0, 0]
                citers.append(0)
            elif self.coarse_solver == 1:
                citers.append(cg_solver(self.coeffs[nl], xc, self.b[nl], 1000, tolerance))
            else:
                citers.append(rbgs_solver(self.coeffs[nl], xc, self.b[nl], 1000, tolerance, omega))
            for l in range(nl - 1, 0, -1):
                self._prolong(l, self.x[l + 1], self.r[l])
                self.x[l] = self.x[l] + self.r[l]
                rbgs_iterator(self.coeffs[l], self.x[l], self.b[l], maxiteration, omega)
            self._prolong(0, self.x[1], rsd)
            sol[...] = sol + rsd
            rbgs_iterator(c0, sol, rhs, maxiteration, omega)
            rsd[...] = residual(c0, sol, rhs)
            rv = vv_dot(rsd, rsd)
            hist.append((np.sqrt(rv), np.sqrt(res0), np.sqrt(rv / res0)))
            if np.sqrt(rv / res0) < tolerance:
                break
        return len(hist), np.array(hist), np.array(citers)
