"""Seeded synthetic problems of the benchmark configurations (host numpy setup).

All right-hand sides are returned as Fortran-ordered (nx+2, ny+2, nz+2) float64
arrays with zero ghost cells (homogeneous Dirichlet boundary values), together with
the mesh as three (dm, dg, xg) triples.

* sine(n)            unit cube, b = -3 pi^2 sin(pi x) sin(pi y) sin(pi z) at cell
                     centres, exact u = sin sin sin (the 64^3 plain FP64 case)
* tanh_z(n, seed)    uniform in x, y; z clustered by tanh (beta 1.5); b ~ U[-1,1]
                     from PCG64(seed) (the 256^3 CGA / CGPSA case)
* gaussian_blobs(n)  unit cube, sum of 8 Gaussians (sigma 0.05, centres U[0.1,0.9]^3,
                     amplitudes U[-10,10]) plus 1e-3 U[-1,1] noise, PCG64(3) (the 512^3
                     mixed-precision case)
* batch_dims(count)  the batched case: `count` problems, each axis size drawn from
                     {32, 48, 64, 96, 128, 192} by PCG64(4); batch_rhs fills a packed
                     right-hand side with U[-1,1] (PCG64(seed + 100)) problem by problem
"""
import numpy as np

from . import geometry as G


def _interior(shape_xyz, values_kji):
    nx, ny, nz = shape_xyz
    b = G.field(nx, ny, nz)
    b[1:-1, 1:-1, 1:-1] = values_kji.transpose(2, 1, 0)
    return b


def sine(n):
    ax = G.uniform_axis(n, 0.0, 1.0)
    xc = ax[2][1:-1]
    s = np.sin(np.pi * xc)
    u = s[None, None, :] * s[None, :, None] * s[:, None, None]       # (k, j, i)
    b = _interior((n, n, n), -3.0 * np.pi ** 2 * u)
    return [ax, ax, ax], b, u.transpose(2, 1, 0)


def tanh_z(n, seed=2, beta=1.5):
    ax = G.uniform_axis(n, 0.0, 1.0)
    az = G.tanh_axis(n, 0.0, 1.0, beta)
    rng = np.random.Generator(np.random.PCG64(seed))
    vals = rng.uniform(-1.0, 1.0, size=(n, n, n))                     # (k, j, i)
    return [ax, ax, az], _interior((n, n, n), vals)


def gaussian_blobs(n, seed=3, blobs=8, sigma=0.05, noise=1e-3):
    ax = G.uniform_axis(n, 0.0, 1.0)
    xc = ax[2][1:-1]
    rng = np.random.Generator(np.random.PCG64(seed))
    centres = rng.uniform(0.1, 0.9, size=(blobs, 3))
    amps = rng.uniform(-10.0, 10.0, size=blobs)
    vals = noise * rng.uniform(-1.0, 1.0, size=(n, n, n))             # (k, j, i)
    inv = 1.0 / (2.0 * sigma * sigma)
    for c, a in zip(centres, amps):
        gx = np.exp(-(xc - c[0]) ** 2 * inv)
        gy = np.exp(-(xc - c[1]) ** 2 * inv)
        gz = np.exp(-(xc - c[2]) ** 2 * inv)
        vals += a * (gz[:, None, None] * (gy[None, :, None] * gx[None, None, :]))
    return [ax, ax, ax], _interior((n, n, n), vals)


BATCH_SIZES = (32, 48, 64, 96, 128, 192)


def batch_dims(count=128, seed=4, sizes=BATCH_SIZES):
    """(count, 3) int array of (nx, ny, nz)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.choice(np.asarray(sizes), size=(count, 3))


def batch_rhs(dims, seed=4):
    """Interior values U[-1,1] per problem, in (k, j, i) order."""
    rng = np.random.Generator(np.random.PCG64(seed + 100))
    return [rng.uniform(-1.0, 1.0, size=(int(d[2]), int(d[1]), int(d[0]))) for d in dims]
