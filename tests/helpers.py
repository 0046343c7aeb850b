"""Shared test helpers: host <-> device grid arrays and seeded problems."""
import numpy as np

from peps_mg_gb300 import geometry as G


def to_dev(a):
    """Fortran-ordered numpy (nx+2, ny+2, nz+2) -> CUDA tensor with the same memory layout."""
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.asfortranarray(a).T)).cuda()


def from_dev(t):
    """CUDA tensor -> Fortran-ordered numpy (nx+2, ny+2, nz+2)."""
    return np.asfortranarray(t.detach().cpu().numpy().T)


def mesh_of(g, p):
    return [(g[p + "d%sm" % a], g[p + "d%sg" % a], g[p + "%sg" % a]) for a in "xyz"]


def sine_problem(n):
    """The unit-cube benchmark problem: b = -3 pi^2 sin(pi x) sin(pi y) sin(pi z) at cell
    centres, zero Dirichlet ghosts; returns (mesh, rhs, exact u)."""
    ax = G.uniform_axis(n, 0.0, 1.0)
    xc = ax[2][1:-1]
    X, Y, Z = np.meshgrid(xc, xc, xc, indexing="ij")
    u = np.sin(np.pi * X) * np.sin(np.pi * Y) * np.sin(np.pi * Z)
    rhs = G.field(n, n, n)
    rhs[1:-1, 1:-1, 1:-1] = -3.0 * np.pi ** 2 * u
    return [ax, ax, ax], rhs, u


def tanh_z_problem(n, seed=2, beta=1.5):
    """Uniform in x and y, tanh-clustered in z, rhs i.i.d. U[-1,1] (PCG64(seed))."""
    ax = G.uniform_axis(n, 0.0, 1.0)
    az = G.tanh_axis(n, 0.0, 1.0, beta)
    rng = np.random.Generator(np.random.PCG64(seed))
    rhs = G.field(n, n, n)
    rhs[1:-1, 1:-1, 1:-1] = rng.uniform(-1.0, 1.0, size=(n, n, n)).transpose(2, 1, 0).T
    return [ax, ax, az], rhs


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.max(np.abs(a - b))
    s = np.max(np.abs(b))
    return d / s if s > 0 else d
