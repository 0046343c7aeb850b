"""Cell-centred meshes in the reference's form (host-side setup).

A mesh along one axis is the triple (dm, dg, xg) of length n+2, indexed 0..n+1 as the
subdomain type of src/geometry.f90:59-118: dm = cell widths with zero-width boundary
ghosts (so a ghost centre lies on the face and the Dirichlet value sits in the ghost
cell), dg(i) = (dm(i) + dm(i-1)) / 2, xg = cell centres.
"""
import numpy as np


def mesh_from_widths(widths, origin=0.0):
    """Mesh from interior cell widths (ghost widths zero), src/geometry.f90:194-208."""
    w = np.asarray(widths, dtype=np.float64)
    n = w.size
    dm = np.zeros(n + 2)
    dg = np.zeros(n + 2)
    xg = np.zeros(n + 2)
    dm[1:n + 1] = w
    xg[0] = origin
    for i in range(1, n + 1):
        dg[i] = 0.5 * (dm[i] + dm[i - 1])
        xg[i] = xg[i - 1] + dg[i]
    dg[n + 1] = 0.5 * (dm[n + 1] + dm[n])
    xg[n + 1] = xg[n] + dg[n + 1]
    return dm, dg, xg


def uniform_axis(n, origin, length):
    """Uniform mesh, src/geometry.f90:180-189 (dm = length / n)."""
    return mesh_from_widths(np.full(n, length / float(n)), origin)


def _ipow(a, n):
    r, b, e = 1.0, a, n
    while e > 0:
        if e & 1:
            r = r * b
        e >>= 1
        if e:
            b = b * b
    return r


def stretched_axis(n, origin, length, ratio):
    """Symmetric geometric stretch with ratio `ratio`, src/geometry.f90:190-209
    (ratio 1.0 gives the uniform mesh, as in the reference)."""
    if ratio == 1.0:
        return uniform_axis(n, origin, length)
    dm = np.zeros(n + 2)
    dm[1] = 0.5 * length * (ratio - 1.0) / (_ipow(ratio, n // 2) - 1.0)
    for i in range(2, n // 2 + 1):
        dm[i] = dm[i - 1] * ratio
        dm[n - i + 1] = dm[i]
    dm[n] = dm[1]
    return mesh_from_widths(dm[1:n + 1], origin)


def tanh_axis(n, origin, length, beta):
    """Mesh clustered at both ends by tanh: faces z_k = L/2 (1 + tanh(beta(2k/n - 1)) / tanh(beta))."""
    k = np.arange(n + 1, dtype=np.float64)
    faces = 0.5 * length * (1.0 + np.tanh(beta * (2.0 * k / n - 1.0)) / np.tanh(beta))
    return mesh_from_widths(np.diff(faces), origin)


def field(nx, ny, nz, fill=0.0):
    """A host grid array in the library's layout: numpy float64 of shape
    (nx+2, ny+2, nz+2) in Fortran order (i fastest)."""
    return np.full((nx + 2, ny + 2, nz + 2), fill, dtype=np.float64, order="F")
