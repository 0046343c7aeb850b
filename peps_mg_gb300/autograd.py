"""torch.autograd binding of the solve and its hand-written adjoint.

    u = PoissonSolve.apply(b, g, mg, maxiteration, tolerance, omega)

solves A u = b on the interior with the six Dirichlet face values g (x-, x+, y-, y+,
z-, z+; each face's ghost layer holds one scalar) using the context `mg` (a
`Multigrid`), and returns the full (nz+2, ny+2, nx+2) array (ghosts = the face values).
The backward pass calls the library's adjoint (pmg_adjoint): dL/db = A^{-T} dL/du,
dL/dg_f = -sum_face c_f (A^{-T} dL/du) plus the direct dependence of the returned ghost
entries on g.  Only the finest-level state is kept between forward and backward.
"""
import torch

FACES = ("x-", "x+", "y-", "y+", "z-", "z+")


def set_faces(sol, g):
    """Write the six face values into the ghost layers (later faces own shared edges)."""
    sol[:, :, 0] = g[0]
    sol[:, :, -1] = g[1]
    sol[:, 0, :] = g[2]
    sol[:, -1, :] = g[3]
    sol[0] = g[4]
    sol[-1] = g[5]


def face_sums(a):
    """Sum of a over the ghost entries each face owns under set_faces."""
    return torch.stack([a[1:-1, 1:-1, 0].sum(), a[1:-1, 1:-1, -1].sum(), a[1:-1, 0, :].sum(),
                        a[1:-1, -1, :].sum(), a[0].sum(), a[-1].sum()])


class PoissonSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, b, g, mg, maxiteration, tolerance, omega):
        b = b.contiguous()
        sol = torch.zeros_like(b)
        set_faces(sol, [float(v) for v in g.detach().cpu()])
        rsd = torch.zeros_like(b)
        ctx.report = mg.solve_vcycle(sol, rsd, b, maxiteration, tolerance, omega)
        ctx.mg = mg
        ctx.params = (maxiteration, tolerance, omega)
        ctx.g_dtype = g.dtype
        ctx.g_device = g.device
        return sol

    @staticmethod
    def backward(ctx, gu):
        gu = gu.contiguous()
        dldb = torch.empty_like(gu)
        _, dldg = ctx.mg.adjoint(gu, dldb, *ctx.params)
        dg = torch.as_tensor(dldg, dtype=ctx.g_dtype, device=gu.device) + face_sums(gu).to(ctx.g_dtype)
        return dldb, dg.to(ctx.g_device), None, None, None, None
