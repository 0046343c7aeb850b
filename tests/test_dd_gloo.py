"""The multi-rank path with real process ranks on the CPU: two gloo ranks, each owning one
subdomain, run the reference's CGS V-cycle with the oracle's level operations.

Each rank takes its subdomain (sizes, meshes with the neighbours' ghost widths on every
level, RBGS colour offsets) from the library's host-only pmg_dd_partition, exchanges its
ghost planes with gloo send/receive where the reference's MPI code does
(src/geometry.f90:621-660), and all-reduces its dot products over the process group
(src/poisson_matrix_operator.f90:68-97).  The gathered solution must equal the oracle's
one-rank solution bit for bit.
"""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

N, NL, TOL, MAXIT, OMEGA = 24, 2, 1e-10, 2, 1.0


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _problem():
    from peps_mg_gb300 import geometry as G
    mesh = [G.stretched_axis(N, 0.0, 1.0, 1.1), G.uniform_axis(N, 0.0, 2.0), G.tanh_axis(N, 0.0, 1.0, 1.3)]
    rng = np.random.Generator(np.random.PCG64(9))
    rhs = G.field(N, N, N)
    rhs[1:-1, 1:-1, 1:-1] = rng.uniform(-1.0, 1.0, size=(N, N, N))
    return mesh, np.asfortranarray(rhs)


def _plane(a, d, idx):
    return a[idx, :, :] if d == 0 else a[:, idx, :] if d == 1 else a[:, :, idx]


def _set_plane(a, d, idx, v):
    if d == 0:
        a[idx, :, :] = v
    elif d == 1:
        a[:, idx, :] = v
    else:
        a[:, :, idx] = v


def _rank(rank, world, port, procs, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import peps_mg_gb300 as pmg
        from oracle import oracle as O
        mesh, grhs = _problem()
        co = (rank % procs[0], (rank // procs[0]) % procs[1], rank // (procs[0] * procs[1]))

        def rank_of(c):
            return c[0] + procs[0] * (c[1] + procs[1] * c[2])

        lv = [pmg.dd_partition(mesh, procs, co, l, NL) for l in range(NL + 1)]
        dims = [v[0] for v in lv]
        meshes = [[tuple(np.asfortranarray(a) for a in ax) for ax in v[1]] for v in lv]
        offs = [v[2] for v in lv]
        coeff = [O.matrix_create(meshes[l]) for l in range(NL + 1)]
        lvc = [max([l for l in range(1, NL + 1) if 2 * dims[l][d] == dims[l - 1][d]] + [0]) for d in range(3)]
        n0 = dims[0]
        o = [co[d] * n0[d] for d in range(3)]
        rhs = np.asfortranarray(grhs[o[0]:o[0] + n0[0] + 2, o[1]:o[1] + n0[1] + 2, o[2]:o[2] + n0[2] + 2])
        x = [O.field(*dims[l]) for l in range(NL + 1)]        # x[0] is sol
        b = [rhs] + [O.field(*dims[l]) for l in range(1, NL + 1)]
        r = [O.field(*dims[l]) for l in range(NL + 1)]          # r[0] is rsd

        def halo(a):
            n = a.shape
            for d in range(3):
                if procs[d] == 1:
                    continue
                reqs, recv = [], {}
                for side, step in (("east", 1), ("west", -1)):
                    c = list(co)
                    c[d] += step
                    if not 0 <= c[d] < procs[d]:
                        continue
                    peer = rank_of(c)
                    send = np.ascontiguousarray(_plane(a, d, n[d] - 2 if step == 1 else 1))
                    recv[side] = torch.empty(send.shape, dtype=torch.float64)
                    reqs.append(dist.isend(torch.from_numpy(send), peer, tag=d))
                    reqs.append(dist.irecv(recv[side], peer, tag=d))
                for q in reqs:
                    q.wait()
                if "east" in recv:
                    _set_plane(a, d, n[d] - 1, recv["east"].numpy())
                if "west" in recv:
                    _set_plane(a, d, 0, recv["west"].numpy())

        def dot(u, v):
            t = torch.tensor([O.vv_dot(u, v)], dtype=torch.float64)
            dist.all_reduce(t)
            return float(t.item())

        def rbgs(l, iters):
            for _ in range(iters):
                for c in (0, 1):
                    halo(x[l])
                    O.rbgs_colour(coeff[l], x[l], b[l], OMEGA, c, offs[l])

        def residual(l):
            halo(x[l])
            r[l][...] = O.residual(coeff[l], x[l], b[l])

        residual(0)
        res0 = dot(r[0], r[0])
        cycles = 0
        for cyc in range(1, 61):
            rbgs(0, MAXIT)
            residual(0)
            O.restriction(meshes[1], meshes[0], 0, lvc, r[0], b[1])
            for l in range(1, NL):
                x[l][...] = 0.0
                rbgs(l, MAXIT)
                residual(l)
                O.restriction(meshes[l + 1], meshes[l], l, lvc, r[l], b[l + 1])
            x[NL][...] = 0.0
            residual(NL)
            r0 = dot(r[NL], r[NL])
            for _ in range(1000):
                rbgs(NL, 1)
                residual(NL)
                if np.sqrt(dot(r[NL], r[NL]) / r0) <= TOL:
                    break
            residual(NL)
            for l in range(NL - 1, 0, -1):
                O.prolongation(meshes[l + 1], meshes[l], l, lvc, x[l + 1], r[l])
                x[l] += r[l]
                rbgs(l, MAXIT)
                halo(x[l])
            O.prolongation(meshes[1], meshes[0], 0, lvc, x[1], r[0])
            x[0] += r[0]
            rbgs(0, MAXIT)
            residual(0)
            cycles = cyc
            if np.sqrt(dot(r[0], r[0]) / res0) < TOL:
                break
        interior = torch.from_numpy(np.ascontiguousarray(x[0][1:-1, 1:-1, 1:-1]))
        parts = [torch.empty_like(interior) for _ in range(world)] if rank == 0 else None
        dist.gather(interior, parts, dst=0)
        if rank == 0:
            g = O.field(N, N, N)
            for q in range(world):
                cq = (q % procs[0], (q // procs[0]) % procs[1], q // (procs[0] * procs[1]))
                oq = [cq[d] * n0[d] for d in range(3)]
                g[oq[0] + 1:oq[0] + 1 + n0[0], oq[1] + 1:oq[1] + 1 + n0[1], oq[2] + 1:oq[2] + 1 + n0[2]] = parts[q].numpy()
            one = O.OracleMG(mesh, NL, 60, 0)
            s1, r1 = O.field(N, N, N), O.field(N, N, N)
            c1, _, _ = one.solve(s1, r1, grhs, MAXIT, TOL, OMEGA)
            out.put((cycles, c1, bool(np.array_equal(g, s1)), float(np.abs(g - s1).max()), offs))
        else:
            out.put(None)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("procs", [(2, 1, 1), (1, 1, 2)])
def test_two_gloo_ranks_equal_one_rank(procs):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, procs, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = [q.get(timeout=300) for _ in ps]
    for p in ps:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = [v for v in res if v is not None]
    assert len(res) == 1
    cycles, c1, equal, diff, offs = res[0]
    assert cycles == c1
    assert equal, diff
