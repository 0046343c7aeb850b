"""Drop-in for the reference's driver program (src/main_peps.f90) on one GPU.

    python -m peps_mg_gb300.driver [PARA_INPUT.inp] [--precision fp64|mixed]
                                   [--coarse rbgs|cg] [--write DIR]

reads the namelist file of the reference (&meshes, &origin, &length, &mesh_stretch,
&procs, &control, &coefficients; src/main_peps.f90:44-60), builds the global mesh
(uniform, or the reference's symmetric geometric stretch when a stretch ratio is not 1;
src/geometry.f90:177-280), sets up the reference's test problem (problem 1: b = -cos cos
cos * pi^2 (1/lx^2 + 1/ly^2 + 1/lz^2), exact u = cos(x pi/lx) cos(y pi/ly) cos(z pi/lz),
zero initial guess and ghost cells; src/main_peps.f90:79-90), solves it with the
V-cycle of &control on the GPU, and prints the reference's log lines: the [MG] cycle
lines, the RMS error against the exact solution (sum of squares / (nx ny nz),
src/main_peps.f90:172-181) and the execution time.  With --write it also writes the
reference's solution files into DIR (solution_all.dat, solution_all.bin,
solution_all_MPI_IO.bin; src/main_peps.f90:204-446, which the reference itself leaves
switched off).

One GPU solves the whole domain: &procs is reported and otherwise ignored (the reference
with npx = npy = npz = 1 runs the same arithmetic); &coefficients is read and, as in the
reference, not used.
"""
import argparse
import math
import os
import sys
import time

import numpy as np

from . import geometry as G
from . import io as pio

_METHODS = {0: "cgs", 1: "cga", 2: "cgpsa"}


def domain_mesh(n, origin, length, ratio):
    """One axis of the global domain (src/geometry.f90:177-209)."""
    return G.stretched_axis(int(n), float(origin), float(length), float(ratio))


def cosine_problem(mesh, lengths):
    """Right-hand side (field with zero ghosts) and exact solution (interior) of problem 1
    (src/main_peps.f90:79-90)."""
    (lx, ly, lz) = lengths
    xc, yc, zc = (m[2][1:-1] for m in mesh)
    cx, cy, cz = np.cos(xc / lx * math.pi), np.cos(yc / ly * math.pi), np.cos(zc / lz * math.pi)
    ref = cx[:, None, None] * cy[None, :, None] * cz[None, None, :]
    k2 = math.pi * math.pi * (1.0 / (lx * lx) + 1.0 / (ly * ly) + 1.0 / (lz * lz))
    b = G.field(len(xc), len(yc), len(zc))
    b[1:-1, 1:-1, 1:-1] = -(cx[:, None, None] * cy[None, :, None] * cz[None, None, :]) * k2
    return b, ref


def read_config(path):
    """The namelist groups with the reference's names and defaults checked."""
    nl = pio.read_namelists(path)
    need = {"meshes": ("nx", "ny", "nz"), "origin": ("ox", "oy", "oz"), "length": ("lx", "ly", "lz"),
            "mesh_stretch": ("ax", "ay", "az"),
            "control": ("maxiteration", "tolerance", "number_of_vcycles", "number_of_levels",
                        "aggregation_method", "cga_level", "cgpsa_level", "omega_sor")}
    for g, names in need.items():
        if g not in nl:
            raise ValueError("%s: namelist group &%s is missing" % (path, g))
        for nm in names:
            if nm not in nl[g]:
                raise ValueError("%s: &%s has no %s" % (path, g, nm))
    c = nl["control"]
    cg = c["cgpsa_level"]
    c["cgpsa_level"] = list(cg) if isinstance(cg, list) else [cg, 0, 0]
    if len(c["cgpsa_level"]) != 3:
        raise ValueError("%s: CGPSA_level needs three values" % path)
    if c["aggregation_method"] not in _METHODS:
        raise ValueError("Aggregation method should be 0, 1, or 2")
    return nl


def run(path="PARA_INPUT.inp", precision="fp64", coarse_solver="rbgs", write_dir=None, log=print):
    """Run the driver; returns a dict with the solve report, the RMS error, the solution
    field (numpy, Fortran order, with ghosts) and the elapsed time."""
    from .multigrid import Multigrid

    nl = read_config(path)
    m, o, ln, st, c = nl["meshes"], nl["origin"], nl["length"], nl["mesh_stretch"], nl["control"]
    procs = nl.get("procs", {})
    nprocs = (procs.get("npx", 1), procs.get("npy", 1), procs.get("npz", 1))
    if nprocs != (1, 1, 1):
        log("[Poisson] &procs asks for %d x %d x %d ranks; one GPU solves the whole domain." % nprocs)
    n = (int(m["nx"]), int(m["ny"]), int(m["nz"]))
    mesh = [domain_mesh(n[d], o["o" + a], ln["l" + a], st["a" + a]) for d, a in enumerate("xyz")]
    log("[Poisson] Geometry and matrix size initialized.")
    lengths = (float(ln["lx"]), float(ln["ly"]), float(ln["lz"]))
    rhs, ref = cosine_problem(mesh, lengths)
    sol = G.field(*n)
    rsd = G.field(*n)
    log("[Poisson] Geometry and rhs constructed.")
    log("[Poisson] Poisson matrix constructed.")
    log("[Poisson] Start solving equations.")
    t0 = time.perf_counter()
    with Multigrid(mesh, int(c["number_of_levels"]), int(c["number_of_vcycles"]),
                   _METHODS[int(c["aggregation_method"])], int(c["cga_level"]), [int(v) for v in c["cgpsa_level"]],
                   coarse_solver=coarse_solver, precision=precision) as mg:
        rep = mg.solve_vcycle(sol, rsd, rhs, int(c["maxiteration"]), float(c["tolerance"]), float(c["omega_sor"]))
    elapsed = time.perf_counter() - t0
    for line in rep.log_lines():
        log(line)
    rms = float(np.sum((sol[1:-1, 1:-1, 1:-1] - ref) ** 2)) / n[0] / n[1] / n[2]
    log("[Poisson] RMS = " + pio.fortran_exp(rms, 20, 10, "E"))
    log("[Poisson] Solution obtained. Execution time = %12.6f" % elapsed)
    if write_dir:
        os.makedirs(write_dir, exist_ok=True)
        inner = sol[1:-1, 1:-1, 1:-1]
        pio.write_ascii(os.path.join(write_dir, "solution_all.dat"), mesh[0][2][1:-1], mesh[1][2][1:-1],
                        mesh[2][2][1:-1], inner)
        pio.write_fortran_record(os.path.join(write_dir, "solution_all.bin"), inner)
        pio.write_raw(os.path.join(write_dir, "solution_all_MPI_IO.bin"), inner)
    log("[Poisson] Solution printed.")
    log("[Poisson] Memory deallocated.")
    return {"report": rep, "rms": rms, "sol": sol, "elapsed_s": elapsed, "mesh": mesh}


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    p.add_argument("input", nargs="?", default="PARA_INPUT.inp")
    p.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    p.add_argument("--coarse", default="rbgs", choices=["rbgs", "cg"])
    p.add_argument("--write", metavar="DIR", default=None, help="write the reference's solution files into DIR")
    a = p.parse_args(argv)
    res = run(a.input, a.precision, a.coarse, a.write)
    return 0 if res["report"].converged else 1


if __name__ == "__main__":
    sys.exit(main())
