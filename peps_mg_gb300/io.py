"""The reference's input and output formats (host-side; no GPU needed).

* read_namelists(path)  the Fortran namelist groups of PARA_INPUT.inp
                        (src/main_peps.f90:44-60): `&group name = value ... /`, Fortran
                        literals (1.0d-10, .true., lists "9, 6, 8"), `!` comments
* write_ascii           solution_all.dat: one line `x y z u` per interior cell, i fastest,
                        Fortran edit descriptors (3D20.10,1E30.20) (src/main_peps.f90:304-312)
* write_fortran_record  solution_all.bin: one Fortran unformatted sequential record of the
                        nx*ny*nz interior values in Fortran order, framed by 4-byte
                        little-endian length markers (src/main_peps.f90:314-316)
* write_raw             solution_all_MPI_IO.bin: the same values with no framing, as the
                        MPI-IO file view writes them (src/main_peps.f90:418-427)
and the matching readers.  Arrays are numpy, Fortran-ordered (nx, ny, nz) interiors or
(nx+2, ny+2, nz+2) fields with ghosts (the ghosts are dropped on writing).
"""
import math
import re
import struct

import numpy as np

_MAX_RECORD = 2 ** 31 - 1     # one unsplit record; larger records would need sub-records


def _interior(a):
    a = np.asarray(a, dtype=np.float64)
    if a.ndim != 3:
        raise ValueError("expected a 3-D array")
    return a


# ---------------------------------------------------------------------------------------
# namelists
# ---------------------------------------------------------------------------------------
def _fortran_value(tok):
    t = tok.strip()
    low = t.lower()
    if low in (".true.", ".t.", "t"):
        return True
    if low in (".false.", ".f.", "f"):
        return False
    if (t.startswith("'") and t.endswith("'")) or (t.startswith('"') and t.endswith('"')):
        return t[1:-1]
    if re.fullmatch(r"[+-]?\d+", t):
        return int(t)
    num = re.sub(r"[dDqQ]", "e", t)
    try:
        return float(num)
    except ValueError:
        raise ValueError("cannot read the Fortran value %r" % tok)


def parse_namelists(text):
    """{group: {name: value}} for every `&group ... /` block of `text`.  Names are lower
    case; a comma- or blank-separated list of values gives a list."""
    lines = [ln.split("!", 1)[0] for ln in text.splitlines()]
    body = "\n".join(lines)
    groups = {}
    for m in re.finditer(r"&(\w+)(.*?)(?:^\s*/\s*$|/\s*$|&end)", body, flags=re.S | re.M | re.I):
        name = m.group(1).lower()
        content = m.group(2)
        entries = {}
        parts = re.split(r"(\w+(?:\(\s*\d+\s*\))?)\s*=", content)
        # parts: [pre, key1, val1, key2, val2, ...]
        for key, val in zip(parts[1::2], parts[2::2]):
            vals = [v for v in re.split(r"[,\s]+", val.strip()) if v]
            conv = [_fortran_value(v) for v in vals]
            key = key.lower().replace(" ", "")
            km = re.fullmatch(r"(\w+)\((\d+)\)", key)
            if km:                                   # element assignment name(i) = v
                base, idx = km.group(1), int(km.group(2))
                lst = entries.setdefault(base, [])
                while len(lst) < idx:
                    lst.append(None)
                lst[idx - 1] = conv[0]
            else:
                entries[key] = conv[0] if len(conv) == 1 else conv
        groups[name] = entries
    return groups


def read_namelists(path):
    with open(path) as f:
        return parse_namelists(f.read())


# ---------------------------------------------------------------------------------------
# Fortran formatted numbers: Dw.d / Ew.d as gfortran writes them (0.ddddE+ee)
# ---------------------------------------------------------------------------------------
def fortran_exp(value, width, digits, letter="E"):
    """`value` in the Fortran Ew.d (letter E) or Dw.d (letter D) edit descriptor:
    a leading 0, `digits` significant digits after the point, a signed two-digit
    exponent (three digits, without the letter, for |exponent| > 99), right-justified
    in `width` characters."""
    v = float(value)
    if math.isnan(v):
        s = "NaN"
    elif math.isinf(v):
        s = "Infinity" if v > 0 else "-Infinity"
    elif v == 0.0:
        s = ("-" if math.copysign(1.0, v) < 0 else "") + "0." + "0" * digits + letter + "+00"
    else:
        # mantissa in [0.1, 1) with `digits` digits, exponent e: v = 0.m * 10**e
        m = "%.*e" % (digits - 1, abs(v))              # d.ddd...e+XX
        mant, ex = m.split("e")
        e = int(ex) + 1
        mant = mant.replace(".", "")
        sign = "-" if v < 0 else ""
        if abs(e) <= 99:
            es = "%s%c%02d" % (letter, "+" if e >= 0 else "-", abs(e))
        else:
            es = "%c%03d" % ("+" if e >= 0 else "-", abs(e))
        s = "%s0.%s%s" % (sign, mant, es)
    if len(s) > width:
        return "*" * width
    return s.rjust(width)


def write_ascii(path, xg, yg, zg, u):
    """solution_all.dat: `x y z u` per interior cell, i fastest.  xg, yg, zg: the cell
    centres of the interior (nx, ny, nz values); u: the (nx, ny, nz) interior or the
    (nx+2, ny+2, nz+2) field."""
    u = _interior(u)
    n = (len(xg), len(yg), len(zg))
    if u.shape == tuple(m + 2 for m in n):
        u = u[1:-1, 1:-1, 1:-1]
    elif u.shape != n:
        raise ValueError("u has shape %s, the centres give %s" % (u.shape, n))
    xd = [fortran_exp(v, 20, 10, "D") for v in xg]
    yd = [fortran_exp(v, 20, 10, "D") for v in yg]
    zd = [fortran_exp(v, 20, 10, "D") for v in zg]
    with open(path, "w") as f:
        for k in range(n[2]):
            for j in range(n[1]):
                pre = yd[j] + zd[k]
                col = u[:, j, k]
                f.write("".join(xd[i] + pre + fortran_exp(col[i], 30, 20, "E") + "\n" for i in range(n[0])))


def read_ascii(path):
    """(x, y, z, u) columns of a solution_all.dat file."""
    data = []
    with open(path) as f:
        for line in f:
            data.append([float(line[20 * q:20 * q + 20].replace("D", "E")) for q in range(3)] +
                        [float(line[60:90].replace("D", "E"))])
    a = np.array(data)
    return a[:, 0], a[:, 1], a[:, 2], a[:, 3]


def interior_of(field):
    """The (nx, ny, nz) interior of an (nx+2, ny+2, nz+2) field."""
    f = _interior(field)
    return f[1:-1, 1:-1, 1:-1]


def write_fortran_record(path, interior):
    """solution_all.bin: one unformatted sequential record (4-byte markers, little endian)."""
    a = np.asfortranarray(_interior(interior), dtype="<f8")
    nbytes = a.size * 8
    if nbytes > _MAX_RECORD:
        raise ValueError("a record of %d bytes needs Fortran sub-records, which are not written here" % nbytes)
    marker = struct.pack("<i", nbytes)
    with open(path, "wb") as f:
        f.write(marker)
        f.write(a.tobytes(order="F"))
        f.write(marker)


def read_fortran_record(path, shape):
    """The (nx, ny, nz) array of a file written by write_fortran_record (or by the
    reference's `write(unit) sol_all`)."""
    with open(path, "rb") as f:
        raw = f.read()
    n = struct.unpack("<i", raw[:4])[0]
    tail = struct.unpack("<i", raw[4 + n:8 + n])[0]
    if n != tail or n != 8 * int(np.prod(shape)) or len(raw) != n + 8:
        raise ValueError("not a single unformatted record of %s doubles" % (shape,))
    return np.frombuffer(raw[4:4 + n], dtype="<f8").reshape(shape, order="F").copy(order="F")


def write_raw(path, interior):
    """solution_all_MPI_IO.bin: the interior in Fortran order, native doubles, no framing."""
    with open(path, "wb") as f:
        f.write(np.asarray(_interior(interior), dtype="<f8").tobytes(order="F"))


def read_raw(path, shape):
    return np.fromfile(path, dtype="<f8").reshape(shape, order="F")
