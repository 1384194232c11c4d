"""The two ascii header files every Clawpack frame has: ``fort.tNNNN`` with
the time and the array sizes, and the per-patch header at the top of
``fort.qNNNN`` (patch number, AMR level, cells, lower corner, spacing)."""
from __future__ import annotations

import os

import numpy as np


def frame_name(prefix, kind, frame):
    return f"{prefix}.{kind}{int(frame):04d}"


def _num(tok):
    # Fortran writers may use D exponents
    return float(tok.replace("D", "E").replace("d", "e"))


def write_t(path, prefix, frame, t, num_eqn, nstates, num_aux, num_dim, num_ghost,
            file_format):
    with open(os.path.join(path, frame_name(prefix, "t", frame)), "w") as f:
        f.write(f"{t:18.8e}    time\n")
        f.write(f"{num_eqn:5d}                 num_eqn\n")
        f.write(f"{nstates:5d}                 nstates\n")
        f.write(f"{num_aux:5d}                 num_aux\n")
        f.write(f"{num_dim:5d}                 num_dim\n")
        f.write(f"{num_ghost:5d}                 num_ghost\n")
        f.write(f"{file_format:>10s}            file_format\n")


def read_t(path, prefix, frame):
    """dict with t, num_eqn, nstates, num_aux, num_dim, num_ghost, file_format
    (the last two default to 0 and 'ascii' for headers without them)."""
    with open(os.path.join(path, frame_name(prefix, "t", frame))) as f:
        lines = [ln.split() for ln in f if ln.strip()]
    out = {"t": _num(lines[0][0]), "num_eqn": int(lines[1][0]), "nstates": int(lines[2][0]),
           "num_aux": int(lines[3][0]), "num_dim": int(lines[4][0]), "num_ghost": 0,
           "file_format": "ascii"}
    if len(lines) > 5:
        out["num_ghost"] = int(lines[5][0])
    if len(lines) > 6:
        out["file_format"] = lines[6][0]
    return out


def patch_header(patch_index, level, patch):
    dims = patch.dimensions
    lines = [f"{patch_index:5d}                 grid_number", f"{level:5d}                 AMR_level"]
    lines += [f"{d.num_cells:5d}                 m{d.name}" for d in dims]
    lines += [f"{d.lower:18.8e}    {d.name}low" for d in dims]
    lines += [f"{d.delta:18.8e}    d{d.name}" for d in dims]
    return "\n".join(lines) + "\n\n"


def parse_patch_header(lines, pos, num_dim):
    """(patch_index, level, num_cells, lower, delta, names, next position)
    from the non-blank header lines starting at ``pos``."""
    patch_index = int(lines[pos].split()[0])
    level = int(lines[pos + 1].split()[0])
    p = pos + 2
    num_cells = [int(lines[p + d].split()[0]) for d in range(num_dim)]
    names = [lines[p + d].split()[1][1:] for d in range(num_dim)]
    p += num_dim
    lower = [_num(lines[p + d].split()[0]) for d in range(num_dim)]
    p += num_dim
    delta = [_num(lines[p + d].split()[0]) for d in range(num_dim)]
    p += num_dim
    return patch_index, level, num_cells, lower, delta, names, p


def values_from_lines(lines, pos, count):
    """``count`` numbers from the lines starting at ``pos`` (blank lines
    already removed); returns (values, next position)."""
    # fast path: the values of ``count`` numbers on whole lines, parsed at once
    width = len(lines[pos].split()) if pos < len(lines) else 0
    if width and count % width == 0:
        nl = count // width
        text = " ".join(lines[pos:pos + nl])
        if "D" in text or "d" in text:
            text = text.replace("D", "E").replace("d", "e")
        toks = text.split()
        if len(toks) == count:
            return np.array(toks, dtype=np.float64), pos + nl
    vals = []
    p = pos
    while len(vals) < count:
        vals.extend(_num(tok) for tok in lines[p].split())
        p += 1
    if len(vals) != count:
        raise ValueError("frame data does not match the patch header")
    return np.asarray(vals, dtype=np.float64), p
