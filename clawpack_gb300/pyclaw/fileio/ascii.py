"""Clawpack ascii frames: ``write(solution, frame, path, file_prefix)`` and
``read(solution, frame, path, file_prefix)`` with the argument meaning of
upstream pyclaw/src/pyclaw/fileio/ascii.py (absent from the mounted tree).

``fort.qNNNN`` holds, per patch, the header of ``_header.patch_header``, a
blank line, then one line per cell with its ``num_eqn`` values, cells in
x-fastest order with a blank line after each row (and, in 3D, after each
z-slice).  Values are written with
``options['format']`` (default ``%18.8e``, Clawpack's ascii precision;
``%25.17e`` round-trips doubles exactly).
"""
from __future__ import annotations

import io
import os

import numpy as np

from . import _header

DEFAULT_FORMAT = "%18.8e"


def _cells_text(q, fmt):
    """Text of the cell lines of one patch (q is (num_eqn, mx[, my[, mz]])):
    x fastest, a blank line after each row and, in 3D, another after each
    z-slice."""
    m = q.shape[0]
    buf = io.StringIO()
    line = fmt * m
    if q.ndim == 2:
        np.savetxt(buf, q.T, fmt=line)
        buf.write("\n")
    elif q.ndim == 3:
        for j in range(q.shape[2]):
            np.savetxt(buf, q[:, :, j].T, fmt=line)
            buf.write("\n")
    else:
        for k in range(q.shape[3]):
            for j in range(q.shape[2]):
                np.savetxt(buf, q[:, :, j, k].T, fmt=line)
                buf.write("\n")
            buf.write("\n")
    return buf.getvalue()


def write(solution, frame, path="./", file_prefix="fort", write_aux=False, options=None,
          write_p=False):
    """Write ``solution`` as frame ``frame`` under ``path``."""
    if write_aux or write_p:
        raise NotImplementedError("aux and derived-quantity output are not supported")
    options = options or {}
    fmt = options.get("format", DEFAULT_FORMAT)
    file_prefix = file_prefix or "fort"
    os.makedirs(path, exist_ok=True)
    st = solution.state
    _header.write_t(path, file_prefix, frame, solution.t, st.num_eqn, len(solution.states),
                    0, st.num_dim, 0, "ascii")
    with open(os.path.join(path, _header.frame_name(file_prefix, "q", frame)), "w") as f:
        for n, state in enumerate(solution.states, start=1):
            f.write(_header.patch_header(n, 1, state.patch))
            f.write(_cells_text(np.asarray(state.q), fmt))


def read(solution, frame, path="./", file_prefix="fort", read_aux=False, options=None):
    """Load frame ``frame`` into ``solution`` (its state is replaced by the
    frame's patch, sizes and time) and return it."""
    if read_aux:
        raise NotImplementedError("aux arrays are not supported")
    file_prefix = file_prefix or "fort"
    hdr = _header.read_t(path, file_prefix, frame)
    with open(os.path.join(path, _header.frame_name(file_prefix, "q", frame))) as f:
        lines = [ln for ln in f.read().splitlines() if ln.strip()]
    patches = []
    pos = 0
    for _ in range(hdr["nstates"]):
        idx, level, ncells, lower, delta, names, pos = _header.parse_patch_header(
            lines, pos, hdr["num_dim"])
        count = hdr["num_eqn"] * int(np.prod(ncells))
        vals, pos = _header.values_from_lines(lines, pos, count)
        q = vals.reshape([hdr["num_eqn"]] + ncells, order="F")
        patches.append((ncells, lower, delta, names, q))
    return _install(solution, hdr, patches)


def _install(solution, hdr, patches):
    from ..geometry import Dimension, Domain
    from ..state import Solution, State

    if len(patches) != 1:
        raise NotImplementedError("frames with more than one patch are not supported")
    ncells, lower, delta, names, q = patches[0]
    dims = [Dimension(lo, lo + n * d, n, name=nm) for lo, d, n, nm in zip(lower, delta, ncells,
                                                                          names)]
    domain = Domain(dims)
    state = State(domain, hdr["num_eqn"])
    state.q = q
    state.t = hdr["t"]
    if solution is None:
        solution = Solution(state, domain)
    else:
        if solution.states:
            state.problem_data = dict(solution.state.problem_data)
        solution.states = [state]
        solution.domain = domain
    solution.t = hdr["t"]
    return solution
