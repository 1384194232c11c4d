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
    """Write ``solution`` as frame ``frame`` under ``path``; with
    ``write_aux`` the aux arrays too, as ``fort.aNNNN`` in the layout of
    ``fort.qNNNN``."""
    if write_p:
        raise NotImplementedError("derived-quantity output is not supported")
    options = options or {}
    fmt = options.get("format", DEFAULT_FORMAT)
    file_prefix = file_prefix or "fort"
    os.makedirs(path, exist_ok=True)
    st = solution.state
    _header.write_t(path, file_prefix, frame, solution.t, st.num_eqn, len(solution.states),
                    getattr(st, "num_aux", 0), st.num_dim, 0, "ascii")
    with open(os.path.join(path, _header.frame_name(file_prefix, "q", frame)), "w") as f:
        for n, state in enumerate(solution.states, start=1):
            f.write(_header.patch_header(n, 1, state.patch))
            f.write(_cells_text(np.asarray(state.q), fmt))
    if write_aux and getattr(st, "num_aux", 0):
        with open(os.path.join(path, _header.frame_name(file_prefix, "a", frame)), "w") as f:
            for n, state in enumerate(solution.states, start=1):
                f.write(_header.patch_header(n, 1, state.patch))
                f.write(_cells_text(np.asarray(state.aux), fmt))


def _read_cells(path, name, hdr, nfields):
    """The patches of an ascii cell file: (ncells, lower, delta, names,
    values of shape (nfields, *ncells))."""
    with open(os.path.join(path, name)) as f:
        lines = [ln for ln in f.read().splitlines() if ln.strip()]
    patches = []
    pos = 0
    for _ in range(hdr["nstates"]):
        idx, level, ncells, lower, delta, names, pos = _header.parse_patch_header(
            lines, pos, hdr["num_dim"])
        count = nfields * int(np.prod(ncells))
        vals, pos = _header.values_from_lines(lines, pos, count)
        patches.append((ncells, lower, delta, names,
                        vals.reshape([nfields] + ncells, order="F")))
    return patches


def read(solution, frame, path="./", file_prefix="fort", read_aux=False, options=None):
    """Load frame ``frame`` into ``solution`` (its state is replaced by the
    frame's patch, sizes and time) and return it; with ``read_aux`` the aux
    arrays of ``fort.aNNNN`` too."""
    file_prefix = file_prefix or "fort"
    hdr = _header.read_t(path, file_prefix, frame)
    patches = _read_cells(path, _header.frame_name(file_prefix, "q", frame), hdr, hdr["num_eqn"])
    aux = None
    if read_aux:
        if not hdr["num_aux"]:
            raise ValueError("the frame's header lists no aux arrays")
        aux = [p[4] for p in _read_cells(path, _header.frame_name(file_prefix, "a", frame), hdr,
                                         hdr["num_aux"])]
    return _install(solution, hdr, patches, aux)


def _install(solution, hdr, patches, aux=None):
    from ..geometry import Dimension, Domain
    from ..state import Solution, State

    if len(patches) != 1:
        raise NotImplementedError("frames with more than one patch are not supported")
    ncells, lower, delta, names, q = patches[0]
    dims = [Dimension(lo, lo + n * d, n, name=nm) for lo, d, n, nm in zip(lower, delta, ncells,
                                                                          names)]
    domain = Domain(dims)
    state = State(domain, hdr["num_eqn"], hdr["num_aux"] if aux is not None else 0)
    state.q = q
    if aux is not None:
        if list(aux[0].shape[1:]) != list(ncells):
            raise ValueError("aux file and q file disagree on the patch size")
        state.aux = aux[0]
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
