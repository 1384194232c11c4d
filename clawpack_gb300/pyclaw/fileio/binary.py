"""Binary frames: the ascii headers (``fort.tNNNN`` with ``file_format
binary64``, the patch header in ``fort.qNNNN``) and the cell values as
little-endian float64 in ``fort.bNNNN``, in the order of the ascii values
(component fastest, then x, then y, then z; no ghost cells, ``num_ghost
0``)."""
from __future__ import annotations

import os

import numpy as np

from . import _header
from .ascii import _install


def write(solution, frame, path="./", file_prefix="fort", write_aux=False, options=None,
          write_p=False):
    """Write ``solution`` as frame ``frame`` under ``path``; with
    ``write_aux`` the aux arrays too, as float64 in ``fort.aNNNN`` in the
    order of ``fort.bNNNN``."""
    if write_p:
        raise NotImplementedError("derived-quantity output is not supported")
    file_prefix = file_prefix or "fort"
    os.makedirs(path, exist_ok=True)
    st = solution.state
    _header.write_t(path, file_prefix, frame, solution.t, st.num_eqn, len(solution.states),
                    getattr(st, "num_aux", 0), st.num_dim, 0, "binary64")
    with open(os.path.join(path, _header.frame_name(file_prefix, "q", frame)), "w") as f:
        for n, state in enumerate(solution.states, start=1):
            f.write(_header.patch_header(n, 1, state.patch))
    with open(os.path.join(path, _header.frame_name(file_prefix, "b", frame)), "wb") as f:
        for state in solution.states:
            np.asarray(state.q, dtype="<f8").ravel(order="F").tofile(f)
    if write_aux and getattr(st, "num_aux", 0):
        with open(os.path.join(path, _header.frame_name(file_prefix, "a", frame)), "wb") as f:
            for state in solution.states:
                np.asarray(state.aux, dtype="<f8").ravel(order="F").tofile(f)


def read(solution, frame, path="./", file_prefix="fort", read_aux=False, options=None):
    """Load frame ``frame`` into ``solution``; with ``read_aux`` the aux
    arrays of ``fort.aNNNN`` too."""
    file_prefix = file_prefix or "fort"
    hdr = _header.read_t(path, file_prefix, frame)
    if hdr["num_ghost"] != 0:
        raise NotImplementedError("binary frames with ghost cells are not supported")
    with open(os.path.join(path, _header.frame_name(file_prefix, "q", frame))) as f:
        lines = [ln for ln in f.read().splitlines() if ln.strip()]
    data = np.fromfile(os.path.join(path, _header.frame_name(file_prefix, "b", frame)),
                       dtype="<f8")
    patches, pos, off = [], 0, 0
    for _ in range(hdr["nstates"]):
        idx, level, ncells, lower, delta, names, pos = _header.parse_patch_header(
            lines, pos, hdr["num_dim"])
        count = hdr["num_eqn"] * int(np.prod(ncells))
        if off + count > data.size:
            raise ValueError("binary frame is shorter than its header")
        q = data[off:off + count].reshape([hdr["num_eqn"]] + ncells, order="F")
        off += count
        patches.append((ncells, lower, delta, names, q.astype(np.float64)))
    aux = None
    if read_aux:
        if not hdr["num_aux"]:
            raise ValueError("the frame's header lists no aux arrays")
        adata = np.fromfile(os.path.join(path, _header.frame_name(file_prefix, "a", frame)),
                            dtype="<f8")
        aux, off = [], 0
        for ncells, *_ in patches:
            count = hdr["num_aux"] * int(np.prod(ncells))
            if off + count > adata.size:
                raise ValueError("binary aux file is shorter than its header")
            aux.append(adata[off:off + count].reshape([hdr["num_aux"]] + list(ncells),
                                                      order="F").astype(np.float64))
            off += count
    return _install(solution, hdr, patches, aux)
