"""Frame files in Clawpack's output formats (upstream pyclaw/src/pyclaw/fileio/;
absent from the mounted tree, restated from the published format).

``ascii``: ``fort.tNNNN`` (time and sizes) plus ``fort.qNNNN`` (patch header
and one line of ``num_eqn`` values per cell, x fastest, a blank line after
each row).  ``binary``: the same two header files with
``file_format binary64`` and the cell values as little-endian float64 in
``fort.bNNNN``, in the order of the ascii values (component fastest, then
x, then y), without ghost cells.
"""
from . import ascii, binary  # noqa: F401

FORMATS = ("ascii", "binary")


def module(file_format):
    if file_format == "ascii":
        return ascii
    if file_format in ("binary", "binary64"):
        return binary
    raise ValueError(f"unsupported output format {file_format!r} (supported: {FORMATS})")
