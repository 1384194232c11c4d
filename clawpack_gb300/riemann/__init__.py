"""Riemann-solver descriptors named like the clawpack.riemann modules.

PyClaw passes a solver module to ``ClawSolver2D(riemann.<name>)`` and reads its
shape from ``riemann.static`` (upstream riemann/riemann/static.py; the
riemann submodule is empty in the mounted clawpack 5.14.0 tree,
meson.build:65).  Here each name is a small descriptor object carrying the
same ``__name__``, ``num_eqn`` and ``num_waves`` plus the id of the device
solver in libgclaw.so.
"""
from __future__ import annotations

from types import SimpleNamespace

from .. import _lib
from . import static


def _descriptor(name, rp_id, fwave=False, num_dim=2):
    # cparam plays the role of the f2py module's Fortran common block, which
    # PyClaw fills from state.problem_data before stepping.
    return SimpleNamespace(__name__=f"clawpack_gb300.riemann.{name}", name=name, rp_id=rp_id,
                           num_eqn=static.num_eqn[name], num_waves=static.num_waves[name],
                           num_aux=static.num_aux[name], fwave=fwave, num_dim=num_dim,
                           cparam=SimpleNamespace())


acoustics_2D = _descriptor("acoustics_2D", _lib.RP_ACOUSTICS_2D)
shallow_roe_with_efix_2D = _descriptor("shallow_roe_with_efix_2D",
                                       _lib.RP_SHALLOW_ROE_WITH_EFIX_2D)
euler_4wave_2D = _descriptor("euler_4wave_2D", _lib.RP_EULER_4WAVE_2D)
# variable-coefficient acoustics: state.aux = (rho, c) per cell
vc_acoustics_2D = _descriptor("vc_acoustics_2D", _lib.RP_VC_ACOUSTICS_2D)
# shallow water over bathymetry, f-wave form (solver.fwave = True): state.aux =
# (b,) per cell
shallow_bathymetry_fwave_2D = _descriptor("shallow_bathymetry_fwave_2D",
                                          _lib.RP_SHALLOW_BATHYMETRY_FWAVE_2D, fwave=True)

# 3D (ClawSolver3D): constant-coefficient acoustics, q = (p, u, v, w)
acoustics_3D = _descriptor("acoustics_3D", _lib.RP3_ACOUSTICS_3D, num_dim=3)
# 3D Euler, q = (rho, rho u, rho v, rho w, E), Roe with 3 wave families
euler_3D = _descriptor("euler_3D", _lib.RP3_EULER_3D, num_dim=3)

__all__ = ["acoustics_2D", "shallow_roe_with_efix_2D", "euler_4wave_2D", "vc_acoustics_2D",
           "shallow_bathymetry_fwave_2D", "acoustics_3D", "euler_3D", "static"]
