"""Shapes of the supported Riemann solvers, as in clawpack.riemann.static."""
num_eqn = {
    "acoustics_2D": 3,
    "shallow_roe_with_efix_2D": 3,
    "euler_4wave_2D": 4,
    "vc_acoustics_2D": 3,
    "shallow_bathymetry_fwave_2D": 3,
    "acoustics_3D": 4,
    "euler_3D": 5,
}
num_aux = {
    "acoustics_2D": 0,
    "shallow_roe_with_efix_2D": 0,
    "euler_4wave_2D": 0,
    "vc_acoustics_2D": 2,
    "shallow_bathymetry_fwave_2D": 1,
    "acoustics_3D": 0,
    "euler_3D": 0,
}
num_waves = {
    "acoustics_2D": 2,
    "shallow_roe_with_efix_2D": 3,
    "euler_4wave_2D": 4,
    "vc_acoustics_2D": 2,
    "shallow_bathymetry_fwave_2D": 3,
    "acoustics_3D": 2,
    "euler_3D": 3,
}
