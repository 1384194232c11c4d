"""Field indices of shallow_bathymetry_fwave_2D: q = (h, hu, hv), aux = (b,)."""
num_eqn = 3
num_waves = 3
depth = 0
x_momentum = 1
y_momentum = 2
bathymetry = 0
