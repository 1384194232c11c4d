"""Field indices of acoustics_3D: q = (p, u, v, w)."""
num_eqn = 4
num_waves = 2
pressure = 0
x_velocity = 1
y_velocity = 2
z_velocity = 3
