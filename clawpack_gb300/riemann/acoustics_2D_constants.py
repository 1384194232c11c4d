"""Field indices of acoustics_2D: q = (p, u, v)."""
num_eqn = 3
num_waves = 2
pressure = 0
x_velocity = 1
y_velocity = 2
