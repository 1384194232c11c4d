"""Field indices of vc_acoustics_2D: q = (p, u, v), aux = (rho, c)."""
num_eqn = 3
num_waves = 2
pressure = 0
x_velocity = 1
y_velocity = 2
density = 0
sound_speed = 1
