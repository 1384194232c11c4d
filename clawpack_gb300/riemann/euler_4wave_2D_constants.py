"""Field indices of euler_4wave_2D: q = (rho, rho u, rho v, E)."""
num_eqn = 4
num_waves = 4
density = 0
x_momentum = 1
y_momentum = 2
energy = 3
