"""Field indices of euler_3D: q = (rho, rho u, rho v, rho w, E)."""
num_eqn = 5
num_waves = 3
density = 0
x_momentum = 1
y_momentum = 2
z_momentum = 3
energy = 4
