"""Field indices of shallow_roe_with_efix_2D: q = (h, hu, hv)."""
num_eqn = 3
num_waves = 3
depth = 0
x_momentum = 1
y_momentum = 2
