"""Wave-limiter ids, as in pyclaw.limiters.tvd (the values the Fortran
limiter dispatches on)."""
minmod = 1
superbee = 2
vanleer = 3
van_leer = 3
MC = 4
monotonized_centered = 4
