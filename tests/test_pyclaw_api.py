"""The PyClaw-compatible API surface (no GPU needed for these checks)."""
import numpy as np
import pytest

from clawpack_gb300 import _lib, pyclaw, riemann, workloads


def test_solver_defaults_follow_pyclaw():
    s = pyclaw.ClawSolver2D(riemann.euler_4wave_2D)
    assert (s.num_eqn, s.num_waves) == (4, 4)
    assert s.dimensional_split is True
    assert s.transverse_waves == s.trans_inc == 1
    assert s.order == 2 and s.num_ghost == 2
    assert s.limiters == pyclaw.limiters.tvd.minmod
    assert s.cfl_max == 1.0 and s.cfl_desired == 0.9 and s.dt_initial == 0.1
    assert s.max_steps == 10000 and s.dt_variable
    assert s.kernel_language == "CUDA"
    assert s._mthlim == [1, 1, 1, 1]
    s.limiters = [4, 2, 2, 4]
    assert s._mthlim == [4, 2, 2, 4]
    s.limiters = [1, 2]
    with pytest.raises(ValueError):
        s._mthlim


def test_bc_and_limiter_ids():
    assert (pyclaw.BC.custom, pyclaw.BC.extrap, pyclaw.BC.periodic, pyclaw.BC.wall) == (0, 1, 2, 3)
    t = pyclaw.limiters.tvd
    assert (t.minmod, t.superbee, t.vanleer, t.MC) == (1, 2, 3, 4)
    assert riemann.static.num_eqn["shallow_roe_with_efix_2D"] == 3


def test_grid_and_state():
    x = pyclaw.Dimension(-1.0, 1.0, 4, name="x")
    y = pyclaw.Dimension(0.0, 1.0, 2, name="y")
    d = pyclaw.Domain([x, y])
    st = pyclaw.State(d, 3)
    assert st.q.shape == (3, 4, 2) and st.q.flags.f_contiguous
    X, Y = st.grid.p_centers
    assert X.shape == (4, 2)
    np.testing.assert_allclose(X[:, 0], [-0.75, -0.25, 0.25, 0.75])
    assert st.grid.x is x and d.grid.delta == [0.5, 0.5]


def test_unsupported_options_fail_loudly():
    claw = workloads.make_claw(workloads.acoustics_radial(8, 8))
    s = claw.solver
    st = claw.solution.state
    s.kernel_language = "Fortran"
    with pytest.raises(NotImplementedError):
        s.solver_struct(st)
    s.kernel_language = "CUDA"
    s.bc_lower[0] = pyclaw.BC.custom
    with pytest.raises(NotImplementedError):
        s.solver_struct(st)


def test_problem_data_mapping():
    claw = workloads.make_claw(workloads.acoustics_radial(8, 8))
    s, st = claw.solver, claw.solution.state
    del st.problem_data["cc"], st.problem_data["zz"]
    ss = s.solver_struct(st)
    assert list(ss.problem_data)[:4] == [1.0, 4.0, 2.0, 2.0]
    claw = workloads.make_claw(workloads.euler_quadrants(8, 8))
    ss = claw.solver.solver_struct(claw.solution.state)
    assert list(ss.problem_data)[:2] == [1.4, 1.0]


def test_workloads_shapes():
    w = workloads.shallow_dam_break(64, 32)
    assert w.q0.shape == (3, 64, 32) and set(np.unique(w.q0[0])) == {1.0, 2.0}
    e = workloads.euler_quadrants(16, 16)
    assert len(e.meta["states"]) == 4 and e.q0.shape == (4, 16, 16)
    assert np.all(e.q0[0] > 0)


def test_batched_ensemble_shapes_and_sizes():
    e = workloads.batched_ensemble()
    sides = np.array([s[0] for s in e.shapes])
    assert len(sides) == 4096 and sides.min() >= 32 and sides.max() <= 512
    # log-uniform sides: mean cells per problem near (512^2 - 32^2) / (2 ln 16)
    assert 40000 < e.cells / 4096 < 55000
    q = e.q0(3)
    assert q.shape == (3,) + e.shapes[3] and np.all(q[0] >= 1.0) and np.all(q[1:] == 0.0)
    assert np.all(e.dt0 > 0)


def test_batch_table_size():
    from clawpack_gb300 import _lib

    L = _lib.lib()
    assert L.gclaw_batch_table_bytes(10) == 10 * 48 + 2 * 11 * 4  # entries, tile and strip starts
    assert L.gclaw_batch_table_bytes(0) == 0


def test_fwave_solver_front_end():
    x = pyclaw.Dimension(0.0, 1.0, 8, name="x")
    y = pyclaw.Dimension(0.0, 1.0, 6, name="y")
    domain = pyclaw.Domain([x, y])
    st = pyclaw.State(domain, 3, 1)
    st.problem_data["grav"] = 9.81
    st.aux[0] = -1.0
    st.q[0] = 1.0
    s = pyclaw.ClawSolver2D(riemann.shallow_bathymetry_fwave_2D)
    s.dimensional_split = False
    s.bc_lower = s.bc_upper = [pyclaw.BC.wall, pyclaw.BC.wall]
    s.aux_bc_lower = s.aux_bc_upper = [pyclaw.BC.wall, pyclaw.BC.wall]
    with pytest.raises(ValueError):  # f-wave solvers need solver.fwave = True
        s.solver_struct(st)
    s.fwave = True
    ss = s.solver_struct(st)
    assert ss.rp == _lib.RP_SHALLOW_BATHYMETRY_FWAVE_2D and ss.problem_data[0] == 9.81
    assert s.num_waves == 3
    s2 = pyclaw.ClawSolver2D(riemann.shallow_roe_with_efix_2D)
    s2.fwave = True
    claw = workloads.make_claw(workloads.shallow_dam_break(8, 8))
    with pytest.raises(ValueError):  # and the other solvers fwave = False
        s2.solver_struct(claw.solution.state)


def test_clawsolver3d_front_end():
    dims = [pyclaw.Dimension(0.0, 1.0, n, name=c) for n, c in ((8, "x"), (6, "y"), (5, "z"))]
    st = pyclaw.State(pyclaw.Domain(dims), 4)
    st.problem_data.update(rho=1.0, bulk=4.0)
    s = pyclaw.ClawSolver3D(riemann.acoustics_3D)
    assert s.transverse_waves == s.trans_cor == 22 and s.trans_inc == 11
    s.bc_lower = s.bc_upper = [pyclaw.BC.wall] * 3
    assert s.dimensional_split  # split sweeps by default, unsplit on request
    s.solver_struct(st)
    s.dimensional_split = False
    ss = s.solver_struct(st)
    assert (ss.mx, ss.my, ss.mz) == (8, 6, 5) and list(ss.problem_data)[:4] == [1, 4, 2, 2]
    s.transverse_waves = 21
    with pytest.raises(NotImplementedError):
        s.solver_struct(st)
    s2 = pyclaw.ClawSolver2D(riemann.acoustics_3D)
    with pytest.raises(ValueError):  # a 3D solver in the 2D class
        s2.solver_struct(st)
