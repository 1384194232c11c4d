"""Frame files (clawpack_gb300.pyclaw.fileio): the ascii and binary formats,
their round trips, the committed format fixture, readers for older headers
and Fortran D exponents, and Controller output."""
import os

import numpy as np
import pytest

from clawpack_gb300 import pyclaw

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "frame_ascii")


def small_solution(mx=3, my=2, t=0.25):
    d = pyclaw.Domain([pyclaw.Dimension(-1, 1, mx, name="x"), pyclaw.Dimension(0, 2, my, name="y")])
    st = pyclaw.State(d, 3)
    st.q = np.arange(3 * mx * my, dtype=float).reshape(3, mx, my, order="F") * 0.1
    sol = pyclaw.Solution(st, d)
    sol.t = t
    return sol


def test_ascii_matches_committed_fixture(tmp_path):
    """The 3x2 frame of the fixture (written once and checked by hand against
    the format: time/size header, patch header, one line per cell with the
    components, x fastest, a blank line after each row)."""
    small_solution().write(0, str(tmp_path))
    for name in ("fort.t0000", "fort.q0000"):
        assert (tmp_path / name).read_text() == open(os.path.join(GOLDEN, name)).read()


def test_fixture_layout():
    lines = open(os.path.join(GOLDEN, "fort.q0000")).read().splitlines()
    assert lines[0].split() == ["1", "grid_number"]
    assert [ln.split()[1] for ln in lines[2:8]] == ["mx", "my", "xlow", "ylow", "dx", "dy"]
    cells = [ln.split() for ln in lines[9:]]
    assert cells[0] == ["0.00000000e+00", "1.00000000e-01", "2.00000000e-01"]  # q[:, 0, 0]
    assert cells[3] == []  # blank line after the first row of 3 cells
    assert cells[4] == ["9.00000000e-01", "1.00000000e+00", "1.10000000e+00"]  # q[:, 0, 1]


@pytest.mark.parametrize("mx,my", [(1, 1), (5, 3), (64, 17)])
def test_ascii_round_trip(tmp_path, mx, my):
    rng = np.random.default_rng(mx * my)
    sol = small_solution(mx, my, t=1.0 / 3.0)
    sol.state.q = rng.normal(size=(3, mx, my)) * 10.0 ** rng.integers(-5, 5, size=(3, mx, my))
    sol.write(4, str(tmp_path))
    back = pyclaw.Solution(4, path=str(tmp_path))
    assert back.q.shape == (3, mx, my)
    assert abs(back.t - sol.t) <= 1e-8 * sol.t
    assert np.all(np.abs(back.q - sol.q) <= 5e-9 * np.abs(sol.q))
    d0, d1 = back.patch.dimensions
    assert (d0.num_cells, d1.num_cells) == (mx, my)
    assert (d0.name, d1.name) == ("x", "y")
    assert abs(d0.lower + 1.0) < 1e-12 and abs(d1.delta - 2.0 / my) < 1e-8
    # full precision on request
    sol.write(5, str(tmp_path), options={"format": "%25.17e"})
    assert np.array_equal(pyclaw.Solution(5, path=str(tmp_path)).q, sol.q)


def test_binary_round_trip_is_exact(tmp_path):
    sol = small_solution(37, 11)
    sol.state.q = np.random.default_rng(1).normal(size=(3, 37, 11))
    sol.write(2, str(tmp_path), file_format="binary", file_prefix="run")
    assert (tmp_path / "run.b0002").stat().st_size == 8 * 3 * 37 * 11
    assert "binary64" in (tmp_path / "run.t0002").read_text()
    back = pyclaw.Solution(2, path=str(tmp_path), file_format="binary", file_prefix="run")
    assert np.array_equal(back.q, sol.q) and back.t == sol.t


def test_reader_accepts_old_headers_and_d_exponents(tmp_path):
    (tmp_path / "fort.t0007").write_text(
        "  0.50000000D+00    time\n    1    num_eqn\n    1    nstates\n"
        "    0    num_aux\n    2    num_dim\n")
    (tmp_path / "fort.q0007").write_text(
        "    1    grid_number\n    1    AMR_level\n    2    mx\n    1    my\n"
        "  0.0D+00  xlow\n  0.0D+00  ylow\n  0.5D+00  dx\n  1.0D+00  dy\n\n"
        "  1.5D+00\n  -2.25d-01\n\n")
    sol = pyclaw.Solution(7, path=str(tmp_path))
    assert sol.t == 0.5
    assert np.array_equal(sol.q, np.array([[[1.5], [-0.225]]]))


def test_unknown_format_raises(tmp_path):
    with pytest.raises(ValueError):
        small_solution().write(0, str(tmp_path), file_format="hdf5")


class _StubSolver:
    """Moves the solution to each output time without stepping."""

    status = 0

    def setup(self, solution):
        pass

    def evolve_to_time(self, solution, t):
        solution.state.q = solution.state.q + 1.0
        solution.t = t
        return 0


def test_controller_writes_every_frame(tmp_path):
    claw = pyclaw.Controller()
    claw.solution = small_solution(4, 3, t=0.0)
    claw.solver = _StubSolver()
    claw.tfinal, claw.num_output_times = 1.0, 4
    claw.output_format, claw.outdir = "ascii", str(tmp_path / "_output")
    claw.run()
    for k in range(5):
        s = pyclaw.Solution(k, path=claw.outdir)
        assert abs(s.t - 0.25 * k) < 1e-12
        assert np.allclose(s.q, claw.frames[k].q, rtol=5e-9, atol=0)


def small_solution3(mx, my, mz, t=0.25):
    dims = [pyclaw.Dimension(-1.0, 1.0, n, name=c) for n, c in ((mx, "x"), (my, "y"), (mz, "z"))]
    domain = pyclaw.Domain(dims)
    state = pyclaw.State(domain, 4)
    sol = pyclaw.Solution(state, domain)
    sol.t = t
    return sol


@pytest.mark.parametrize("fmt", ["ascii", "binary"])
def test_3d_round_trip(tmp_path, fmt):
    """3D frames (ClawSolver3D's output): x fastest, then y, then z, with
    the three dimensions in the patch header; exact at full precision."""
    mx, my, mz = 7, 4, 3
    sol = small_solution3(mx, my, mz, t=0.125)
    sol.state.q = np.random.default_rng(5).normal(size=(4, mx, my, mz))
    opts = {"format": "%25.17e"} if fmt == "ascii" else None
    sol.write(3, str(tmp_path), file_format=fmt, options=opts)
    assert " 3                 num_dim" in (tmp_path / "fort.t0003").read_text()
    back = pyclaw.Solution(3, path=str(tmp_path), file_format=fmt)
    assert back.q.shape == (4, mx, my, mz) and back.t == sol.t
    assert np.array_equal(back.q, sol.q)
    assert [d.num_cells for d in back.patch.dimensions] == [mx, my, mz]
    assert [d.name for d in back.patch.dimensions] == ["x", "y", "z"]
    if fmt == "ascii":
        # the first value lines are the first row: q(:, i, 0, 0) for i = 0..mx-1
        text = (tmp_path / "fort.q0003").read_text().split("\n\n", 1)[1]
        rows = [ln for ln in text.splitlines() if ln.strip()]
        assert len(rows) == mx * my * mz
        first = np.array([[float(v) for v in ln.split()] for ln in rows[:mx]])
        assert np.array_equal(first.T, sol.q[:, :, 0, 0])
        second_slice = np.array([float(v) for v in rows[mx * my].split()])
        assert np.array_equal(second_slice, sol.q[:, 0, 0, 1])


@pytest.mark.parametrize("fmt", ["ascii", "binary"])
def test_aux_round_trip(tmp_path, fmt):
    """Aux arrays (variable-coefficient and bathymetry solvers) go to
    fort.aNNNN beside fort.qNNNN, num_aux in fort.tNNNN, and come back with
    read_aux."""
    mx, my = 9, 5
    dims = [pyclaw.Dimension(0.0, 1.0, mx, name="x"), pyclaw.Dimension(0.0, 2.0, my, name="y")]
    domain = pyclaw.Domain(dims)
    state = pyclaw.State(domain, 3, 2)
    rng = np.random.default_rng(9)
    state.q = rng.normal(size=(3, mx, my))
    state.aux = rng.random(size=(2, mx, my)) + 0.5
    sol = pyclaw.Solution(state, domain)
    opts = {"format": "%25.17e"} if fmt == "ascii" else None
    sol.write(1, str(tmp_path), file_format=fmt, write_aux=True, options=opts)
    assert "    2                 num_aux" in (tmp_path / "fort.t0001").read_text()
    assert (tmp_path / "fort.a0001").exists()
    back = pyclaw.Solution(1, path=str(tmp_path), file_format=fmt, read_aux=True)
    assert np.array_equal(back.q, sol.q)
    assert back.state.num_aux == 2 and np.array_equal(back.state.aux, state.aux)
    # without read_aux the frame loads as before
    assert pyclaw.Solution(1, path=str(tmp_path), file_format=fmt).state.aux is None
    # a frame written without aux cannot be read with it
    plain = pyclaw.Solution(pyclaw.State(domain, 3), domain)
    plain.write(2, str(tmp_path), file_format=fmt)
    with pytest.raises(ValueError):
        pyclaw.Solution(2, path=str(tmp_path), file_format=fmt, read_aux=True)


def test_controller_aux_output_options(tmp_path):
    """write_aux_init writes the aux arrays with frame 0 only,
    write_aux_always with every frame (PyClaw's Controller options)."""
    dims = [pyclaw.Dimension(0.0, 1.0, 4, name="x"), pyclaw.Dimension(0.0, 1.0, 3, name="y")]
    domain = pyclaw.Domain(dims)
    state = pyclaw.State(domain, 3, 1)
    state.aux = np.ones((1, 4, 3))
    claw = pyclaw.Controller()
    claw.solution = pyclaw.Solution(state, domain)
    claw.output_format = "ascii"
    for flag, sub in (("write_aux_init", "init"), ("write_aux_always", "always")):
        claw.outdir = str(tmp_path / sub)
        claw.write_aux_init = claw.write_aux_always = False
        setattr(claw, flag, True)
        claw._output(0)
        claw._output(1)
        has = [(tmp_path / sub / f"fort.a000{k}").exists() for k in (0, 1)]
        assert has == ([True, False] if sub == "init" else [True, True])
