"""Controller output of a real run: the 200^2 acoustics problem on the GPU,
written as ascii and binary frames and read back."""
import numpy as np
import pytest

from clawpack_gb300 import pyclaw, workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fmt,tol", [("ascii", 5e-9), ("binary", 0.0)])
def test_acoustics_frames_written_and_read_back(cuda, tmp_path, fmt, tol):
    w = workloads.acoustics_radial(200, 200)
    claw = workloads.make_claw(w)
    claw.output_format, claw.outdir = fmt, str(tmp_path)
    claw.run()
    assert len(claw.frames) == claw.num_output_times + 1
    for k, fr in enumerate(claw.frames):
        s = pyclaw.Solution(k, path=str(tmp_path), file_format=fmt)
        assert abs(s.t - fr.t) <= 1e-8 * max(fr.t, 1.0)
        assert s.q.shape == fr.q.shape
        assert np.all(np.abs(s.q - fr.q) <= tol * np.abs(fr.q) + (1e-300 if tol else 0.0))
