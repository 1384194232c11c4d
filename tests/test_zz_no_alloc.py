"""gclaw_step2_noalloc, the step2 drop-in for callers that cannot allocate.

A host code that reaches the step through f2py or ctypes with nothing but
the state arrays it was handed, or a process whose device memory belongs to
another framework's caching allocator, cannot supply the gclaw_ctrl
workspace that gclaw_step2 borrows.  gclaw_step2_noalloc keeps that scratch
in a static device array instead, shared by every call.  These tests call it
through the C ABI twice in a row on different problems -- so the second call
starts from the scratch the first one left behind -- and require the same
states and Courant numbers as gclaw_step2, within the 1e-13 relative L1
tolerance of the other product-build parity tests.  The file is named to be
collected last, and it needs nothing set up by other test files.
"""
import ctypes

import numpy as np
import pytest
import torch

from clawpack_gb300 import _lib
from clawpack_gb300.device import make_solver_struct
from tests.helpers import PD, SHAPES, random_state, rel_l1

pytestmark = pytest.mark.gpu

# (riemann solver, mx, my, bc_lower, bc_upper, precision)
PROBLEMS = [
    (2, 150, 97, [3, 1], [1, 3], _lib.PREC_FP64),
    (3, 64, 203, [1, 2], [1, 2], _lib.PREC_FP32_BULK),
]


def _setup(oracle, rp, mx, my, bcl, bcu, prec, seed):
    rng = np.random.default_rng(seed)
    q = random_state(rp, mx, my, rng)
    dx, dy = 1.0 / mx, 1.0 / my
    s = make_solver_struct(rp, mx, my, dx, dy, bcl, bcu, [4] * SHAPES[rp][1], 2, 2, prec, PD[rp])
    qbc = oracle.fill_ghosts(q, bcl, bcu)
    d_old = torch.from_numpy(np.ascontiguousarray(qbc.T)).cuda()
    return s, d_old, 0.1 * min(dx, dy)


def _call(s, d_old, dt, ws=None):
    L = _lib.lib()
    d_new = d_old.clone()
    cfl = ctypes.c_double()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if ws is None:
        rc = L.gclaw_step2_noalloc(ctypes.byref(s), ctypes.c_void_p(d_old.data_ptr()),
                                   ctypes.c_void_p(d_new.data_ptr()), dt, ctypes.byref(cfl),
                                   stream)
    else:
        rc = L.gclaw_step2(ctypes.byref(s), ctypes.c_void_p(d_old.data_ptr()),
                           ctypes.c_void_p(d_new.data_ptr()), dt, ctypes.c_void_p(ws.data_ptr()),
                           ctypes.byref(cfl), stream)
    return rc, np.asfortranarray(d_new.cpu().numpy().T)[:, 2:-2, 2:-2], cfl.value


def test_noalloc_matches_step2_on_two_calls_in_a_row(oracle):
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a GPU")
    cases = [_setup(oracle, *p, seed=k) for k, p in enumerate(PROBLEMS)]
    got = [_call(s, d, dt) for s, d, dt in cases]  # back-to-back no-allocation calls
    for (s, d, dt), (rc, q, cfl) in zip(cases, got):
        ws = torch.zeros(256, dtype=torch.uint8, device="cuda")
        rc_ref, q_ref, cfl_ref = _call(s, d, dt, ws)
        assert rc == rc_ref == _lib.OK
        assert rel_l1(q, q_ref) <= 1e-13
        assert abs(cfl - cfl_ref) <= 1e-15 * cfl_ref
    # and once more on the first problem, after the second left its scratch behind
    s, d, dt = cases[0]
    rc, q, cfl = _call(s, d, dt)
    assert rc == _lib.OK and rel_l1(q, got[0][1]) <= 1e-13 and cfl == got[0][2]


def test_noalloc_rejects_grids_beyond_its_scratch():
    """A grid beyond the scratch is refused before any launch.  The state
    pointers are NULL, which the entry point would also refuse, so no kernel
    can run on this call whatever the tile shape."""
    L = _lib.lib()
    # 16384^2 cells: at least 524288 thread blocks for every tile shape (<= 512 cells)
    for rp, prec in ((2, _lib.PREC_FP64), (3, _lib.PREC_FP64), (2, _lib.PREC_FP32_BULK)):
        mw = SHAPES[rp][1]
        s = make_solver_struct(rp, 16384, 16384, 1e-4, 1e-4, [3, 3], [3, 3], [4] * mw, 2, 2,
                               prec, PD[rp])
        cfl = ctypes.c_double(-1.0)
        rc = L.gclaw_step2_noalloc(ctypes.byref(s), None, None, 1e-5, ctypes.byref(cfl), None)
        assert rc == _lib.ERR_TOO_LARGE == -6
        assert cfl.value == -1.0
    assert b"GCLAW_NOALLOC_MAX_BLOCKS" in L.gclaw_strerror(_lib.ERR_TOO_LARGE)
