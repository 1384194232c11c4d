"""The C oracle and the independent numpy restatement agree bit for bit."""
import numpy as np
import pytest

from oracle import classic2_np as cnp
from tests.helpers import PD, random_state

CASES = [(rp, bcs, lim, order, tw)
         for rp in (1, 2, 3)
         for bcs in ((1, 1), (2, 2), (3, 3), (1, 3), (3, 1))
         for lim in (0, 1, 2, 3, 4)
         for order, tw in ((2, 2), (2, 1), (2, 0), (1, 1), (1, 0))]


@pytest.mark.parametrize("rp,bcs,lim,order,tw", CASES)
def test_step2_bitwise(oracle, rp, bcs, lim, order, tw):
    rng = np.random.default_rng(hash((rp, bcs, lim, order, tw)) & 0xffff)
    mx, my = 7, 5
    q = random_state(rp, mx, my, rng)
    bcl = list(bcs)
    bcu = [bcs[1], bcs[0]] if 2 not in bcs else list(bcs)
    qbc_c = oracle.fill_ghosts(q, bcl, bcu)
    qbc_n = cnp.fill_ghosts(q, bcl, bcu)
    assert np.array_equal(qbc_c, qbc_n)
    qc, cflc = oracle.step2(rp, PD[rp], qbc_c, 0.1, 0.13, 0.02, order, tw, [lim] * 4)
    qn, cfln = cnp.step2(rp, PD[rp], qbc_n, 0.1, 0.13, 0.02, order, tw, [lim] * 4)
    assert np.array_equal(qc[:, 2:-2, 2:-2], qn)
    assert cflc == cfln


def test_step_matches_ghosted_step(oracle):
    rng = np.random.default_rng(3)
    q = random_state(2, 9, 6, rng)
    qa, cfla, rc = oracle.step(2, PD[2], q, 0.1, 0.1, 0.01, [3, 1], [3, 1])
    qbc = oracle.fill_ghosts(q, [3, 1], [3, 1])
    qb, cflb = oracle.step2(2, PD[2], qbc, 0.1, 0.1, 0.01)
    assert rc == 0 and cfla == cflb
    assert np.array_equal(qa, qb[:, 2:-2, 2:-2])


def test_threads_do_not_change_bits(oracle):
    rng = np.random.default_rng(4)
    q = random_state(3, 40, 33, rng)
    a = oracle.step(3, PD[3], q, 0.02, 0.03, 0.002, [1, 1], [1, 1], nthreads=1)
    b = oracle.step(3, PD[3], q, 0.02, 0.03, 0.002, [1, 1], [1, 1], nthreads=4)
    assert np.array_equal(a[0], b[0]) and a[1] == b[1]
