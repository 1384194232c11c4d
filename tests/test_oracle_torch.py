"""The PyTorch transcription used as the gradient reference: FP64 values
equal the C oracle bit for bit; its autograd gradient agrees with central
finite differences."""
import numpy as np
import pytest
import torch

from oracle import classic2_torch as ct
from tests.helpers import PD, random_state


@pytest.mark.parametrize("rp", [1, 2])
@pytest.mark.parametrize("bcs", [([1, 1], [1, 1]), ([2, 2], [2, 2]), ([3, 1], [1, 3])])
@pytest.mark.parametrize("lim,order,tw", [(4, 2, 2), (2, 2, 1), (1, 1, 0), (3, 2, 2), (0, 2, 2)])
def test_transcription_equals_oracle(oracle, rp, bcs, lim, order, tw):
    rng = np.random.default_rng(rp * 100 + lim * 10 + order + tw)
    q = random_state(rp, 11, 8, rng)
    qo, cflo, _ = oracle.step(rp, PD[rp], q, 0.1, 0.13, 0.01, bcs[0], bcs[1], order, tw, [lim] * 4)
    qt, cflt = ct.step(rp, PD[rp], torch.from_numpy(np.ascontiguousarray(q)), 0.1, 0.13, 0.01,
                       bcs[0], bcs[1], order, tw, [lim] * 4)
    assert np.array_equal(qt.numpy(), qo)
    assert abs(cflt - cflo) <= 1e-15 * cflo


@pytest.mark.parametrize("rp", [1, 2])
def test_transcription_gradient_vs_finite_differences(rp):
    rng = np.random.default_rng(5 + rp)
    q = random_state(rp, 10, 9, rng)
    lam = rng.normal(size=q.shape)
    qt = torch.from_numpy(np.ascontiguousarray(q)).requires_grad_(True)
    qn, _ = ct.step(rp, PD[rp], qt, 0.1, 0.1, 0.01, [3, 3], [3, 3], 2, 2, [4] * 4)
    (qn * torch.from_numpy(lam)).sum().backward()
    for _ in range(3):
        v = rng.normal(size=q.shape)
        eps = 1e-6
        fp = ct.step(rp, PD[rp], torch.from_numpy(q + eps * v), 0.1, 0.1, 0.01, [3, 3], [3, 3],
                     2, 2, [4] * 4)[0].numpy()
        fm = ct.step(rp, PD[rp], torch.from_numpy(q - eps * v), 0.1, 0.1, 0.01, [3, 3], [3, 3],
                     2, 2, [4] * 4)[0].numpy()
        fd = float(((fp - fm) / (2 * eps) * lam).sum())
        ad = float((qt.grad.numpy() * v).sum())
        assert abs(fd - ad) <= 1e-6 * max(abs(fd), 1.0), (fd, ad)
