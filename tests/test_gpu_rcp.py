"""The FP64 reciprocal of the product build (Newton-Raphson from an FP32
seed) against the correctly rounded 1/x: within one unit in the last place
over the whole normal range, both signs of the special cases handled by the
IEEE division."""
import numpy as np
import pytest
import torch

from clawpack_gb300 import _lib

pytestmark = pytest.mark.gpu


def device_rcp(x, strict=False):
    d = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    y = torch.empty_like(d)
    L = _lib.lib(strict)
    _lib.check(L.gclaw_rcp_fp64(d.data_ptr(), y.data_ptr(), d.numel(),
                                torch.cuda.current_stream().cuda_stream), "gclaw_rcp_fp64")
    return y.cpu().numpy()


def test_within_one_ulp_over_the_normal_range(cuda):
    rng = np.random.default_rng(0)
    m = 1.0 + rng.random(200000)
    e = rng.integers(-1020, 1020, size=m.size)
    x = np.ldexp(m, e)
    x = np.concatenate([x, [1.0, 2.0, 0.5, 1.5, np.nextafter(2.0, 0.0), 3.0, 1e-300, 1e300]])
    y = device_rcp(x)
    exact = 1.0 / x
    ulps = np.abs(y - exact) / np.spacing(exact)
    assert ulps.max() <= 1.0, ulps.max()
    assert (ulps == 0).mean() > 0.9  # mostly correctly rounded


def test_special_values_take_the_division(cuda):
    x = np.array([0.0, -0.0, -2.0, np.inf, -np.inf, np.nan, 5e-324, 2.2e-308, 1.7e308])
    y = device_rcp(x)
    with np.errstate(divide="ignore", over="ignore"):
        exact = 1.0 / x
    assert np.array_equal(np.isnan(y), np.isnan(exact))
    ok = ~np.isnan(exact)
    assert np.array_equal(y[ok], exact[ok])


def test_strict_library_divides_exactly(cuda):
    x = np.ldexp(1.0 + np.random.default_rng(1).random(1000), 7)
    assert np.array_equal(device_rcp(x, strict=True), 1.0 / x)
