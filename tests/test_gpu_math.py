"""Accuracy of the kernels' hand-written reciprocal and reciprocal square root
against CUDA's own rsqrt() and IEEE division, over a logarithmic sweep of the
arguments the kernels see (exponent sums p + q and Rys arguments X).

* rsqrt64: FP32 seed rsqrtf(x truncated to FP32), then one third-order step of
  the binomial series y0 (1 - t)^(-1/2), t = 1 - x y0^2 (Householder order 3):
  within 2 ulp of the exact value and of CUDA's rsqrt().
* rcp64: rcp.approx.f64 and two Newton-Raphson steps r <- r + r (1 - x r):
  within 1 ulp of IEEE 1.0 / x.
* df_rsqrt / df_rcp (double-float, ~44 bits): FP32 approximation and one
  Newton step in double-float arithmetic: relative error below 1e-13.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ULP = 2.0 ** -52


@pytest.fixture(scope="module")
def results():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("no CUDA device")
    from openqp_gb300 import build
    build.build()
    from openqp_gb300._lib import lib
    rng = np.random.default_rng(0)
    x = np.concatenate([np.exp(rng.uniform(np.log(2.0 ** -60), np.log(2.0 ** 100), 400000)),
                        2.0 ** np.arange(-60, 101, dtype=np.float64),
                        np.nextafter(2.0 ** np.arange(-60, 101, dtype=np.float64), 0.0)])
    xd = torch.from_numpy(x).cuda()
    out = torch.empty((x.size, 6), dtype=torch.float64, device="cuda")
    assert lib().oqpg_math_check(ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(out.data_ptr()), x.size) == 0
    return x, out.cpu().numpy()


def _rel(a, ref):
    return np.abs((a.astype(np.longdouble) - ref) / ref).astype(np.float64)


def test_rsqrt64(results):
    x, o = results
    exact = 1 / np.sqrt(x.astype(np.longdouble))
    assert _rel(o[:, 0], exact).max() < 2 * ULP
    assert np.abs((o[:, 0] - o[:, 1]) / o[:, 1]).max() < 2 * ULP


def test_rcp64(results):
    x, o = results
    assert np.abs((o[:, 2] - o[:, 3]) / o[:, 3]).max() <= ULP


def test_double_float_rcp_rsqrt(results):
    x, o = results
    xl = x.astype(np.longdouble)
    assert _rel(o[:, 4], 1 / np.sqrt(xl)).max() < 1e-13
    assert _rel(o[:, 5], 1 / xl).max() < 1e-13
