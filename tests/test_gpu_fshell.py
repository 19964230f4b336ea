"""GPU parity of f-shell (L = 3) Fock builds against the oracle.

The f classes (21-54) run FP64 kernels only; the precision modes keep them
in FP64. Tolerance: 1e-10 max-abs (the plain-FP64 gate).
"""
import numpy as np
import pytest

from conftest import h2o_basis

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("no CUDA device")
    from openqp_gb300 import build
    build.build()
    from openqp_gb300 import fock
    return fock


@pytest.mark.parametrize("spherical", [True, False])
def test_h2o_ccpvtz_rhf_uhf(gpu, oracle_lib, spherical):
    from openqp_gb300 import workloads
    bas = h2o_basis("cc-pvtz", spherical=spherical)
    assert bas.nbf == (58 if spherical else 65)
    fb = gpu.FockBuilder(bas)
    o = oracle_lib.Oracle(bas)
    d = workloads.density(bas, 5, 0)
    assert np.abs(fb.fock_jk(d) - o.fock_jk(d)).max() < TOL
    du = workloads.density_open(bas, 6, 4, 1)
    assert np.abs(fb.fock_jk(du, scale_exch=0.8, scale_coul=1.1) - o.fock_jk(du, se=0.8, sc=1.1)).max() < TOL
    st = fb.stats()
    assert sum(st["per_class"][21:]) > 0   # f classes ran


def test_schwarz_with_f(gpu, oracle_lib):
    bas = h2o_basis("cc-pvtz")
    q = gpu.FockBuilder(bas).schwarz()
    qr = oracle_lib.Oracle(bas).schwarz()
    assert np.abs(q - qr).max() < 1e-13 * max(1.0, qr.max())


def test_water2_ccpvtz(gpu, oracle_lib):
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(2, workloads.cube_edge_like_c1(2), seed=1, basis="cc-pvtz")
    d = workloads.density(bas, 10, 1)
    f = gpu.FockBuilder(bas).fock_jk(d)
    assert np.abs(f - oracle_lib.Oracle(bas).fock_jk(d)).max() < TOL


def test_f_response_and_precision_modes(gpu, oracle_lib):
    from openqp_gb300 import workloads
    bas = h2o_basis("cc-pvtz")
    fb = gpu.FockBuilder(bas)
    o = oracle_lib.Oracle(bas)
    x = np.random.default_rng(0).standard_normal((2, bas.nbf, bas.nbf)) * 0.2
    pa, ma = fb.fock_td(x, apb=True, amb=True)
    rp, rm = o.fock_td(x, 3)
    assert np.abs(pa - rp).max() < TOL and np.abs(ma - rm).max() < TOL
    d = workloads.density(bas, 5, 2)
    ref = o.fock_jk(d)
    for mode, tol in (("df", 1e-9), ("mixed-df", 1e-6), ("mixed", 1e-6)):
        fb.set_precision(mode, 1e-6)
        assert np.abs(fb.fock_jk(d) - ref).max() < tol
    fb.set_precision("fp64")


def test_gradient_declines_f(gpu):
    from openqp_gb300 import workloads
    bas = h2o_basis("cc-pvtz")
    fb = gpu.FockBuilder(bas)
    with pytest.raises(gpu.FockError) as e:
        fb.grad2(workloads.density(bas, 5, 0))
    assert e.value.code == 3
