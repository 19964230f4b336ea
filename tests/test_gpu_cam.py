"""GPU parity of the CAM (range-separated) builds against the oracle's
restatement of OpenQP's int2_run_cam: pass 1 over 1/r with (alpha,
alpha_coulomb), pass 2 over erf(mu r)/r -- its own Schwarz bounds -- with
(beta, beta_coulomb), for the SCF Fock build, the TD, TD-gradient and
RPA-gradient builds and the MRSF build.

Tolerance: 1e-10 max-abs (the plain-FP64 gate).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-10
CAM = (0.19, 0.46, 0.33, 1.0, 0.0)   # CAM-B3LYP-like alpha, beta, mu; reference default Coulomb scales


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("no CUDA device")
    from openqp_gb300 import build
    build.build()
    from openqp_gb300 import fock
    return fock


@pytest.mark.parametrize("basis", ["6-31g(d)", "cc-pvdz"])
def test_cam_fock_rhf_uhf(gpu, oracle_lib, basis):
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(4, 6.0, seed=0, basis=basis)
    fb = gpu.FockBuilder(bas)
    o = oracle_lib.Oracle(bas)
    d = workloads.density(bas, 20, 0)
    assert np.abs(fb.fock_jk_cam(d, *CAM) - o.fock_jk_cam(d, *CAM)).max() < TOL
    du = workloads.density_open(bas, 21, 19, 1)
    cam = (0.2, 0.65, 0.4, 1.0, 0.3)
    assert np.abs(fb.fock_jk_cam(du, *cam) - o.fock_jk_cam(du, *cam)).max() < TOL
    # a plain build after the CAM build on the same context is unaffected
    assert np.abs(fb.fock_jk(d) - o.fock_jk(d)).max() < TOL


def test_cam_mu_change_and_routec(gpu, oracle_lib):
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(2, workloads.cube_edge_like_c1(2), seed=3, basis="6-31g(d)")
    fb = gpu.FockBuilder(bas)
    o = oracle_lib.Oracle(bas)
    d = workloads.density(bas, 10, 3)
    for mu in (0.33, 0.9, 0.33):
        assert np.abs(fb.fock_jk_cam(d, 0.2, 0.6, mu) - o.fock_jk_cam(d, 0.2, 0.6, mu)).max() < TOL
    assert gpu.routec_init(bas) == 0
    try:
        f, info = gpu.routec_fock_jk_cam(d, bas.nbf, 1, *CAM)
        assert info == 0
        assert np.abs(f - o.fock_jk_cam(d, *CAM)).max() < TOL
        _, info = gpu.routec_fock_jk_cam(d, bas.nbf + 1, 1, *CAM)
        assert info == 1
    finally:
        gpu.routec_finalize()


def test_cam_td(gpu, oracle_lib):
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(4, 6.0, seed=1, basis="cc-pvdz")
    x = np.random.default_rng(5).standard_normal((3, bas.nbf, bas.nbf)) * 0.2
    fb = gpu.FockBuilder(bas)
    o = oracle_lib.Oracle(bas)
    for flags in (3, 12):
        pa, ma = fb.fock_td(x, apb=bool(flags & 1), amb=bool(flags & 2), tda=bool(flags & 4),
                            tda_coulomb=bool(flags & 8), cam=CAM)
        rp, rm = o.fock_td_cam(x, flags, *CAM)
        assert np.abs(pa - rp).max() < TOL and np.abs(ma - rm).max() < TOL


def test_cam_gradient_side_builds(gpu, oracle_lib):
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(4, 6.0, seed=2, basis="6-31g(d)")
    n = bas.nbf
    rng = np.random.default_rng(11)
    fb = gpu.FockBuilder(bas)
    o = oracle_lib.Oracle(bas)
    x = rng.standard_normal((2, n, n)) * 0.2
    pa, ma = fb.fock_tdgrd(x, apb=True, amb=True, cam=CAM)
    rp, rm = o.fock_tdgrd_cam(x, 3, *CAM)
    assert np.abs(pa - rp).max() < TOL and np.abs(ma - rm).max() < TOL
    sym = lambda a: 0.5 * (a + a.swapaxes(-1, -2))
    xpy = sym(rng.standard_normal((1, 2, n, n)) * 0.2)
    xmy = rng.standard_normal((1, 1, n, n)) * 0.2
    got = fb.fock_rpagrd(xpy, xmy, xpy[:, 1:2], 1, cam=CAM)
    ref = o.fock_rpagrd(xpy, xmy, xpy[:, 1:2], 1, cam=CAM)
    for g, r in zip(got, ref):
        assert np.abs(g - r).max() < TOL


@pytest.mark.parametrize("nmat", [7, 11])
def test_cam_mrsf(gpu, oracle_lib, nmat):
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(2, workloads.cube_edge_like_c1(2), seed=4, basis="6-31g(d)")
    x = np.random.default_rng(nmat).standard_normal((2, nmat, bas.nbf, bas.nbf)) * 0.2
    f = gpu.FockBuilder(bas).fock_mrsf(x, cam=CAM)
    ref = oracle_lib.Oracle(bas).fock_mrsf_cam(x, *CAM)
    assert np.abs(f - ref).max() < TOL


def test_cam_rejects_bad_mu(gpu):
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(1, workloads.cube_edge_like_c1(1), seed=0, basis="6-31g(d)")
    fb = gpu.FockBuilder(bas)
    d = workloads.density(bas, 5, 0)
    with pytest.raises(ValueError):
        fb.fock_jk_cam(d, 0.2, 0.6, 0.0)
    from openqp_gb300._lib import lib, ptr
    f = np.zeros_like(d)
    cam = np.array([0.2, 0.6, -1.0, 1.0, 0.0])
    assert lib().oqpg_fock_jk_cam(fb.h, ptr(d), ptr(f), 1, ptr(cam)) == 3
