"""GPU parity of f-shell (L = 3) Fock builds against the oracle.

The f classes (21-54) run FP64 kernels only; the precision modes keep them
in FP64. Tolerance: 1e-10 max-abs on Fock matrices (the plain-FP64 gate),
1e-9 Eh/Bohr on gradients.
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


@pytest.mark.parametrize("spherical", [True, False])
def test_grad2_with_f_matches_oracle(gpu, oracle_lib, spherical):
    """Two-electron gradient with f shells (derivative tables raised to g; the
    largest classes build their tables one root at a time)."""
    from openqp_gb300 import workloads
    from openqp_gb300.basis import unpack
    bas = h2o_basis("cc-pvtz", spherical=spherical)
    fb = gpu.FockBuilder(bas)
    o = oracle_lib.Oracle(bas)
    n = bas.nbf
    d = workloads.density(bas, 5, 0)
    g = fb.grad2(d)
    ref = o.grad2e(unpack(d, n))
    assert np.abs(g - ref).max() < 1e-9
    assert np.abs(g.sum(axis=0)).max() < 1e-10
    du = workloads.density_open(bas, 6, 4, 1)
    Da, Db = unpack(du[0], n), unpack(du[1], n)
    g = fb.grad2(du, hfscale=0.7, coulscale=1.1)
    ref = o.grad2e(Da + Db, Da - Db, coulscale=1.1, hfscale=0.7)
    assert np.abs(g - ref).max() < 1e-9


def test_grad2_water2_ccpvtz(gpu, oracle_lib):
    from openqp_gb300 import workloads
    from openqp_gb300.basis import unpack
    bas = workloads.water_cluster_basis(2, workloads.cube_edge_like_c1(2), seed=2, basis="cc-pvtz")
    d = workloads.density(bas, 10, 2)
    g = gpu.FockBuilder(bas).grad2(d)
    ref = oracle_lib.Oracle(bas).grad2e(unpack(d, bas.nbf))
    assert np.abs(g - ref).max() < 1e-9


def test_ccpvtz_scf_matches_oracle_scf(gpu, oracle_lib):
    """RHF SCF of water in cc-pVTZ with the GPU build as its two-electron part
    and with the oracle's: the same energy (both converged to 1e-10)."""
    from openqp_gb300 import onee, scf
    bas = h2o_basis("cc-pvtz")
    S, T = onee.overlap_kinetic(bas)
    H = T + onee.nuclear(bas)
    enuc = onee.nuclear_repulsion(bas)
    fb = gpu.FockBuilder(bas)
    o = oracle_lib.Oracle(bas)
    rg = scf.run_scf(bas.nbf, S, H, enuc, 5, 5, lambda d: fb.fock_jk(d), conv=1e-11, dconv=1e-8)
    ro = scf.run_scf(bas.nbf, S, H, enuc, 5, 5, lambda d: o.fock_jk(d), conv=1e-11, dconv=1e-8)
    assert rg["converged"] and ro["converged"]
    assert abs(rg["energy"] - ro["energy"]) < 1e-9
    assert -76.07 < rg["energy"] < -76.04   # HF/cc-pVTZ water near equilibrium
