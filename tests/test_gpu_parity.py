"""GPU parity: the CUDA Fock build through the C ABI against the oracle.

Tolerance: 1e-10 max-abs on the packed Fock matrix (the plain-FP64 gate).
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


def _compare(fock, oracle_lib, bas, d, se=1.0, sc=1.0, cutoff=1e-10):
    fb = fock.FockBuilder(bas, cutoff=cutoff)
    f = fb.fock_jk(d, scale_exch=se, scale_coul=sc)
    ref = oracle_lib.Oracle(bas, cutoff=cutoff).fock_jk(d, se=se, sc=sc)
    return float(np.abs(f - ref).max()), fb


@pytest.mark.parametrize("basis", ["6-31g*", "cc-pvdz", "sto-3g"])
def test_h2o_rhf_uhf(gpu, oracle_lib, basis):
    from openqp_gb300 import workloads
    bas = h2o_basis(basis)
    err, _ = _compare(gpu, oracle_lib, bas, workloads.density(bas, 5, 0))
    assert err < TOL
    err, _ = _compare(gpu, oracle_lib, bas, workloads.density_open(bas, 6, 4, 1), se=0.8, sc=1.1)
    assert err < TOL


def test_schwarz_matches_oracle(gpu, oracle_lib):
    for basis in ("6-31g*", "cc-pvdz"):
        bas = h2o_basis(basis)
        q = gpu.FockBuilder(bas).schwarz()
        qr = oracle_lib.Oracle(bas).schwarz()
        assert np.abs(q - qr).max() < 1e-13 * max(1.0, qr.max())


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_water4_631gd_config(gpu, oracle_lib, seed):
    """(H2O)4 / 6-31G(d) Cartesian, 76 bf, tau = 1e-10 (the plain FP64 gate)."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(4, 6.0, seed=seed, basis="6-31g(d)")
    assert bas.nbf == 76
    d = workloads.density(bas, 20, seed)
    err, fb = _compare(gpu, oracle_lib, bas, d)
    assert err < TOL
    st = fb.stats()
    assert st["quartets"] > 0 and st["prim_quartets"] > 0


def test_water8_ccpvdz_spherical_uhf(gpu, oracle_lib):
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(8, workloads.cube_edge_like_c1(8), seed=5, basis="cc-pvdz")
    assert int(bas.harmonic.sum()) == 8
    d = workloads.density_open(bas, 41, 39, 5)
    err, _ = _compare(gpu, oracle_lib, bas, d)
    assert err < TOL


def test_routec_seam_matches_oracle(gpu, oracle_lib):
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(4, 6.0, seed=3, basis="6-31g(d)")
    d = workloads.density(bas, 20, 3)
    assert gpu.routec_init(bas, 1e-10) == 0
    f, info = gpu.routec_fock_jk(d, bas.nbf, 1)
    assert info == 0
    ref = oracle_lib.Oracle(bas).fock_jk(d)
    assert np.abs(f - ref).max() < TOL
    # a caller whose basis does not match the registered one is declined
    _, info = gpu.routec_fock_jk(np.zeros(10), 4, 1)
    assert info != 0
    gpu.routec_finalize()
    _, info = gpu.routec_fock_jk(d, bas.nbf, 1)
    assert info == 1


def test_golden_energy_through_gpu(gpu):
    """OpenQP's RHF/6-31G* water energy with the GPU two-electron part."""
    import json
    import os
    from conftest import ROOT
    from openqp_gb300 import onee, scf
    from openqp_gb300.basis import build_basis
    case = json.load(open(os.path.join(ROOT, "tests", "golden", "hf_golden.json")))["cases"][0]
    bas = build_basis(case["atoms"], np.array(case["coord_bohr"]).reshape(-1, 3), case["basis"])
    fb = gpu.FockBuilder(bas, 1e-10)
    S, T = onee.overlap_kinetic(bas)
    r = scf.run_scf(bas.nbf, S, T + onee.nuclear(bas), onee.nuclear_repulsion(bas), 5, 5, fb.fock_jk, conv=1e-11)
    assert r["converged"] and abs(r["energy"] - case["energy"]) < 1e-7


def test_device_path_matches_host_path(gpu):
    import torch
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(3, workloads.cube_edge_like_c1(3), seed=9, basis="6-31g(d)")
    d = workloads.density(bas, 15, 9)
    fb = gpu.FockBuilder(bas)
    f_host = fb.fock_jk(d)
    f_dev = fb.fock_jk_device(torch.from_numpy(d[None]).cuda()).cpu().numpy()
    assert np.abs(f_host - f_dev).max() < 1e-12
