"""Shell families on the GPU: the generally contracted s shells of cc-pVXZ
sets (OpenQP stores them as separate segmented shells and int2.F90 evaluates
every shell quartet on its own) share their primitive integrals in the
(ss|ss), (ss|sp), (ss|sd), (ss|pp), (ss|pd), (sp|sp), (sp|sd), (sp|pp)
classes.  The result must be the shell-by-shell sum: against the oracle at
the plain-FP64 gate (1e-10), and
against the same context with families off to 1e-12 (only the order of the
additions differs); the number of shell quartets evaluated must not change.
"""
import numpy as np
import pytest

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


def _on_off(fb, d, **kw):
    fb.set_shell_families(True)
    f_on = fb.fock_jk(d, **kw)
    st_on = fb.stats()
    fb.set_shell_families(False)
    f_off = fb.fock_jk(d, **kw)
    st_off = fb.stats()
    fb.set_shell_families(True)
    return f_on, f_off, st_on, st_off


@pytest.mark.parametrize("nwater,basis,spherical", [(4, "cc-pvdz", True), (3, "cc-pvdz", False),
                                                    (2, "cc-pvtz", True)])
def test_families_match_oracle_and_shell_quartets(gpu, oracle_lib, nwater, basis, spherical):
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(nwater, workloads.cube_edge_like_c1(nwater), 3, basis, spherical=spherical)
    fb = gpu.FockBuilder(bas)
    on, nshared = fb.shell_families_info()
    assert on and nshared > 0
    d = workloads.density(bas, 5 * nwater, 1)
    f_on, f_off, st_on, st_off = _on_off(fb, d)
    ref = oracle_lib.Oracle(bas).fock_jk(d)
    assert np.abs(f_on - ref).max() < TOL
    assert np.abs(f_on - f_off).max() < 1e-12
    # the same shell quartets are evaluated, from fewer primitive integrals
    assert st_on["quartets"] == st_off["quartets"]
    assert st_on["prim_quartets"] < st_off["prim_quartets"]
    # open shell, scaled exchange and Coulomb
    du = workloads.density_open(bas, 5 * nwater + 1, 5 * nwater - 1, 2)
    f_on, f_off, _, _ = _on_off(fb, du, scale_exch=0.7, scale_coul=1.2)
    assert np.abs(f_on - oracle_lib.Oracle(bas).fock_jk(du, se=0.7, sc=1.2)).max() < TOL
    assert np.abs(f_on - f_off).max() < 1e-12


def test_families_device_graph_and_cutoff(gpu, oracle_lib):
    import torch
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(4, workloads.cube_edge_like_c1(4), 5, "cc-pvdz", spherical=True)
    d = workloads.density(bas, 20, 4)
    fb = gpu.FockBuilder(bas)
    ref = oracle_lib.Oracle(bas).fock_jk(d)
    dt = torch.from_numpy(np.ascontiguousarray(d[None])).cuda()
    assert np.abs(fb.fock_jk_device(dt).cpu().numpy() - ref).max() < TOL
    for _ in range(2):   # capture, then replay
        assert np.abs(fb.fock_jk_graph(dt).cpu().numpy() - ref).max() < TOL
    # a looser run-time cutoff rebuilds the family tables at that cutoff
    fb.set_cutoff(1e-8)
    f8 = fb.fock_jk(d)
    assert np.abs(f8 - oracle_lib.Oracle(bas, cutoff=1e-8).fock_jk(d)).max() < TOL
    fb.set_shell_families(False)
    assert np.abs(fb.fock_jk(d) - f8).max() < 1e-12


def test_no_families_without_shared_exponents(gpu):
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(2, 6.0, 0, "6-31g(d)")
    assert gpu.FockBuilder(bas).shell_families_info() == (True, 0)


def test_families_in_a_batch(gpu, oracle_lib):
    from openqp_gb300 import workloads
    from openqp_gb300.onee import one_electron
    bases, dens = [], []
    for k, n in enumerate([2, 1, 3]):
        bas = workloads.water_cluster_basis(n, workloads.cube_edge_like_c1(n), 40 + k, "cc-pvdz", spherical=True)
        bases.append(bas)
        dens.append(workloads.density(bas, 5 * n, k, S=one_electron(bas)[0])[None])
    bb = gpu.BatchFockBuilder(bases)
    assert bb.shell_families_info()[1] > 0
    fs = bb.fock_jk(dens)
    for bas, d, f in zip(bases, dens, fs):
        assert np.abs(f - oracle_lib.Oracle(bas).fock_jk(d[0])).max() < TOL


@pytest.mark.parametrize("mode", ["mixed", "mixed-fast", "df", "mixed-df"])
def test_families_in_precision_modes(gpu, oracle_lib, mode):
    """In the FP32-split modes a family quartet runs in FP32 when all the
    member quartets it lists are below the threshold, else in FP64 (in
    double-float in the df modes).  The mode's own bounds hold with families
    on and off (max |dF| 1e-6 for the FP32 split, 1e-10 for double-float),
    the same shell quartets are evaluated, from fewer primitive integrals."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(4, workloads.cube_edge_like_c1(4), 6, "cc-pvdz", spherical=True)
    d = workloads.density(bas, 20, 3)
    ref = oracle_lib.Oracle(bas).fock_jk(d)
    fb = gpu.FockBuilder(bas)
    fb.set_precision(mode, 1e-6)
    f_on, f_off, st_on, st_off = _on_off(fb, d)
    tol = 1e-10 if mode == "df" else 1e-6
    assert np.abs(f_on - ref).max() < tol
    assert np.abs(f_off - ref).max() < tol
    assert st_on["quartets"] == st_off["quartets"]
    assert st_on["prim_quartets"] < st_off["prim_quartets"]
    if mode == "df":
        assert st_on["f32_quartets"] == st_off["f32_quartets"] == 0
    else:
        assert 0 < st_on["f32_quartets"] <= st_off["f32_quartets"]
