"""Petite-list builds on the GPU (OpenQP's int2.F90:411-469 quartet weights
and scf_addons.F90:1563-1615 skeleton symmetrisation, abelian tier): with the
symmetry registered, a totally symmetric density is built from one quartet per
orbit and the symmetrised result must be the complete Fock matrix, against
the oracle's complete build at the plain-FP64 gate (1e-10).  A density that
is not invariant must fall back to the complete build, with the same result.
"""
import numpy as np
import pytest

from test_symmetry import ethylene, symmetric_density, water

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


@pytest.mark.parametrize("mol,basis", [("ethylene", "6-31g(d)"), ("ethylene", "cc-pvdz"), ("water", "cc-pvtz")])
def test_petite_rhf_matches_complete_build(gpu, oracle_lib, mol, basis):
    from openqp_gb300 import symmetry
    bas = (water if mol == "water" else ethylene)(basis)
    sym = symmetry.abelian_symmetry(bas)
    d = symmetric_density(bas, sym, 5 if mol == "water" else 8, 4)
    ref = oracle_lib.Oracle(bas).fock_jk(d)
    fb = gpu.FockBuilder(bas)
    full = fb.fock_jk(d)
    nq_full = fb.stats()["quartets"]
    fb.set_symmetry(sym)
    f = fb.fock_jk(d)
    assert fb.symmetry_info() == (sym[0], True)
    nq = fb.stats()["quartets"]
    # one quartet per orbit: at least 1/|G| of the quartets (orbits of quartets
    # on the symmetry elements are smaller than |G|); measured 1/1.9 for C2v
    # water, 1/3.4 and 1/3.7 for D2h ethylene
    assert nq_full / sym[0] <= nq < nq_full / 1.5
    assert np.abs(f - ref).max() < TOL
    assert np.abs(f - full).max() < TOL
    # a density that is not invariant: every quartet, same answer as the oracle
    from openqp_gb300 import workloads
    da = workloads.density(bas, 5 if mol == "water" else 8, 11)
    fa = fb.fock_jk(da)
    assert fb.symmetry_info()[1] is False
    assert np.abs(fa - oracle_lib.Oracle(bas).fock_jk(da)).max() < TOL
    fb.set_symmetry(None)
    assert fb.symmetry_info() == (1, False)
    assert np.abs(fb.fock_jk(d) - ref).max() < TOL


def test_petite_uhf_device_and_graph(gpu, oracle_lib):
    import torch
    from openqp_gb300 import symmetry, workloads
    from openqp_gb300.basis import pack, unpack
    bas = ethylene("6-31g(d)")
    sym = symmetry.abelian_symmetry(bas)
    du = workloads.density_open(bas, 9, 7, 5)
    du = np.stack([pack(symmetry.project(unpack(x, bas.nbf), sym[2], sym[3])) for x in du])
    ref = oracle_lib.Oracle(bas).fock_jk(du, se=0.8, sc=1.1)
    fb = gpu.FockBuilder(bas)
    fb.set_symmetry(sym)
    assert np.abs(fb.fock_jk(du, scale_exch=0.8, scale_coul=1.1) - ref).max() < TOL
    dt = torch.from_numpy(du).cuda()
    assert np.abs(fb.fock_jk_device(dt, 0.8, 1.1).cpu().numpy() - ref).max() < TOL
    for _ in range(2):   # capture, then replay
        assert np.abs(fb.fock_jk_graph(dt, 0.8, 1.1).cpu().numpy() - ref).max() < TOL


def test_petite_through_the_seam_with_increments(gpu, oracle_lib):
    """routec_fock_set_symmetry with OpenQP's staged layout (1-based images),
    a full build and an incremental one (the increment is symmetrised before
    F_old is added, as in scf_addons.F90:1186-1210)."""
    from openqp_gb300 import symmetry
    bas = ethylene("cc-pvdz")
    sym = symmetry.abelian_symmetry(bas)
    d1 = symmetric_density(bas, sym, 8, 6)
    d2 = symmetric_density(bas, sym, 8, 7)
    o = oracle_lib.Oracle(bas)
    assert gpu.routec_init(bas, 1e-10) == 0
    assert gpu.routec_fock_set_symmetry(*sym) == 0
    f1, info = gpu.routec_fock_jk(d1, bas.nbf, 1)
    assert info == 0
    g1 = o.fock_jk(d1).reshape(1, -1)
    assert np.abs(f1 - g1).max() < TOL
    f_old = np.ascontiguousarray(g1.copy())
    f2, info = gpu.routec_fock_jk_inc(d2 - d1, f_old, bas.nbf, 1)
    assert info == 0
    assert np.abs(f2 - (g1 + o.fock_jk(d2 - d1).reshape(1, -1))).max() < TOL
    assert np.array_equal(f_old, f2)
    bad = (sym[0], sym[1], sym[2][:, ::-1].copy(), sym[3])   # not a map of components onto components
    assert gpu.routec_fock_set_symmetry(*bad) == 3
    gpu.routec_finalize()
