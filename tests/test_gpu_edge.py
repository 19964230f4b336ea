"""GPU edge cases of the Fock build and the gradient against the oracle.

The cases the reference's screening and loop structure meet at their limits
(OpenQP int2.F90:755-805 pair/quartet screens, grd2.F90:145-391): a density
that screens out every quartet, a basis of one shell, one atom with s, p and d
shells on one centre, a single non-zero density element, two molecules far
enough apart that most quartets vanish, and an open-shell pair with one empty
spin density.  Tolerance: 1e-10 max-abs on the packed Fock matrix, 1e-9 on
the gradient (the plain-FP64 gates of the other parity tests).
"""
import numpy as np
import pytest

from conftest import h2o_basis

pytestmark = pytest.mark.gpu
TOL = 1e-10
GTOL = 1e-9


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("no CUDA device")
    from openqp_gb300 import build
    build.build()
    from openqp_gb300 import fock
    return fock


def _basis(charges, xyz, name, spherical=None):
    from openqp_gb300.basis import build_basis
    return build_basis(charges, np.asarray(xyz, dtype=np.float64), name, spherical=spherical)


def _check(fock, oracle_lib, bas, d, se=1.0, sc=1.0):
    f = fock.FockBuilder(bas).fock_jk(d, scale_exch=se, scale_coul=sc)
    ref = oracle_lib.Oracle(bas).fock_jk(d, se=se, sc=sc)
    assert f.shape == np.atleast_2d(ref).shape
    err = float(np.abs(f - np.atleast_2d(ref)).max())
    assert err < TOL, err
    return f


def test_zero_density_screens_everything(gpu, oracle_lib):
    bas = h2o_basis("6-31g*")
    ntri = bas.nbf * (bas.nbf + 1) // 2
    fb = gpu.FockBuilder(bas)
    for nf in (1, 2):
        f = fb.fock_jk(np.zeros((nf, ntri)))
        assert not f.any()
        assert fb.stats()["quartets"] == 0
    assert not fb.grad2(np.zeros(ntri)).any()


def test_one_shell_basis(gpu, oracle_lib):
    """A hydrogen atom in STO-3G: one s shell, nbf = 1, one quartet."""
    bas = _basis([1], [[0.0, 0.0, 0.0]], "sto-3g")
    assert bas.nbf == 1
    d = np.array([0.7])
    f = _check(gpu, oracle_lib, bas, d)
    # F = J - K/2 = D (ss|ss) / 2 for a single function
    eri = oracle_lib.Oracle(bas).eri_dense().reshape(-1)[0]
    assert abs(f[0, 0] - 0.5 * 0.7 * eri) < TOL
    _check(gpu, oracle_lib, bas, np.stack([d, 0.5 * d]), se=0.9, sc=1.2)
    # a single atom has no two-electron gradient: every quartet sits on one centre
    assert not gpu.FockBuilder(bas).grad2(d).any()


@pytest.mark.parametrize("basis,spherical", [("cc-pvdz", None), ("6-31g*", None), ("cc-pvtz", None)])
def test_one_atom_all_shells(gpu, oracle_lib, basis, spherical):
    """One oxygen atom: s, p, d (and f for cc-pVTZ) shells on a single centre."""
    from openqp_gb300 import workloads
    bas = _basis([8], [[0.3, -0.2, 0.1]], basis, spherical)
    _check(gpu, oracle_lib, bas, workloads.density(bas, 4, 3))
    _check(gpu, oracle_lib, bas, workloads.density_open(bas, 5, 3, 4), se=0.7)


def test_single_nonzero_element(gpu, oracle_lib):
    """Only D_ij (and D_ji) non-zero: the shell-density screen keeps just the
    quartets that touch that element's shell pair."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(2, 5.0, seed=1, basis="6-31g(d)")
    ntri = bas.nbf * (bas.nbf + 1) // 2
    rng = np.random.default_rng(7)
    for k in rng.choice(ntri, size=3, replace=False):
        d = np.zeros(ntri)
        d[k] = 0.9
        _check(gpu, oracle_lib, bas, d)


def test_distant_fragments(gpu, oracle_lib):
    """Two waters 80 Bohr apart: inter-fragment pairs fail the pair screen,
    and the Coulomb coupling of the fragments is all that crosses the gap."""
    from openqp_gb300 import workloads
    b1 = h2o_basis("6-31g*")
    xyz = np.concatenate([b1.xyz, b1.xyz + np.array([80.0, 0.0, 0.0])])
    charges = np.concatenate([b1.charges, b1.charges]).astype(int)
    bas = _basis(charges, xyz, "6-31g*")
    d = workloads.density(bas, 10, 2)
    _check(gpu, oracle_lib, bas, d)
    fb = gpu.FockBuilder(bas)
    g = fb.grad2(d)
    n = bas.nbf
    ref = oracle_lib.Oracle(bas).grad2e(_unpack(d, n))
    assert np.abs(g - ref).max() < GTOL


def test_open_shell_with_empty_beta(gpu, oracle_lib):
    """Fσ with D_beta = 0 (a one-electron open shell, as for H atom UHF)."""
    from openqp_gb300 import workloads
    bas = h2o_basis("cc-pvdz")
    d = workloads.density_open(bas, 5, 1, 5)
    d[1] = 0.0
    _check(gpu, oracle_lib, bas, d, se=1.0)


def _unpack(p, n):
    from openqp_gb300.basis import unpack
    return unpack(p, n)
