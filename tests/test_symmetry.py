"""CPU checks of the abelian symmetry data the petite list consumes
(openqp_gb300.symmetry): the operations found for water (C2v) and ethylene
(D2h) in their standard frames, the projector, and the AO sign tables against
the integrals themselves.  The oracle's Fock matrix of a totally symmetric
density must be totally symmetric; that holds only if every shell image and
every AO sign (Cartesian, pure d, pure f) is right."""
import numpy as np
import pytest

from openqp_gb300 import symmetry
from openqp_gb300.basis import ANGSTROM, build_basis, pack, unpack


def water(basis):
    xyz = np.array([[0.0, 0.0, 0.0], [0.0, 0.757, 0.587], [0.0, -0.757, 0.587]]) * ANGSTROM
    return build_basis([8, 1, 1], xyz, basis)


def ethylene(basis):
    c, hy, hz = 0.6695, 0.9235, 1.2345
    xyz = np.array([[0, 0, c], [0, 0, -c], [0, hy, hz], [0, -hy, hz], [0, hy, -hz], [0, -hy, -hz]]) * ANGSTROM
    return build_basis([6, 6, 1, 1, 1, 1], xyz, basis)


def symmetric_density(bas, sym, nocc, seed):
    from openqp_gb300 import workloads
    d = unpack(workloads.density(bas, nocc, seed), bas.nbf)
    return pack(symmetry.project(d, sym[2], sym[3]))


def test_groups_found():
    assert symmetry.abelian_symmetry(water("6-31g(d)"))[0] == 4
    n, sm, at, sg = symmetry.abelian_symmetry(ethylene("cc-pvdz"))
    assert n == 8
    assert np.all(sm[0] == np.arange(sm.shape[1])) and np.all(sg[0] == 1.0)
    for k in range(n):   # every operation permutes shells and AOs
        assert sorted(sm[k]) == list(range(sm.shape[1])) and sorted(at[k]) == list(range(at.shape[1]))
    # a distorted molecule keeps only the operations it still has
    b = ethylene("6-31g")
    b = b.with_geometry(b.xyz + np.array([[0.0, 0.01, 0.0]] + [[0.0, 0.0, 0.0]] * 5))
    assert symmetry.abelian_symmetry(b)[0] < 8


@pytest.mark.parametrize("mol,basis", [("water", "6-31g(d)"), ("ethylene", "6-31g(d)"), ("ethylene", "cc-pvdz"),
                                       ("water", "cc-pvtz")])
def test_fock_of_symmetric_density_is_symmetric(oracle_lib, mol, basis):
    bas = (water if mol == "water" else ethylene)(basis)
    sym = symmetry.abelian_symmetry(bas)
    d = symmetric_density(bas, sym, 5 if mol == "water" else 8, 3)
    dm = unpack(d, bas.nbf)
    assert np.abs(symmetry.project(dm, sym[2], sym[3]) - dm).max() < 1e-14
    f = unpack(oracle_lib.Oracle(bas).fock_jk(d).reshape(-1), bas.nbf)
    assert np.abs(f).max() > 1e-2
    assert np.abs(symmetry.project(f, sym[2], sym[3]) - f).max() < 1e-10
