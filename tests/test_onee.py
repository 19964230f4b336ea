"""The library's host one-electron integrals (S, T, V for the SCF around the
Fock build) against the oracle's and the numpy restatement, Cartesian and pure
d, and the golden HF energy reached with them.  CPU only."""
import json
import os

import numpy as np
import pytest

from conftest import ROOT, h2o_basis


@pytest.fixture(scope="module")
def built():
    from openqp_gb300 import build
    build.build()


@pytest.mark.parametrize("basis,spherical", [("6-31g*", None), ("cc-pvdz", None), ("sto-3g", None)])
def test_one_electron_matches_oracle(built, oracle_lib, basis, spherical):
    from openqp_gb300 import onee, workloads
    bas = workloads.water_cluster_basis(3, 6.0, 11, basis=basis)
    S, T, V = onee.one_electron(bas)
    o = oracle_lib.Oracle(bas)
    for name, m in zip("STV", (S, T, V)):
        ref = o.one_electron(name)
        assert np.abs(m - ref).max() < 1e-12, name
        assert np.abs(m - m.T).max() == 0.0


def test_one_electron_matches_numpy(built):
    from openqp_gb300 import onee
    bas = h2o_basis("6-31g*")
    S, T, V = onee.one_electron(bas)
    S0, T0 = onee.overlap_kinetic(bas)
    V0 = onee.nuclear(bas)
    assert np.abs(S - S0).max() < 1e-13
    assert np.abs(T - T0).max() < 1e-12
    assert np.abs(V - V0).max() < 1e-12
    assert np.allclose(np.diag(S), 1.0, atol=1e-12)


def test_one_electron_declines_bad_input(built):
    from openqp_gb300 import onee
    from openqp_gb300._lib import FockError
    bas = h2o_basis("6-31g*")
    bad = bas.with_geometry(bas.xyz)
    bad.am = bad.am.copy()
    bad.am[-1] = 4   # g shells are not supported
    with pytest.raises(FockError):
        onee.one_electron(bad)
