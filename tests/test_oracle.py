"""CPU tests that pin the oracle (the CPU restatement of OpenQP's Fock build)
before it is trusted as the checker of the GPU path.

Pins, in order of strength:
  * OpenQP's own golden HF energies (examples/HF, examples/NMR) reproduced by
    an SCF whose two-electron part is the oracle's fock_jk restatement;
  * J/K semantics of the restated storeints + digestion + scaling against a
    dense ERI contraction;
  * Rys ERIs against an independent McMurchie-Davidson code;
  * the Rys tables against 60-digit values.
"""
import json
import os

import numpy as np
import pytest

from conftest import ROOT, h2o_basis

GOLD = json.load(open(os.path.join(ROOT, "tests", "golden", "hf_golden.json")))["cases"]


def test_rys_tables_match_exact_values(oracle_lib):
    g = json.load(open(os.path.join(ROOT, "tests", "golden", "rys_exact.json")))
    worst = 0.0
    for c in g["cases"]:
        x, w = oracle_lib.rys(c["n"], c["X"])
        worst = max(worst, np.max(np.abs(x - c["x"]) / np.abs(c["x"])), np.max(np.abs(w - c["w"]) / np.abs(c["w"])))
    assert worst < 1e-14


@pytest.mark.parametrize("basis", ["6-31g*", "cc-pvdz"])
def test_rys_matches_mcmurchie_davidson(oracle_lib, basis):
    bas = h2o_basis(basis)
    o = oracle_lib.Oracle(bas)
    ns = len(bas.am)
    worst = 0.0
    rng = np.random.default_rng(3)
    for _ in range(250):
        i, j, k, l = (int(v) for v in rng.integers(0, ns, 4))
        worst = max(worst, np.abs(o.eri_quartet(i, j, k, l) - o.md_quartet(i, j, k, l)).max())
    assert worst < 1e-12


@pytest.mark.parametrize("basis", ["6-31g*", "cc-pvdz"])
def test_fock_jk_matches_dense_contraction(oracle_lib, basis):
    from openqp_gb300 import workloads
    from openqp_gb300.basis import unpack
    bas = h2o_basis(basis)
    o = oracle_lib.Oracle(bas, cutoff=1e-12)
    n = o.nbf
    eri = o.eri_dense()
    D = workloads.density(bas, 5, 0)
    Df = unpack(D, n)
    J = np.einsum("ijkl,kl->ij", eri, Df)
    K = np.einsum("ikjl,kl->ij", eri, Df)
    F = o.fock_jk(D)
    assert np.abs(unpack(F[0], n) - (J - 0.5 * K)).max() < 1e-11
    Dab = workloads.density_open(bas, 5, 4, 1)
    Da, Db = unpack(Dab[0], n), unpack(Dab[1], n)
    Jt = np.einsum("ijkl,kl->ij", eri, Da + Db)
    F2 = o.fock_jk(Dab, se=0.7, sc=0.9)
    assert np.abs(unpack(F2[0], n) - (0.9 * Jt - 0.7 * np.einsum("ikjl,kl->ij", eri, Da))).max() < 1e-11
    assert np.abs(unpack(F2[1], n) - (0.9 * Jt - 0.7 * np.einsum("ikjl,kl->ij", eri, Db))).max() < 1e-11


def test_one_electron_two_implementations_agree(oracle_lib):
    from openqp_gb300 import onee
    for basis in ("6-31g*", "cc-pvdz"):
        bas = h2o_basis(basis)
        o = oracle_lib.Oracle(bas)
        S, T = onee.overlap_kinetic(bas)
        assert np.abs(o.one_electron("S") - S).max() < 1e-13
        assert np.abs(o.one_electron("T") - T).max() < 1e-12
        assert np.abs(o.one_electron("V") - onee.nuclear(bas)).max() < 1e-12


@pytest.mark.parametrize("case", [c for c in GOLD if "GRADIENT" not in c["source"]], ids=lambda c: c["source"].split("/")[-1])
def test_golden_hf_energy(oracle_lib, case):
    """OpenQP's own example energies; their CI gate is 4 decimals, we ask 1e-7."""
    from openqp_gb300 import onee, scf
    from openqp_gb300.basis import build_basis
    bas = build_basis(case["atoms"], np.array(case["coord_bohr"]).reshape(-1, 3), case["basis"])
    o = oracle_lib.Oracle(bas, cutoff=1e-10)
    S, T = onee.overlap_kinetic(bas)
    H = T + onee.nuclear(bas)
    nel = int(sum(case["atoms"]))
    nunp = case["multiplicity"] - 1
    na, nb = (nel + nunp) // 2, (nel - nunp) // 2
    kind = case["scf"]
    r = scf.run_scf(o.nbf, S, H, onee.nuclear_repulsion(bas), na, nb,
                    lambda d: o.fock_jk(d, urohf=(kind != "rhf")), kind=kind, conv=1e-11)
    assert r["converged"]
    assert abs(r["energy"] - case["energy"]) < 1e-7
