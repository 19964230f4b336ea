"""Shared pieces of the MRSF sigma tests: the ROHF triplet reference of
OpenQP's h2o_rohf_mrsf-{s,t}_6-31g_hf examples and the full (A-B) matrix of a
sigma routine over the active trial space."""
import numpy as np


def rohf_reference(case, fock2e):
    """ROHF triplet through the given two-electron builder; the closed-shell
    RHF orbitals of the neutral molecule are the guess (the reference starts
    from a Hueckel guess, which lands in the same state)."""
    from openqp_gb300 import onee, scf
    from openqp_gb300.basis import build_basis
    bas = build_basis(case["atoms"], np.array(case["coord_bohr"]).reshape(-1, 3), case["basis"])
    S, T = onee.overlap_kinetic(bas)
    H = T + onee.nuclear(bas)
    en = onee.nuclear_repulsion(bas)
    nel = sum(case["atoms"])
    rr = scf.run_scf(bas.nbf, S, H, en, nel // 2, nel // 2, fock2e, conv=1e-12, dconv=1e-10)
    c0 = rr["C"][0]
    na, nb = nel // 2 + 1, nel // 2 - 1
    r = scf.run_scf(bas.nbf, S, H, en, na, nb, fock2e, kind="rohf", conv=1e-12, dconv=1e-10, maxit=300,
                    guess=(c0, c0))
    C = r["C"][0]
    fa, fb = (C.T @ F @ C for F in r["Fock"])
    return bas, r, C, fa, fb, na, nb


def active(nbf, na, nb, mrst):
    """Trial-space coordinates the MRSF products keep (mrsfmntoia /
    mrsfesum zero the open-open (O2, O2) element, and for triplets also
    (O1, O2) and (O2, O1))."""
    lr1, lr2 = na - 2, na - 1
    drop = {(lr2, lr2)} if mrst == 1 else {(lr2, lr2), (lr1, lr2), (lr2, lr1)}
    return [k for k in range(na * (nbf - nb)) if (k % na, nb + k // na) not in drop]


def mrsf_energies(sigma, nbf, na, nb, mrst, nroots):
    act = active(nbf, na, nb, mrst)
    E = np.eye(na * (nbf - nb))[:, act]
    A = np.asarray(sigma(E))[act]
    assert np.abs(A - A.T).max() < 1e-9
    return np.linalg.eigvalsh(0.5 * (A + A.T))[:nroots]
