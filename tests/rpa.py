"""Full-matrix TDHF (RPA / TDA) singlet excitation energies from a TD build.

The TD build (int2_td_data_t semantics) is applied to every occupied-virtual
unit vector X_ia, as OpenQP's Davidson driver applies it to its trial vectors
(tdhf_energy.F90:211-270: iatogen + orthogonal_transform to the AO density
C_occ X C_vir^T, the int2 run, mntoia back to the MO block, esum adds
(e_a - e_i) X).  For the small test molecules the whole A+B / A-B matrices
are built this way and diagonalised exactly instead of iteratively.
"""
import numpy as np


def canonical_orbitals(S, F):
    w, U = np.linalg.eigh(S)
    X = U / np.sqrt(w)
    e, Cp = np.linalg.eigh(X.T @ F @ X)
    return e, X @ Cp


def unit_densities(C, nocc):
    n = C.shape[0]
    Co, Cv = C[:, :nocc], C[:, nocc:]
    nv = n - nocc
    out = np.empty((nocc * nv, n, n))
    k = 0
    for i in range(nocc):
        for a in range(nv):
            out[k] = np.outer(Co[:, i], Cv[:, a])
            k += 1
    return out


def mo_block(mats, C, nocc):
    Co, Cv = C[:, :nocc], C[:, nocc:]
    return np.array([(Co.T @ m @ Cv).reshape(-1) for m in mats]).T


def rpa_energies(td_build, C, e, nocc):
    """td_build(x, flags) -> (apb, amb) for x (nvec, n, n); flags as OQPG_TD_*."""
    x = unit_densities(C, nocc)
    de = (e[nocc:][None, :] - e[:nocc][:, None]).reshape(-1)
    pa, ma = td_build(x, 3)
    apb = mo_block(pa, C, nocc) + np.diag(de)
    amb = mo_block(ma, C, nocc) + np.diag(de)
    w, U = np.linalg.eigh(0.5 * (amb + amb.T))
    sq = U @ np.diag(np.sqrt(w)) @ U.T
    return np.sqrt(np.sort(np.linalg.eigvalsh(sq @ apb @ sq))), apb, amb


def tda_energies(td_build, C, e, nocc):
    x = unit_densities(C, nocc)
    de = (e[nocc:][None, :] - e[:nocc][:, None]).reshape(-1)
    pa, ma = td_build(x, 4 | 8)
    a = mo_block(0.5 * pa + ma, C, nocc) + np.diag(de)
    return np.sort(np.linalg.eigvalsh(0.5 * (a + a.T)))
