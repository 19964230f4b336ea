"""Abelian point-group symmetry of a molecule in its given frame, as the
signed AO permutations the petite list needs (``FockBuilder.set_symmetry``,
``oqpg_set_symmetry``).

OpenQP's Python front end finds the point group and stages, per operation,
the image of every shell and every AO with a sign (tagarrays
``OQP_sym_shell_map``, ``OQP_sym_ao_target``, ``OQP_sym_ao_sign``; consumed by
``int2_compute_t_enable_petite``, ``source/integrals/int2.F90:312-365``, and
``symmetrize_skeleton_signed``, ``source/scf_addons.F90:1563-1615``).  This
module covers the same abelian tier for a molecule whose symmetry elements
lie on the coordinate axes and planes: the operations are the diagonal sign
matrices diag(sx, sy, sz) (identity, the three C2 axes, the three mirror
planes, inversion) that map every atom onto an atom of the same element, a
subgroup of D2h.  Each maps a shell onto the same shell of the image atom,
and each AO onto the same component of the image shell times a sign: for a
Cartesian x^a y^b z^c the sign is sx^a sy^b sz^c, for the pure d and f
components (OpenQP's order, m = -l .. l) the parity of their solid harmonic.
"""
import itertools

import numpy as np

# parity exponents (a, b, c) of the pure components: sign = sx^a sy^b sz^c
_PURE = {
    2: [(1, 1, 0), (0, 1, 1), (0, 0, 0), (1, 0, 1), (0, 0, 0)],               # xy, yz, z2, xz, x2-y2
    3: [(0, 1, 0), (1, 1, 1), (0, 1, 0), (0, 0, 1), (1, 0, 0), (0, 0, 1), (1, 0, 0)],
}


def _cart(l):
    """Cartesian exponents in OpenQP's order (constants.F90:33-60)."""
    if l == 0:
        return [(0, 0, 0)]
    if l == 1:
        return [(1, 0, 0), (0, 1, 0), (0, 0, 1)]
    if l == 2:
        return [(2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1)]
    return [(3, 0, 0), (0, 3, 0), (0, 0, 3), (2, 1, 0), (2, 0, 1), (1, 2, 0), (0, 2, 1), (1, 0, 2), (0, 1, 2),
            (1, 1, 1)]


def _component_parities(bas, s):
    l = int(bas.am[s])
    if int(bas.harmonic[s]) and l >= 2:
        return _PURE[l]
    return _cart(l)


def abelian_symmetry(bas, tol=1e-6):
    """(nops, shell_map, ao_target, ao_sign) of the operations diag(+-1, +-1,
    +-1) that leave the molecule invariant (atoms of the same charge onto each
    other, within tol Bohr): int32 (nops, nshell) and (nops, nbf), float64
    (nops, nbf), 0-based, the identity first.  nops is 1, 2, 4 or 8."""
    xyz = np.asarray(bas.xyz, dtype=np.float64).reshape(-1, 3)
    z = np.asarray(bas.charges)
    ops, atom_maps = [], []
    for signs in itertools.product((1, -1), repeat=3):
        img = xyz * np.array(signs, dtype=np.float64)
        amap = []
        for a in range(len(xyz)):
            d = np.linalg.norm(xyz - img[a], axis=1)
            b = int(np.argmin(d))
            if d[b] > tol or z[b] != z[a]:
                amap = None
                break
            amap.append(b)
        if amap is not None:
            ops.append(signs)
            atom_maps.append(amap)
    # shells of each atom in order (the same basis on atoms of one element)
    first = {}
    for s in range(bas.nshell):
        first.setdefault(int(bas.origin[s]) - 1, s)
    nops, ns, nbf = len(ops), bas.nshell, bas.nbf
    shell_map = np.zeros((nops, ns), dtype=np.int32)
    ao_target = np.zeros((nops, nbf), dtype=np.int32)
    ao_sign = np.zeros((nops, nbf), dtype=np.float64)
    for k, (signs, amap) in enumerate(zip(ops, atom_maps)):
        for s in range(ns):
            a = int(bas.origin[s]) - 1
            t = first[amap[a]] + (s - first[a])
            if bas.am[t] != bas.am[s] or bas.ncontr[t] != bas.ncontr[s]:
                raise ValueError("atoms %d and %d carry different shells" % (a, amap[a]))
            shell_map[k, s] = t
            for i, (ex, ey, ez) in enumerate(_component_parities(bas, s)):
                mu = int(bas.ao_offset[s]) + i
                ao_target[k, mu] = int(bas.ao_offset[t]) + i
                ao_sign[k, mu] = float(signs[0] ** ex * signs[1] ** ey * signs[2] ** ez)
    return nops, shell_map, ao_target, ao_sign


def project(m, ao_target, ao_sign):
    """The totally symmetric component (1/|G|) sum_op T m T^T of a full
    (nbf, nbf) matrix: the projector of the petite-list symmetrisation."""
    out = np.zeros_like(m)
    for t, sg in zip(ao_target, ao_sign):
        ms = m * sg[:, None] * sg[None, :]
        out[np.ix_(t, t)] += ms
    return out / len(ao_target)
