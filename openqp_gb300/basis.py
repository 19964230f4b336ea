"""Basis-set data model in OpenQP's ``basis_set`` layout.

A basis is a list of shells, each with an angular momentum, a contraction of
Gaussian primitives (exponents and coefficients), the atom it sits on, and a
``harmonic`` flag (1 = pure spherical for l >= 2).  The arrays produced by
``BasisArrays`` are exactly what ``routec_fock_init`` takes: the fields of
OpenQP's ``basis_set`` type (``source/basis_tools.F90:32-84``):

* ``am[nshell]``, ``ncontr[nshell]``, ``origin[nshell]`` (1-based atom index),
  ``harmonic[nshell]``;
* ``ex[nprim]``, ``cc[nprim]`` concatenated shell by shell, with ``cc``
  already primitive-normalised (``normalize_primitives``,
  ``source/basis_tools.F90:277-303``; OpenQP's Python front end does not
  renormalise the contraction, ``source/basis_api.F90:316-317``);
* ``xyz[3*natom]`` in Bohr.

AO order inside a shell is OpenQP's: s; x y z; xx yy zz xy xz yz
(``source/constants.F90:33-60``); pure d is m = -2..2 (xy, yz, z^2, xz,
x^2-y^2; ``source/integrals/int2_pure_generated.F90:119-129``).
"""
import json
import math
import os
from dataclasses import dataclass, field

import numpy as np

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "basis_data")
_ALIASES = {"6-31g*": "6-31g_d", "6-31g(d)": "6-31g_d", "6-31g_d": "6-31g_d", "6-31g": "6-31g",
            "cc-pvdz": "cc-pvdz", "cc-pvtz": "cc-pvtz", "sto-3g": "sto-3g"}
ANGSTROM = 1.0 / 0.52917721092   # Bohr per Angstrom (CODATA 2010, as in OpenQP's UNITS_ANGSTROM)


def gauss_norm(e, l):
    """Integral of (x^l exp(-e r^2 / 2))^2 ... i.e. OpenQP's gauss_norm(e, l)
    (source/basis_tools.F90:612-623): pi^{3/2} (2l-1)!! / 2^l / e^{l+3/2}."""
    dfact = [1.0, 0.5, 0.75, 1.875, 6.5625, 29.53125, 162.421875]
    return math.pi * math.sqrt(math.pi) * dfact[l] / (e * math.sqrt(e) * e ** l)


def load_basis_set(name):
    key = _ALIASES.get(name.lower())
    if key is None:
        raise ValueError("unknown basis set %r (have %s)" % (name, sorted(set(_ALIASES.values()))))
    with open(os.path.join(_DATA, key + ".json")) as fh:
        return json.load(fh)


@dataclass
class BasisArrays:
    am: np.ndarray
    ncontr: np.ndarray
    origin: np.ndarray
    harmonic: np.ndarray
    ex: np.ndarray
    cc: np.ndarray
    xyz: np.ndarray          # (natom, 3) Bohr
    charges: np.ndarray      # nuclear charges per atom
    nbf: int = 0
    ao_offset: np.ndarray = field(default=None)
    naos: np.ndarray = field(default=None)

    @property
    def nshell(self):
        return len(self.am)

    @property
    def natom(self):
        return len(self.charges)

    def shell_prims(self, s):
        off = int(self.ncontr[:s].sum())
        return self.ex[off:off + self.ncontr[s]], self.cc[off:off + self.ncontr[s]]

    def with_geometry(self, xyz):
        """Same shells on moved atoms (for finite differences)."""
        return BasisArrays(self.am, self.ncontr, self.origin, self.harmonic, self.ex, self.cc,
                           np.ascontiguousarray(np.asarray(xyz, dtype=np.float64).reshape(-1, 3)),
                           self.charges, self.nbf, self.ao_offset, self.naos)


def build_basis(charges, xyz_bohr, basis_name, spherical=None):
    """Shells for a molecule, in atom order, shells of an atom in file order.

    ``spherical=None`` follows the convention the basis was published with
    (OpenQP's ``ispher=auto``); True/False force pure / Cartesian d."""
    bs = load_basis_set(basis_name)
    sph = bs["spherical"] if spherical is None else bool(spherical)
    am, ncontr, origin, harm, ex, cc = [], [], [], [], [], []
    for a, z in enumerate(charges):
        shells = bs["elements"].get(str(int(z)))
        if shells is None:
            raise ValueError("basis %s has no element Z=%d" % (basis_name, z))
        for sh in shells:
            l = sh["l"]
            am.append(l)
            ncontr.append(len(sh["exps"]))
            origin.append(a + 1)
            harm.append(1 if (sph and l >= 2) else 0)
            for e, c in zip(sh["exps"], sh["coefs"]):
                ex.append(e)
                cc.append(c / math.sqrt(gauss_norm(2.0 * e, l)))
    am = np.array(am, dtype=np.int32)
    harm = np.array(harm, dtype=np.int32)
    naos = np.where((harm == 1) & (am >= 2), 2 * am + 1, (am + 1) * (am + 2) // 2).astype(np.int32)
    ao = np.concatenate([[0], np.cumsum(naos)[:-1]]).astype(np.int32)
    return BasisArrays(am=am, ncontr=np.array(ncontr, dtype=np.int32), origin=np.array(origin, dtype=np.int32),
                       harmonic=harm, ex=np.array(ex, dtype=np.float64), cc=np.array(cc, dtype=np.float64),
                       xyz=np.ascontiguousarray(np.asarray(xyz_bohr, dtype=np.float64).reshape(-1, 3)),
                       charges=np.asarray(charges, dtype=np.float64), nbf=int(naos.sum()), ao_offset=ao,
                       naos=naos)


def packed_index(i, j):
    """0-based packed lower-triangle index of (i, j): OpenQP's i(i-1)/2 + j."""
    if i < j:
        i, j = j, i
    return i * (i + 1) // 2 + j


def pack(m):
    """Full symmetric (nbf, nbf) -> packed lower triangle, row-major."""
    n = m.shape[0]
    il = np.tril_indices(n)
    order = np.lexsort((il[1], il[0]))
    return np.ascontiguousarray(m[il[0][order], il[1][order]])


def unpack(p, n):
    m = np.zeros((n, n))
    il = np.tril_indices(n)
    order = np.lexsort((il[1], il[0]))
    m[il[0][order], il[1][order]] = p
    m = m + m.T - np.diag(np.diag(m))
    return m
