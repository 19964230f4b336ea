"""Seeded synthetic molecules and densities for the Fock-build workloads.

No public benchmark suite is involved: every input is generated from a seed
(``numpy.random.default_rng``) with the shapes the workloads name:

* water clusters -- O-H 0.9572 A, HOH 104.52 deg, each molecule rotated by a
  Haar-random quaternion, oxygens uniform in a cube with all O-O >= 2.7 A
  (rejection sampling);
* all-trans alkanes CnH(2n+2) -- C-C 1.54 A, C-H 1.09 A, tetrahedral angles,
  uniform +-0.02 A jitter on every coordinate;
* densities D = 2 C_occ C_occ^T (RHF) or D_a = C_a C_a^T, D_b = C_b C_b^T
  (UHF/ROHF), with C drawn from N(0, 1) and made S-orthonormal by Loewdin
  orthogonalisation C <- C (C^T S C)^{-1/2}.
"""
import math

import numpy as np

from .basis import ANGSTROM, build_basis, pack
from .onee import overlap_kinetic

ROH = 0.9572
THETA = math.radians(104.52)
TETRA = math.acos(-1.0 / 3.0)


def _quat_rot(q):
    a, b, c, d = q / np.linalg.norm(q)
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                     [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def water_cluster(nwater, edge_angstrom, seed):
    """(charges, xyz_bohr) of a seeded water cluster."""
    rng = np.random.default_rng(seed)
    local = np.array([[0.0, 0.0, 0.0],
                      [ROH * math.sin(THETA / 2), 0.0, ROH * math.cos(THETA / 2)],
                      [-ROH * math.sin(THETA / 2), 0.0, ROH * math.cos(THETA / 2)]])
    oxy = []
    tries = 0
    while len(oxy) < nwater:
        tries += 1
        if tries > 200000:
            raise RuntimeError("cannot place %d waters in a %.2f A cube" % (nwater, edge_angstrom))
        o = rng.uniform(0.0, edge_angstrom, 3)
        if all(np.linalg.norm(o - p) >= 2.7 for p in oxy):
            oxy.append(o)
    xyz, z = [], []
    for o in oxy:
        R = _quat_rot(rng.standard_normal(4))
        for k, atom in enumerate(local):
            xyz.append(o + R @ atom)
            z.append(8 if k == 0 else 1)
    return np.array(z, dtype=np.float64), np.array(xyz) * ANGSTROM


def cube_edge_like_c1(nwater):
    """Cube edge giving the number density of four waters in a 6 A cube."""
    return (6.0 ** 3 / 4.0 * nwater) ** (1.0 / 3.0)


def alkane(ncarbon, seed, jitter=0.02):
    """(charges, xyz_bohr) of an all-trans CnH(2n+2) chain."""
    rng = np.random.default_rng(seed)
    dcc, dch = 1.54, 1.09
    hx = dcc * math.sin(TETRA / 2)
    hy = dcc * math.cos(TETRA / 2)
    C = np.array([[k * hx, (k % 2) * hy, 0.0] for k in range(ncarbon)])
    H = []
    ez = np.array([0.0, 0.0, 1.0])
    for k in range(ncarbon):
        nb = []
        for j in (k - 1, k + 1):
            if 0 <= j < ncarbon:
                nb.append(C[j])
            else:   # virtual continuation of the zig-zag marks the in-plane H of a methyl
                nb.append(np.array([j * hx, (j % 2) * hy, 0.0]))
        u1 = (nb[0] - C[k]) / np.linalg.norm(nb[0] - C[k])
        u2 = (nb[1] - C[k]) / np.linalg.norm(nb[1] - C[k])
        b = -(u1 + u2)
        b /= np.linalg.norm(b)
        for s in (+1, -1):
            H.append(C[k] + dch * (math.cos(TETRA / 2) * b + s * math.sin(TETRA / 2) * ez))
        for j, u in ((k - 1, u1), (k + 1, u2)):
            if not (0 <= j < ncarbon):
                H.append(C[k] + dch * u)
    xyz = np.vstack([C, np.array(H)])
    xyz = xyz + rng.uniform(-jitter, jitter, xyz.shape)
    z = np.array([6.0] * ncarbon + [1.0] * len(H))
    return z, xyz * ANGSTROM


def loewdin_columns(S, ncol, rng):
    C = rng.standard_normal((S.shape[0], ncol))
    M = C.T @ S @ C
    w, U = np.linalg.eigh(M)
    return C @ (U * (1.0 / np.sqrt(w))) @ U.T


def density(bas, nocc, seed, S=None):
    """Packed RHF density D = 2 C C^T with nocc Loewdin-orthonormal columns."""
    if S is None:
        S, _ = overlap_kinetic(bas)
    rng = np.random.default_rng(seed)
    C = loewdin_columns(S, nocc, rng)
    return pack(2.0 * C @ C.T)


def transition_densities(bas, nocc, nvec, seed, S=None):
    """(nvec, nbf, nbf) AO transition densities X_v = C_occ Y_v C_vir^T of
    seeded unit-norm occupied-virtual amplitudes Y_v, with C a full
    Loewdin-orthonormal set of columns (the AO form of TDHF trial vectors,
    tdhf_energy.F90:211-218)."""
    if S is None:
        S, _ = overlap_kinetic(bas)
    rng = np.random.default_rng(seed)
    n = S.shape[0]
    C = loewdin_columns(S, n, rng)
    Co, Cv = C[:, :nocc], C[:, nocc:]
    out = np.empty((nvec, n, n))
    for v in range(nvec):
        Y = rng.standard_normal((nocc, n - nocc))
        Y /= np.linalg.norm(Y)
        out[v] = Co @ Y @ Cv.T
    return out


def mrsf_session_inputs(bas, nocca, noccb, nvec, seed, S=None):
    """Inputs of an MRSF sigma session: a full Loewdin-orthonormal MO set C
    (alpha = beta, as for an ROHF reference), MO Fock matrices with an
    ascending orbital-energy ladder plus a small symmetric coupling, and nvec
    seeded unit-norm trial vectors (nocca (nbf - noccb), nvec)."""
    if S is None:
        S, _ = overlap_kinetic(bas)
    rng = np.random.default_rng(seed)
    n = S.shape[0]
    C = loewdin_columns(S, n, rng)
    eps = np.linspace(-1.5, 2.5, n)
    fmo = []
    for _ in range(2):
        w = rng.standard_normal((n, n)) * 0.01
        fmo.append(np.diag(eps) + 0.5 * (w + w.T))
    b = rng.standard_normal((nocca * (n - noccb), nvec))
    b /= np.linalg.norm(b, axis=0)
    return C, fmo[0], fmo[1], b


def mrsf_gradient_inputs(bas, seed, S=None):
    """Inputs of an MRSF two-electron gradient: raw alpha / beta densities of
    a triplet reference (nocca = noccb + 2, Loewdin-orthonormal columns), a
    symmetric relaxed difference density pair and seven general response
    densities of the same scale (seeded); (2, n, n), (2, n, n), (7, n, n)."""
    from .basis import unpack
    n = bas.nbf
    nel = nelectrons(bas)
    du = density_open(bas, nel // 2 + 1, nel // 2 - 1, seed, S=S)
    d = np.stack([unpack(du[0], n), unpack(du[1], n)])
    if S is None:
        S, _ = overlap_kinetic(bas)
    rng = np.random.default_rng(seed + 1)
    C = loewdin_columns(S, 2 * (nel // 2 + 1), rng)
    h = C.shape[1] // 2
    p = np.stack([0.1 * (C[:, :h] @ C[:, h:].T + C[:, h:] @ C[:, :h].T)] * 2)
    spc = np.stack([0.1 * C[:, (k % h):(k % h) + 1] @ C[:, h + (k % h):h + (k % h) + 1].T for k in range(6)]
                   + [0.1 * C[:, :h] @ C[:, h:].T])
    return d, p, spc


def density_open(bas, nalpha, nbeta, seed, S=None):
    """Packed (2, ntri) alpha/beta densities."""
    if S is None:
        S, _ = overlap_kinetic(bas)
    rng = np.random.default_rng(seed)
    Ca = loewdin_columns(S, nalpha, rng)
    Cb = Ca[:, :nbeta] if nbeta <= nalpha else loewdin_columns(S, nbeta, rng)
    return np.stack([pack(Ca @ Ca.T), pack(Cb @ Cb.T)])


def water_cluster_basis(nwater, edge, seed, basis="6-31g(d)", spherical=None):
    z, xyz = water_cluster(nwater, edge, seed)
    return build_basis(z, xyz, basis, spherical=spherical)


def nelectrons(bas, charge=0):
    return int(round(bas.charges.sum())) - charge


def water_batch(nclusters, seed, nmin=1, nmax=16, basis="6-31g", overlap=None):
    """Batch of seeded water clusters of uneven size: n ~ U{nmin..nmax} waters
    each, placed in a cube whose edge keeps the number density of four waters
    in a 6 A cube.  Returns (sizes, bases, packed RHF densities); the overlap
    for each Loewdin step comes from overlap(bas), by default the library's
    host routine."""
    if overlap is None:
        from .onee import one_electron

        def overlap(b):
            return one_electron(b)[0]
    rng = np.random.default_rng(seed)
    sizes = rng.integers(nmin, nmax + 1, nclusters)
    bases, dens = [], []
    for k, n in enumerate(sizes):
        bas = water_cluster_basis(int(n), cube_edge_like_c1(int(n)), seed * 100003 + k, basis)
        S = overlap(bas)
        bases.append(bas)
        dens.append(density(bas, nelectrons(bas) // 2, seed * 100003 + k, S=S))
    return [int(v) for v in sizes], bases, dens


def d_lattice(n, spacing_angstrom, dexp):
    """One uncontracted Cartesian d shell of exponent dexp on every point of an
    n x n x n cubic lattice (spacing in A), point charges 6 on the sites: a
    synthetic basis in which every shell quartet is (dd|dd)."""
    import math
    from .basis import BasisArrays, gauss_norm
    g = np.arange(n) * spacing_angstrom * ANGSTROM
    xyz = np.array([[x, y, z] for x in g for y in g for z in g])
    m = len(xyz)
    am = np.full(m, 2, dtype=np.int32)
    naos = np.full(m, 6, dtype=np.int32)
    return BasisArrays(am=am, ncontr=np.ones(m, dtype=np.int32), origin=np.arange(1, m + 1, dtype=np.int32),
                       harmonic=np.zeros(m, dtype=np.int32), ex=np.full(m, float(dexp)),
                       cc=np.full(m, 1.0 / math.sqrt(gauss_norm(2.0 * dexp, 2))), xyz=xyz,
                       charges=np.full(m, 6.0), nbf=6 * m,
                       ao_offset=np.arange(0, 6 * m, 6, dtype=np.int32), naos=naos)
