"""Host-side one-electron integrals (overlap, kinetic, nuclear attraction).

These are O(nbf^2) set-up quantities for the seeded workloads (the S-metric
Loewdin orthonormalisation of the synthetic densities) and for the SCF driver
around the Fock build; they are not on the GPU hot path.  Obara-Saika
recurrences (Obara & Saika, J. Chem. Phys. 84, 3963 (1986)), vectorised over
the primitive pairs of a shell pair with numpy; normalisation and pure-d
projection follow the AO conventions of ``openqp_gb300.basis``.
"""
import math

import numpy as np
from scipy.special import gammainc, gamma

from .basis import BasisArrays

_CART = {0: [(0, 0, 0)], 1: [(1, 0, 0), (0, 1, 0), (0, 0, 1)],
         2: [(2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1)],
         3: [(3, 0, 0), (0, 3, 0), (0, 0, 3), (2, 1, 0), (2, 0, 1), (1, 2, 0), (0, 2, 1), (1, 0, 2), (0, 1, 2),
             (1, 1, 1)]}
_NORM = {0: [1.0], 1: [1.0, 1.0, 1.0], 2: [1.0, 1.0, 1.0, math.sqrt(3), math.sqrt(3), math.sqrt(3)],
         3: [1.0, 1.0, 1.0] + [math.sqrt(5)] * 6 + [math.sqrt(15)]}
_PURE_D = np.array([[0, 0, 0, 1, 0, 0], [0, 0, 0, 0, 0, 1], [-0.5, -0.5, 1, 0, 0, 0],
                    [0, 0, 0, 0, 1, 0], [math.sqrt(3) / 2, -math.sqrt(3) / 2, 0, 0, 0, 0]])
# pure f (m = -3 .. 3) from normalised Cartesians (int2_pure_generated.F90:134-149)
_a, _b, _c, _d, _e = math.sqrt(10) / 4, 3 / (2 * math.sqrt(2)), math.sqrt(6) / 4, math.sqrt(30) / 20, math.sqrt(1.2)
_g = 3 / (2 * math.sqrt(5))
_PURE_F = np.array([[0, -_a, 0, _b, 0, 0, 0, 0, 0, 0],
                    [0, 0, 0, 0, 0, 0, 0, 0, 0, 1],
                    [0, -_c, 0, -_d, 0, 0, 0, 0, _e, 0],
                    [0, 0, 1, 0, -_g, 0, -_g, 0, 0, 0],
                    [-_c, 0, 0, 0, 0, -_d, 0, _e, 0, 0],
                    [0, 0, 0, 0, math.sqrt(3) / 2, 0, -math.sqrt(3) / 2, 0, 0, 0],
                    [_a, 0, 0, 0, 0, -_b, 0, 0, 0, 0]])
_PURE = {2: _PURE_D, 3: _PURE_F}


def _os_1d(imax, jmax, PA, PB, p):
    """1D overlap-type recursion S[i][j] / sqrt(pi/p) / exp(...) over vectors."""
    o = 0.5 / p
    S = [[None] * (jmax + 1) for _ in range(imax + 1)]
    S[0][0] = np.ones_like(p)
    for i in range(imax + 1):
        for j in range(jmax + 1):
            if i == 0 and j == 0:
                continue
            if i > 0:
                v = PA * S[i - 1][j]
                if i > 1:
                    v = v + (i - 1) * o * S[i - 2][j]
                if j > 0:
                    v = v + j * o * S[i - 1][j - 1]
            else:
                v = PB * S[i][j - 1]
                if j > 1:
                    v = v + (j - 1) * o * S[i][j - 2]
            S[i][j] = v
    return S


def _finish(block, la, lb, ha, hb):
    block = block * np.array(_NORM[la])[:, None] * np.array(_NORM[lb])[None, :]
    if ha and la >= 2:
        block = _PURE[la] @ block
    if hb and lb >= 2:
        block = block @ _PURE[lb].T
    return block


def _pair_data(bas, si, sj):
    ea, ca = bas.shell_prims(si)
    eb, cb = bas.shell_prims(sj)
    A = bas.xyz[bas.origin[si] - 1]
    B = bas.xyz[bas.origin[sj] - 1]
    a = np.repeat(ea, len(eb))
    b = np.tile(eb, len(ea))
    c = np.repeat(ca, len(cb)) * np.tile(cb, len(ca))
    p = a + b
    P = (a[:, None] * A + b[:, None] * B) / p[:, None]
    K = c * np.exp(-a * b / p * np.dot(A - B, A - B))
    return a, b, p, P, A, B, K


def overlap_kinetic(bas: BasisArrays):
    """S and T (nbf x nbf)."""
    n = bas.nbf
    S = np.zeros((n, n))
    T = np.zeros((n, n))
    for si in range(bas.nshell):
        for sj in range(si + 1):
            la, lb = int(bas.am[si]), int(bas.am[sj])
            a, b, p, P, A, B, K = _pair_data(bas, si, sj)
            pref = K * (math.pi / p) ** 1.5
            s1 = [_os_1d(la + 1, lb + 1, P[:, d] - A[d], P[:, d] - B[d], p) for d in range(3)]
            sb = np.zeros((len(_CART[la]), len(_CART[lb])))
            tb = np.zeros_like(sb)
            for ia, ta in enumerate(_CART[la]):
                for ib, tb_ in enumerate(_CART[lb]):
                    ov = [s1[d][ta[d]][tb_[d]] for d in range(3)]
                    kin = []
                    for d in range(3):
                        i, j = ta[d], tb_[d]
                        # T_ij = 1/2 [ i j S(i-1,j-1) + 4 a b S(i+1,j+1) - 2 a j S(i+1,j-1) - 2 b i S(i-1,j+1) ]
                        t = 4 * a * b * s1[d][i + 1][j + 1]
                        if i > 0 and j > 0:
                            t = t + i * j * s1[d][i - 1][j - 1]
                        if j > 0:
                            t = t - 2 * a * j * s1[d][i + 1][j - 1]
                        if i > 0:
                            t = t - 2 * b * i * s1[d][i - 1][j + 1]
                        kin.append(0.5 * t)
                    sb[ia, ib] = np.sum(pref * ov[0] * ov[1] * ov[2])
                    tb[ia, ib] = np.sum(pref * (kin[0] * ov[1] * ov[2] + ov[0] * kin[1] * ov[2] +
                                                ov[0] * ov[1] * kin[2]))
            sb = _finish(sb, la, lb, bas.harmonic[si], bas.harmonic[sj])
            tb = _finish(tb, la, lb, bas.harmonic[si], bas.harmonic[sj])
            oi, oj = bas.ao_offset[si], bas.ao_offset[sj]
            S[oi:oi + sb.shape[0], oj:oj + sb.shape[1]] = sb
            S[oj:oj + sb.shape[1], oi:oi + sb.shape[0]] = sb.T
            T[oi:oi + tb.shape[0], oj:oj + tb.shape[1]] = tb
            T[oj:oj + tb.shape[1], oi:oi + tb.shape[0]] = tb.T
    return S, T


def _boys(mmax, x):
    small = x < 1e-12
    xs = np.where(small, 1.0, x)
    out = []
    for m in range(mmax + 1):
        v = gamma(m + 0.5) * gammainc(m + 0.5, xs) / (2.0 * xs ** (m + 0.5))
        v = np.where(small, 1.0 / (2 * m + 1) - x / (2 * m + 3), v)
        out.append(v)
    return out


def nuclear(bas: BasisArrays, charges=None):
    """Nuclear attraction V (nbf x nbf) of point charges at the atoms."""
    if charges is None:
        charges = bas.charges
    n = bas.nbf
    V = np.zeros((n, n))
    for si in range(bas.nshell):
        for sj in range(si + 1):
            la, lb = int(bas.am[si]), int(bas.am[sj])
            a, b, p, P, A, B, K = _pair_data(bas, si, sj)
            L = la + lb
            vb = np.zeros((len(_CART[la]), len(_CART[lb])))
            for at in range(bas.natom):
                Z = charges[at]
                if Z == 0:
                    continue
                C = bas.xyz[at]
                PC = P - C
                F = _boys(L, p * np.sum(PC * PC, axis=1))
                pref = -Z * 2 * math.pi / p * K
                # Obara-Saika nuclear-attraction recursion on (a|V^(m)|b)
                memo = {}

                def th(ia, ib, m):
                    key = (ia, ib, m)
                    if key in memo:
                        return memo[key]
                    if all(v == 0 for v in ia) and all(v == 0 for v in ib):
                        r = F[m]
                    else:
                        if any(v > 0 for v in ia):
                            d = next(k for k in range(3) if ia[k] > 0)
                            am1 = tuple(v - (k == d) for k, v in enumerate(ia))
                            r = (P[:, d] - A[d]) * th(am1, ib, m) - PC[:, d] * th(am1, ib, m + 1)
                            if am1[d] > 0:
                                am2 = tuple(v - (k == d) for k, v in enumerate(am1))
                                r = r + am1[d] * 0.5 / p * (th(am2, ib, m) - th(am2, ib, m + 1))
                            if ib[d] > 0:
                                bm1 = tuple(v - (k == d) for k, v in enumerate(ib))
                                r = r + ib[d] * 0.5 / p * (th(am1, bm1, m) - th(am1, bm1, m + 1))
                        else:
                            d = next(k for k in range(3) if ib[k] > 0)
                            bm1 = tuple(v - (k == d) for k, v in enumerate(ib))
                            r = (P[:, d] - B[d]) * th(ia, bm1, m) - PC[:, d] * th(ia, bm1, m + 1)
                            if bm1[d] > 0:
                                bm2 = tuple(v - (k == d) for k, v in enumerate(bm1))
                                r = r + bm1[d] * 0.5 / p * (th(ia, bm2, m) - th(ia, bm2, m + 1))
                    memo[key] = r
                    return r

                for ia, ta in enumerate(_CART[la]):
                    for ib, tb_ in enumerate(_CART[lb]):
                        vb[ia, ib] += np.sum(pref * th(ta, tb_, 0))
            vb = _finish(vb, la, lb, bas.harmonic[si], bas.harmonic[sj])
            oi, oj = bas.ao_offset[si], bas.ao_offset[sj]
            V[oi:oi + vb.shape[0], oj:oj + vb.shape[1]] = vb
            V[oj:oj + vb.shape[1], oi:oi + vb.shape[0]] = vb.T
    return V


def nuclear_repulsion(bas: BasisArrays):
    e = 0.0
    for i in range(bas.natom):
        for j in range(i):
            e += bas.charges[i] * bas.charges[j] / np.linalg.norm(bas.xyz[i] - bas.xyz[j])
    return e


def one_electron(bas: BasisArrays, charges=None):
    """S, T, V (nbf x nbf) from the library's threaded C++ routine
    (McMurchie-Davidson); the numpy functions above are its slow restatement."""
    from ._lib import FockError, lib, ptr, _i
    if charges is None:
        charges = bas.charges
    am = np.ascontiguousarray(bas.am, dtype=np.int32)
    nc = np.ascontiguousarray(bas.ncontr, dtype=np.int32)
    org = np.ascontiguousarray(bas.origin, dtype=np.int32)
    ex = np.ascontiguousarray(bas.ex, dtype=np.float64)
    cc = np.ascontiguousarray(bas.cc, dtype=np.float64)
    hm = np.ascontiguousarray(bas.harmonic, dtype=np.int32)
    xyz = np.ascontiguousarray(bas.xyz.reshape(-1), dtype=np.float64)
    ch = np.ascontiguousarray(charges, dtype=np.float64)
    out = []
    for which in range(3):
        m = np.empty((bas.nbf, bas.nbf))
        rc = lib().oqpg_one_electron(len(am), ptr(am, _i), ptr(nc, _i), ptr(org, _i), ptr(ex), ptr(cc), ptr(hm, _i),
                                     int(bas.natom), ptr(xyz), ptr(ch), which, ptr(m))
        if rc != 0:
            raise FockError(rc, "oqpg_one_electron")
        out.append(m)
    return tuple(out)
