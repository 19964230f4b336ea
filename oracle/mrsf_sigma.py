"""Oracle (test infrastructure only): NumPy restatement of OpenQP's MRSF
Davidson sigma step, the native path that the routec_sig session replaces
(modules/tdhf_mrsf_energy.F90:693-830 for mrst 1 / 3 without UMRSF, CAM or
spin-pair rescaling):

  iatogen (tdhf_lib.F90:480-498)        trial vector -> (nbf, nbf) block
  mrsfcbc (tdhf_mrsf_lib.F90:940-1273)  MO -> seven AO densities
  int2_mrsf_data_t build                 the oracle's fock_mrsf (nmat 7)
  triplet sign (tdhf_mrsf_energy.F90:762-766): components 1-6 negated
  mrsfmntoia (tdhf_mrsf_lib.F90:1463-1735) AO -> MO product
  mrsfesum (tdhf_mrsf_lib.F90:1918-2036)   orbital-Fock terms

Indices are 0-based: the open shells are lr1 = nocca - 2 and lr2 = nocca - 1
(Fortran nocca - 1 and nocca); the trial space is X[i, j], i < nocca,
j >= noccb, column-major (i fastest) as the reference packs it.
"""
import numpy as np

ISQRT2 = 1.0 / np.sqrt(2.0)


def iatogen(pv, nbf, nocca, noccb):
    """tdhf_lib.F90:480-498."""
    x = np.zeros((nbf, nbf))
    x[:nocca, noccb:] = np.asarray(pv).reshape(nbf - noccb, nocca).T
    return x


def pack_ia(w, nocca, noccb):
    """The (i fastest) packing loop of mrsfmntoia / mrsfesum."""
    return w[:nocca, noccb:].T.reshape(-1).copy()


def mrsfcbc(va, vb, x, nocca, noccb, mrst):
    """tdhf_mrsf_lib.F90:940-1273 -> (7, nbf, nbf): bo2v, bo1v, bco1, bco2,
    o21v, co12, ball."""
    nbf = va.shape[0]
    lr1, lr2 = nocca - 2, nocca - 1
    f = np.zeros((7, nbf, nbf))
    vbv = vb[:, nocca:]
    t2 = vbv @ x[lr2, nocca:]
    t1 = vbv @ x[lr1, nocca:]
    f[0] = np.outer(va[:, lr2], t2)
    f[1] = np.outer(va[:, lr1], t1)
    f[4] = np.outer(t2, va[:, lr1]) - np.outer(t1, va[:, lr2])
    if noccb > 0:
        c1 = va[:, :noccb] @ x[:noccb, lr1]
        c2 = va[:, :noccb] @ x[:noccb, lr2]
        f[2] = np.outer(c1, vb[:, lr1])
        f[3] = np.outer(c2, vb[:, lr2])
        f[5] = np.outer(vb[:, lr2], c1) - np.outer(vb[:, lr1], c2)
    ball = f[0] + f[1] + f[2] + f[3]
    if noccb > 0:
        tmp = vbv @ x[:noccb, nocca:].T
        ball = ball + va[:, :noccb] @ tmp.T
    a1, a2, b1, b2 = va[:, lr1], va[:, lr2], vb[:, lr1], vb[:, lr2]
    if mrst == 1:
        ball = ball + x[lr2, lr1] * np.outer(a2, b1) + x[lr1, lr2] * np.outer(a1, b2) \
            + x[lr1, lr1] * ISQRT2 * (np.outer(a1, b1) - np.outer(a2, b2))
    elif mrst == 3:
        ball = ball + x[lr1, lr1] * ISQRT2 * (np.outer(a1, b1) + np.outer(a2, b2))
    f[6] = ball
    return f


def mrsfmntoia(f, va, vb, nocca, noccb, mrst):
    """tdhf_mrsf_lib.F90:1463-1735: the seven build outputs -> packed MO
    vector."""
    lr1, lr2 = nocca - 2, nocca - 1
    ado2v, ado1v, adco1, adco2, ao21v, aco12, agdlr = f
    scr = va.T @ agdlr @ vb
    wrk = scr.copy()
    if nocca > 2:
        tmp = ado1v @ vb[:, lr2] + aco12 @ vb[:, lr1]
        wrk[:nocca - 2, lr2] += va[:, :nocca - 2].T @ tmp
        tmp = ado2v @ vb[:, lr1] - aco12 @ vb[:, lr2]
        wrk[:nocca - 2, lr1] += va[:, :nocca - 2].T @ tmp
    tmp = adco2.T @ va[:, lr1] + ao21v.T @ va[:, lr2]
    wrk[lr1, nocca:] += vb[:, nocca:].T @ tmp
    tmp = adco1.T @ va[:, lr2] - ao21v.T @ va[:, lr1]
    wrk[lr2, nocca:] += vb[:, nocca:].T @ tmp
    if mrst == 1:
        wrk[lr1, lr1] = (scr[lr1, lr1] - scr[lr2, lr2]) * ISQRT2
        wrk[lr2, lr2] = 0.0
    elif mrst == 3:
        wrk[lr1, lr1] = (scr[lr1, lr1] + scr[lr2, lr2]) * ISQRT2
        wrk[lr2, lr1] = wrk[lr1, lr2] = wrk[lr2, lr2] = 0.0
    return pack_ia(wrk, nocca, noccb)


def mrsfesum(x, fij, fab, nocca, noccb, mrst):
    """tdhf_mrsf_lib.F90:1918-2036: the orbital-Fock part of the product, packed."""
    nbf = x.shape[0]
    lr1, lr2 = nocca - 2, nocca - 1
    scr = x.copy()
    scr[lr1, lr1] = scr[lr2, lr2] = 0.0
    w = np.zeros((nbf, nbf))
    w[:nocca, noccb:] = scr[:nocca, noccb:] @ fab[noccb:, noccb:].T - fij[:nocca, :nocca] @ scr[:nocca, noccb:]
    xlr = x[lr1, lr1] * ISQRT2
    s2 = -1.0 if mrst == 1 else 1.0      # sign of the lr2 terms
    w[lr1, noccb:] += fab[noccb:, lr1] * xlr
    w[lr2, noccb:] += s2 * fab[noccb:, lr2] * xlr
    w[:nocca, lr1] -= fij[:nocca, lr1] * xlr
    w[:nocca, lr2] -= s2 * fij[:nocca, lr2] * xlr
    dumn = -fij[lr1, :nocca] @ scr[:nocca, lr1] + fab[lr1, noccb:] @ scr[lr1, noccb:] \
        + s2 * (-fij[lr2, :nocca] @ scr[:nocca, lr2] + fab[lr2, noccb:] @ scr[lr2, noccb:])
    w[lr1, lr1] = dumn * ISQRT2 + x[lr1, lr1] * (fab[lr1, lr1] + fab[lr2, lr2] - fij[lr1, lr1] - fij[lr2, lr2]) * 0.5
    if mrst == 1:
        w[lr2, lr2] = 0.0
    else:
        w[lr2, lr1] = w[lr1, lr2] = w[lr2, lr2] = 0.0
    return pack_ia(w, nocca, noccb)


def sigma(fock_mrsf, bvec, va, vb, fa, fb, nocca, noccb, mrst, scale=1.0):
    """(A-B) X for the columns of bvec (ntrial, nv): the native triple with
    fock_mrsf(d3 (nv, 7, nbf, nbf), se, sc) -> f3 the int2_mrsf_data_t build
    (scale_exchange = scale_coulomb = scale, tdhf_mrsf_energy.F90:740-745)."""
    bvec = np.asarray(bvec, dtype=np.float64)
    if bvec.ndim == 1:
        bvec = bvec[:, None]
    nbf = va.shape[0]
    nv = bvec.shape[1]
    xs = [iatogen(bvec[:, v], nbf, nocca, noccb) for v in range(nv)]
    d3 = np.stack([mrsfcbc(va, vb, x, nocca, noccb, mrst) for x in xs])
    f3 = np.asarray(fock_mrsf(d3, scale, scale))
    if mrst == 3:
        f3 = f3.copy()
        f3[:, :6] = -f3[:, :6]
    out = np.empty_like(bvec)
    for v in range(nv):
        out[:, v] = mrsfmntoia(f3[v], va, vb, nocca, noccb, mrst) + mrsfesum(xs[v], fa, fb, nocca, noccb, mrst)
    return out
