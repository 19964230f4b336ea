"""Generate the Rys quadrature tables used by the device kernels and the oracle.

For n = 1..7 Rys roots, the quadrature
    int_0^1 f(t^2) exp(-X t^2) dt  ~=  sum_i w_i(X) f(x_i(X)),   x_i = t_i^2,
is exact for polynomials f of degree <= 2n-1.  Its nodes and weights are the
Gauss nodes/weights of the measure exp(-X x) / (2 sqrt(x)) dx on [0, 1], whose
moments are the Boys functions F_k(X).

Method (our own, not the polynomial fits of OpenQP's rys.F90):
  * exact values at any X come from F_0..F_{2n-1}(X) in 60-digit arithmetic
    (series for the top order, downward recursion), the Chebyshev algorithm
    for the three-term recurrence, and the eigen-decomposition of the Jacobi
    matrix (Golub-Welsch), all with mpmath;
  * X in [0, 32) is cut into intervals of width 1/4, X in [32, XMAX(n)) into
    unit intervals; on each interval every x_i and w_i is fitted by a degree-7
    Chebyshev interpolant, stored as monomial coefficients in the local
    variable s = 2 (X - a) / h - 1 in [-1, 1] (Horner evaluation: one FMA per
    coefficient);
  * X >= XMAX(n) uses the large-X limit x_i = r_i^2 / X, w_i = W_i / sqrt(X)
    with (r_i, W_i) the positive nodes and weights of 2n-point Gauss-Hermite.

The script writes ``rys_tables.inc`` (C/C++/CUDA include) next to itself and a
golden file of exact values for the tests.  It needs mpmath, so it runs only
where the tables are regenerated; the generated include is committed.

Usage: python gen_rys_tables.py [golden_json_path]
"""
import json
import multiprocessing as mpr
import os
import sys

import mpmath as mp
import numpy as np

DPS = 60
NMAX = 7
NCOEF = 8             # degree-7 interpolants
NCOEF_F32 = 5         # degree-4 interpolants for the FP32 quartets
X_SPLIT = 32          # quarter-unit intervals below, unit intervals above
H_LO = 0.25
W_HI = 1
XMAX = {1: 40, 2: 48, 3: 56, 4: 64, 5: 72, 6: 80, 7: 88}


def boys_list(X, mmax):
    mp.mp.dps = DPS
    X = mp.mpf(X)
    if X == 0:
        return [mp.mpf(1) / (2 * m + 1) for m in range(mmax + 1)]
    s = mp.mpf(0)
    term = mp.mpf(1) / (2 * mmax + 1)
    i = 0
    eps = mp.mpf(10) ** (-DPS)
    while True:
        s += term
        i += 1
        term = term * 2 * X / (2 * mmax + 2 * i + 1)
        if term < s * eps:
            break
    ex = mp.exp(-X)
    F = [mp.mpf(0)] * (mmax + 1)
    F[mmax] = ex * s
    for k in range(mmax - 1, -1, -1):
        F[k] = (2 * X * F[k + 1] + ex) / (2 * k + 1)
    return F


def rys_exact(X, n):
    """Exact (60-digit) Rys nodes x_i = t_i^2 and weights, ascending nodes."""
    mp.mp.dps = DPS
    mu = boys_list(X, 2 * n - 1)
    sig_prev = [mp.mpf(0)] * (2 * n)
    sig = list(mu)
    alpha = [mu[1] / mu[0]]
    beta = [mu[0]]
    for k in range(1, n):
        new = [mp.mpf(0)] * (2 * n)
        for l in range(k, 2 * n - k):
            new[l] = sig[l + 1] - alpha[k - 1] * sig[l] - beta[k - 1] * sig_prev[l]
        alpha.append(new[k + 1] / new[k] - sig[k] / sig[k - 1])
        beta.append(new[k] / sig[k - 1])
        sig_prev, sig = sig, new
    J = mp.matrix(n, n)
    for i in range(n):
        J[i, i] = alpha[i]
        if i + 1 < n:
            J[i, i + 1] = J[i + 1, i] = mp.sqrt(beta[i + 1])
    E, Q = mp.eigsy(J)
    res = sorted([(E[i], beta[0] * Q[0, i] ** 2) for i in range(n)])
    return [r[0] for r in res], [r[1] for r in res]


def hermite_half(n):
    """Positive nodes r_i (as r_i^2) and weights of 2n-point Gauss-Hermite."""
    mp.mp.dps = DPS
    m = 2 * n
    J = mp.matrix(m, m)
    for k in range(1, m):
        J[k - 1, k] = J[k, k - 1] = mp.sqrt(mp.mpf(k) / 2)
    E, Q = mp.eigsy(J)
    out = sorted([(E[i], mp.sqrt(mp.pi) * Q[0, i] ** 2) for i in range(m) if E[i] > 0])
    return [e ** 2 for e, _ in out], [w for _, w in out]


def intervals(n):
    iv = [(k * H_LO, H_LO) for k in range(int(X_SPLIT / H_LO))]
    a = X_SPLIT
    while a < XMAX[n]:
        iv.append((float(a), float(W_HI)))
        a += W_HI
    return iv


def interval_of(X):
    """(index, start, width) of the interval holding X < XMAX."""
    if X < X_SPLIT:
        k = int(X / H_LO)
        return k, k * H_LO, H_LO
    k0 = int(X_SPLIT / H_LO)
    k = k0 + int((X - X_SPLIT) / W_HI)
    return k, X_SPLIT + (k - k0) * W_HI, float(W_HI)


def fit_interval(args):
    n, a, h, ncoef = args
    mp.mp.dps = DPS
    D = ncoef - 1
    k = np.arange(D + 1)
    nodes = np.cos(np.pi * (k + 0.5) / (D + 1))
    vals = [rys_exact(mp.mpf(a) + mp.mpf(h) * (mp.mpf(float(s)) + 1) / 2, n) for s in nodes]
    rows = []
    for r in range(n):
        for which in (0, 1):
            f = np.array([float(v[which][r]) for v in vals])
            c = np.polynomial.chebyshev.chebfit(nodes, f, D)
            rows.append(np.polynomial.chebyshev.cheb2poly(c))
    return rows


def emit_table(lines, name, tables, ncoef):
    vals = []
    for n in range(1, NMAX + 1):
        for rows in tables[n]:
            for c in rows:
                vals.extend(repr(float(v)) for v in c)
    lines.append("#define %s_SIZE %d" % (name, len(vals)))
    lines.append("RYS_STORAGE double %s[%s_SIZE] = {" % (name, name))
    for i in range(0, len(vals), 4):
        lines.append("  " + ", ".join(vals[i:i + 4]) + ",")
    lines.append("};")


def horner(c, s):
    acc = c[-1]
    for v in c[-2::-1]:
        acc = acc * s + v
    return acc


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    golden_path = sys.argv[1] if len(sys.argv) > 1 else None
    jobs = []
    for ncoef in (NCOEF, NCOEF_F32):
        for n in range(1, NMAX + 1):
            for (a, h) in intervals(n):
                jobs.append((n, a, h, ncoef))
    with mpr.get_context("spawn").Pool() as pool:
        fits = pool.map(fit_interval, jobs)
    tables = {n: [] for n in range(1, NMAX + 1)}
    tables_f32 = {n: [] for n in range(1, NMAX + 1)}
    for (n, a, h, ncoef), rows in zip(jobs, fits):
        (tables if ncoef == NCOEF else tables_f32)[n].append(rows)
    herm = {n: hermite_half(n) for n in range(1, NMAX + 1)}

    lines = [
        "// Generated by gen_rys_tables.py -- do not edit.",
        "// Rys nodes x_i = t_i^2 and weights w_i for n = 1..%d roots." % NMAX,
        "// Interval k covers [a_k, a_k + h_k): width %g below %d, width %d above," % (H_LO, X_SPLIT, W_HI),
        "// up to RYS_XMAX[n]; per interval and root: %d monomial coefficients of x_i," % NCOEF,
        "// then %d of w_i, in s = 2 (X - a_k) / h_k - 1, lowest order first." % NCOEF,
        "#ifndef RYS_STORAGE",
        "#define RYS_STORAGE static const",
        "#endif",
        "#define RYS_NMAX %d" % NMAX,
        "#define RYS_NCOEF %d" % NCOEF,
        "#define RYS_X_SPLIT %d" % X_SPLIT,
        "#define RYS_LO_PER_UNIT %d" % int(round(1 / H_LO)),
        "#define RYS_W_HI %d" % W_HI,
    ]
    lines.append("RYS_STORAGE double RYS_XMAX[%d] = {0.0, %s};" % (
        NMAX + 1, ", ".join("%d.0" % XMAX[n] for n in range(1, NMAX + 1))))
    offs = [0]
    for n in range(1, NMAX + 1):
        offs.append(offs[-1] + len(tables[n]) * 2 * n * NCOEF)
    lines.append("RYS_STORAGE int RYS_OFFSET[%d] = {%s};" % (NMAX + 1, ", ".join(str(o) for o in offs[:-1])))
    emit_table(lines, "RYS_TABLE", tables, NCOEF)
    lines.append("// Same intervals, degree-%d interpolants (relative error ~1e-8): the root" % (NCOEF_F32 - 1))
    lines.append("// evaluation of the FP32 quartets of the precision-split build.")
    lines.append("#define RYS_NCOEF_F32 %d" % NCOEF_F32)
    emit_table(lines, "RYS_TABLE_F32", tables_f32, NCOEF_F32)
    vals = []
    for n in range(1, NMAX + 1):
        for rows in tables_f32[n]:
            for c in rows:
                vals.extend("%.9ef" % float(v) for v in c)
    lines.append("// The same degree-%d table rounded to FP32." % (NCOEF_F32 - 1))
    lines.append("RYS_STORAGE float RYS_TABLE_F32F[RYS_TABLE_F32_SIZE] = {")
    for i in range(0, len(vals), 4):
        lines.append("  " + ", ".join(vals[i:i + 4]) + ",")
    lines.append("};")
    hr, hw = [], []
    for n in range(1, NMAX + 1):
        hr.extend(repr(float(v)) for v in herm[n][0])
        hw.extend(repr(float(v)) for v in herm[n][1])
    lines.append("// large-X limit: x_i = RYS_HERM_R2[o+i] / X, w_i = RYS_HERM_W[o+i] / sqrt(X), o = n(n-1)/2")
    lines.append("RYS_STORAGE double RYS_HERM_R2[%d] = {%s};" % (len(hr), ", ".join(hr)))
    lines.append("RYS_STORAGE double RYS_HERM_W[%d] = {%s};" % (len(hw), ", ".join(hw)))
    with open(os.path.join(here, "rys_tables.inc"), "w") as fh:
        fh.write("\n".join(lines) + "\n")

    # self-check of the tables in float64 against exact values
    rng = np.random.default_rng(7)
    worst = 0.0
    golden = {"note": "exact Rys nodes/weights (mpmath, 60 digits) for the table tests", "cases": []}
    for n in range(1, NMAX + 1):
        xs = list(rng.uniform(0, 1, 20)) + list(rng.uniform(0, XMAX[n] + 10, 60)) + \
            [0.0, 1e-12, 0.999999, 31.999, 32.0, XMAX[n] - 1e-9, XMAX[n], XMAX[n] + 1, 200.0, 5000.0]
        for X in xs:
            ex = rys_exact(X, n)
            golden["cases"].append({"n": n, "X": float(X), "x": [float(v) for v in ex[0]],
                                    "w": [float(v) for v in ex[1]]})
            if X < XMAX[n]:
                k, a, h = interval_of(X)
                s = 2 * (X - a) / h - 1
                rows = tables[n][k]
                ap = [(horner(rows[2 * r], s), horner(rows[2 * r + 1], s)) for r in range(n)]
            else:
                o = 0
                ap = [(herm[n][0][r] / X, herm[n][1][r] / np.sqrt(X)) for r in range(n)]
            for r in range(n):
                worst = max(worst, abs(float(ap[r][0]) - float(ex[0][r])) / float(ex[0][r]),
                            abs(float(ap[r][1]) - float(ex[1][r])) / float(ex[1][r]))
    print("max relative error of the tables: %.3e" % worst)
    if golden_path:
        with open(golden_path, "w") as fh:
            json.dump(golden, fh)


if __name__ == "__main__":
    main()
