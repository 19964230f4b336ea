"""Generate the finer, lower-degree Rys tables of the one- and two-root rules
(``rys_tables_fine.inc``), used by the FP64 thread-per-quartet kernels.

Same method and exact values as ``gen_rys_tables.py`` (60-digit Boys moments,
Golub-Welsch, Chebyshev interpolation at the Chebyshev nodes, monomial
coefficients in s in [-1, 1]); only the grid differs: width 1/8 below X = 32
and 1/2 from 32 to the large-X limit 32 + 8n, with degree-6 interpolants.
That keeps the relative error near 1e-15 (degree 7 on width 1/4 before) and
saves one FMA of each node and weight chain, for the classes that dominate an
s/p-rich build: (ss|ss), (ss|sp), (sp|sp), (ss|pp), (ss|sd).

Usage: python gen_rys_fine.py   (needs mpmath; writes next to itself)
"""
import multiprocessing as mpr
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import gen_rys_tables as g  # noqa: E402

NMAX_FINE = 2
NCOEF = 7            # degree-6 interpolants
H_LO = 0.125         # below X_SPLIT
H_HI = 0.5           # from X_SPLIT to XMAX(n)


def intervals(n):
    iv = [(k * H_LO, H_LO) for k in range(int(g.X_SPLIT / H_LO))]
    a = float(g.X_SPLIT)
    while a < g.XMAX[n]:
        iv.append((a, H_HI))
        a += H_HI
    return iv


def interval_of(X):
    if X < g.X_SPLIT:
        k = int(X / H_LO)
        return k, k * H_LO, H_LO
    k0 = int(g.X_SPLIT / H_LO)
    k = k0 + int((X - g.X_SPLIT) / H_HI)
    return k, g.X_SPLIT + (k - k0) * H_HI, H_HI


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    jobs = [(n, a, h, NCOEF) for n in range(1, NMAX_FINE + 1) for (a, h) in intervals(n)]
    with mpr.get_context("spawn").Pool() as pool:
        fits = pool.map(g.fit_interval, jobs)
    tables = {n: [] for n in range(1, NMAX_FINE + 1)}
    for (n, a, h, _), rows in zip(jobs, fits):
        tables[n].append(rows)
    vals = []
    for n in range(1, NMAX_FINE + 1):
        for rows in tables[n]:
            for c in rows:
                vals.extend(repr(float(v)) for v in c)
    lines = [
        "// Generated by gen_rys_fine.py -- do not edit.",
        "// Rys nodes x_i and weights w_i of the n = 1, 2 root rules on a finer grid:",
        "// width %g below %d, width %g from %d to 32 + 8n; per interval and root: %d"
        % (H_LO, g.X_SPLIT, H_HI, g.X_SPLIT, NCOEF),
        "// monomial coefficients of x_i, then of w_i, in s = 2 (X - a_k) / h_k - 1.",
        "#ifndef RYS_STORAGE",
        "#define RYS_STORAGE static const",
        "#endif",
        "#define RYS_FINE_NMAX %d" % NMAX_FINE,
        "#define RYS_FINE_NCOEF %d" % NCOEF,
        "#define RYS_FINE_LO_PER_UNIT %d" % int(round(1 / H_LO)),
        "#define RYS_FINE_HI_PER_UNIT %d" % int(round(1 / H_HI)),
        "#define RYS_TABLE_FINE_SIZE %d" % len(vals),
        "RYS_STORAGE double RYS_TABLE_FINE[RYS_TABLE_FINE_SIZE] = {",
    ]
    for i in range(0, len(vals), 4):
        lines.append("  " + ", ".join(vals[i:i + 4]) + ",")
    lines.append("};")
    with open(os.path.join(here, "rys_tables_fine.inc"), "w") as fh:
        fh.write("\n".join(lines) + "\n")
    # self-check against exact values
    rng = np.random.default_rng(11)
    worst = 0.0
    for n in range(1, NMAX_FINE + 1):
        for X in list(rng.uniform(0, 1, 40)) + list(rng.uniform(0, g.XMAX[n], 200)):
            ex = g.rys_exact(X, n)
            k, a, h = interval_of(X)
            s = 2 * (X - a) / h - 1
            rows = tables[n][k]
            for r in range(n):
                for which in (0, 1):
                    v = g.horner(list(rows[2 * r + which]), s)
                    e = float(ex[which][r])
                    worst = max(worst, abs(v - e) / abs(e))
    print("worst relative error of the fine tables: %.2e" % worst)


if __name__ == "__main__":
    main()
