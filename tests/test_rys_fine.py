"""The finer one- and two-root Rys tables of the FP64 kernels
(openqp_gb300/csrc/rys_tables_fine.inc: degree 6, width 1/8 below X = 32 and
1/2 from 32 up to 32 + 8n) against the 60-digit nodes and weights of
tests/golden/rys_exact.json, with the interval and Chebyshev-variable
arithmetic of the device's rys_interval<3, 1>.  The large-X form above the
table is the same as for the standard tables and is pinned by the oracle's
table test."""
import json
import os
import re

import numpy as np

from conftest import ROOT

INC = os.path.join(ROOT, "openqp_gb300", "csrc", "rys_tables_fine.inc")


def _load():
    txt = open(INC).read()
    defs = {k: int(v) for k, v in re.findall(r"#define (RYS_\w+) (\d+)", txt)}
    body = txt[txt.index("{") + 1:txt.rindex("}")]
    vals = np.array([float(v) for v in body.replace("\n", " ").split(",") if v.strip()])
    assert vals.size == defs["RYS_TABLE_FINE_SIZE"]
    return defs, vals


def _eval(defs, vals, n, X):
    lo, hi, nc = defs["RYS_FINE_LO_PER_UNIT"], defs["RYS_FINE_HI_PER_UNIT"], defs["RYS_FINE_NCOEF"]
    split = 32
    nint = [0] + [split * lo + 8 * m * hi for m in (1, 2)]
    off = 0 if n == 1 else nint[1] * 2 * nc
    if X < split:
        f = int(np.floor(X * lo))
        k, s = f, 2 * lo * X - (2 * f + 1)
    else:
        f = int(np.floor(X * hi))
        k, s = split * lo + (f - split * hi), 2 * hi * X - (2 * f + 1)
    out = []
    for r in range(n):
        c = vals[off + (k * 2 * n + 2 * r) * nc:][:2 * nc]
        out.append((np.polynomial.polynomial.polyval(s, c[:nc]), np.polynomial.polynomial.polyval(s, c[nc:])))
    return out


def test_fine_tables_match_exact_values():
    defs, vals = _load()
    assert defs["RYS_FINE_NMAX"] == 2 and defs["RYS_FINE_NCOEF"] == 7
    g = json.load(open(os.path.join(ROOT, "tests", "golden", "rys_exact.json")))
    worst, count = 0.0, 0
    for c in g["cases"]:
        n, X = c["n"], c["X"]
        if n > 2 or X >= 32 + 8 * n:
            continue
        for r, (x, w) in enumerate(_eval(defs, vals, n, X)):
            worst = max(worst, abs(x - c["x"][r]) / abs(c["x"][r]), abs(w - c["w"][r]) / abs(c["w"][r]))
        count += 1
    assert count >= 40
    # degree 6 on the halved intervals: as accurate as the degree-7 standard tables
    assert worst < 1e-14


def test_fine_tables_continuous_across_intervals():
    """Neighbouring interpolants agree at their shared end points (s = +1 of
    interval k and s = -1 of interval k+1), including across X = 32."""
    defs, vals = _load()
    worst = 0.0
    for n in (1, 2):
        for X in list(np.arange(1, 256) / 8.0) + list(32 + np.arange(1, 16 * n) / 2.0):
            below = _eval(defs, vals, n, np.nextafter(X, 0))
            above = _eval(defs, vals, n, X)
            for (xb, wb), (xa, wa) in zip(below, above):
                worst = max(worst, abs(xb - xa) / abs(xa), abs(wb - wa) / abs(wa))
    assert worst < 1e-14
