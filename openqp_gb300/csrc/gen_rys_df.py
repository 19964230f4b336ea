"""Emit rys_tables_df.inc: the FP64 Rys tables of rys_tables.inc split into
pairs of FP32 numbers (hi = round(v), lo = round(v - hi)), for the
double-float ("df") precision mode.  Reads the committed rys_tables.inc, so
it needs no arbitrary-precision arithmetic.

Usage: python gen_rys_df.py
"""
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_array(text, name):
    m = re.search(r"RYS_STORAGE double %s\[[A-Z_0-9]+\] = \{(.*?)\};" % name, text, re.S)
    if m is None:
        raise RuntimeError("array %s not found" % name)
    return [float(v) for v in m.group(1).replace("\n", " ").split(",") if v.strip()]


def split(vals):
    out = []
    for v in vals:
        hi = np.float32(v)
        lo = np.float32(v - float(hi))
        out.append((float(hi), float(lo)))
    return out


def emit(lines, name, pairs):
    lines.append("#define %s_SIZE %d" % (name, len(pairs)))
    lines.append("RYS_STORAGE float2 %s[%s_SIZE] = {" % (name, name))
    for i in range(0, len(pairs), 4):
        lines.append("  " + ", ".join("{%r, %r}" % (h, l) for h, l in pairs[i:i + 4]) + ",")
    lines.append("};")


def main():
    text = open(os.path.join(HERE, "rys_tables.inc")).read()
    lines = ["// Generated by gen_rys_df.py from rys_tables.inc: each FP64 coefficient as",
             "// an unevaluated FP32 pair hi + lo (the double-float precision mode).",
             "#ifndef RYS_STORAGE",
             "#define RYS_STORAGE static const",
             "#endif"]
    emit(lines, "RYS_TABLE_DF", split(read_array(text, "RYS_TABLE")))
    emit(lines, "RYS_HERM_R2_DF", split(read_array(text, "RYS_HERM_R2")))
    emit(lines, "RYS_HERM_W_DF", split(read_array(text, "RYS_HERM_W")))
    with open(os.path.join(HERE, "rys_tables_df.inc"), "w") as fh:
        fh.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
