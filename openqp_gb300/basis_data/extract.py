"""Extract the basis sets used by the Fock-build workloads into JSON.

Reads the GAMESS-format basis files shipped with OpenQP (``basis_sets/*.basis``;
the data there come from the Basis Set Exchange) and writes one JSON file per
basis set with the shells of the elements the workloads use (H, C, N, O).

The JSON keeps the published exponents and contraction coefficients exactly as
printed; normalisation happens in ``openqp_gb300.basis`` (primitive
normalisation only, as OpenQP's Python front end feeds shells to
``map_shell2basis_set`` in ``source/basis_api.F90:220-317``).

``spherical`` records the AO convention the basis was published with: Pople
sets are Cartesian (6d), Dunning sets are spherical (5d), matching OpenQP's
``ispher=auto`` (``pyoqp/oqp/molecule/oqpdata.py:51-68``).

Usage: python extract.py <directory holding the *.basis files>
"""
import json
import os
import sys

ELEMENTS = {"HYDROGEN": 1, "CARBON": 6, "NITROGEN": 7, "OXYGEN": 8}
AM = {"S": 0, "P": 1, "D": 2, "F": 3}
SETS = {
    "sto-3g": ("sto-3g.basis", False),
    "6-31g": ("6-31g.basis", False),
    "6-31g(d)": ("6-31g(d).basis", False),
    "cc-pvdz": ("cc-pvdz.basis", True),
    "cc-pvtz": ("cc-pvtz.basis", True),
}


def parse_gamess(path):
    out = {}
    with open(path) as fh:
        lines = [ln.rstrip("\n") for ln in fh]
    i = 0
    cur = None
    while i < len(lines):
        tok = lines[i].split()
        if not tok or tok[0].startswith("!") or tok[0].startswith("$"):
            i += 1
            continue
        if len(tok) == 1 and tok[0].isalpha() and tok[0].upper() == tok[0] and tok[0] not in AM:
            cur = tok[0]
            out[cur] = []
            i += 1
            continue
        if cur is not None and tok[0] in AM and len(tok) == 2:
            n = int(tok[1])
            exps, coefs = [], []
            for k in range(n):
                row = lines[i + 1 + k].split()
                exps.append(float(row[1].replace("D", "E")))
                coefs.append(float(row[2].replace("D", "E")))
            out[cur].append({"l": AM[tok[0]], "exps": exps, "coefs": coefs})
            i += 1 + n
            continue
        i += 1
    return out


def main(src):
    here = os.path.dirname(os.path.abspath(__file__))
    for name, (fname, spherical) in SETS.items():
        data = parse_gamess(os.path.join(src, fname))
        js = {"name": name, "source": "OpenQP basis_sets/" + fname + " (Basis Set Exchange v0.8.13)",
              "spherical": spherical, "elements": {}}
        for el, z in ELEMENTS.items():
            if el in data:
                js["elements"][str(z)] = data[el]
        with open(os.path.join(here, name.replace("(", "_").replace(")", "") + ".json"), "w") as fh:
            json.dump(js, fh, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python extract.py <openqp checkout>/basis_sets")
    main(sys.argv[1])
