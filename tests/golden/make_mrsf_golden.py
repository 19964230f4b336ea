"""Extract OpenQP's MRSF-TDHF golden results into a small fixture.

Reads the example outputs ``examples/other/h2o_rohf_mrsf-{s,t}_6-31g_hf.json``
(ROHF triplet reference, MRSF singlet / triplet response, pure HF):
atoms, coordinates (Bohr, as stored), the ROHF total energy and the MRSF
excitation energies (Hartree, relative to the ROHF reference).  Run once
where the OpenQP checkout exists; the fixture is committed.

Usage: python make_mrsf_golden.py <openqp checkout> > mrsf_golden.json
"""
import json
import os
import sys

CASES = [
    ("examples/other/h2o_rohf_mrsf-s_6-31g_hf.json", "6-31g", 1),
    ("examples/other/h2o_rohf_mrsf-t_6-31g_hf.json", "6-31g", 3),
]


def main(root):
    out = []
    for rel, basis, mult in CASES:
        with open(os.path.join(root, rel)) as fh:
            d = json.load(fh)
        out.append({"source": rel, "basis": basis, "scf": "rohf", "multiplicity": 3, "mrsf_multiplicity": mult,
                    "atoms": d["atoms"], "coord_bohr": d["coord"], "energy": d["energy"],
                    "td_energies": d["td_energies"]})
    json.dump({"cases": out}, sys.stdout, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_mrsf_golden.py <openqp checkout> > mrsf_golden.json")
    main(sys.argv[1])
