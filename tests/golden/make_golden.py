"""Extract OpenQP's own HF golden results into a small fixture.

Reads the example inputs/outputs that OpenQP's ``--validate_examples`` checks
(``examples/HF/*.json``, ``examples/NMR/*.json``, ``examples/TDHF/*.json``):
atoms, coordinates (Bohr, as stored in the JSON) and the reference total
energy (and gradient, and TDHF excitation energies, where present).  Run once where the OpenQP checkout exists; the fixture is committed.

Usage: python make_golden.py <openqp checkout> > hf_golden.json
"""
import json
import os
import sys

CASES = [
    ("examples/HF/H2O_RHF-HF_ENERGY.json", "6-31g*", "rhf", 1),
    ("examples/HF/H2O_UHF-HF_ENERGY.json", "6-31g*", "uhf", 3),
    ("examples/HF/H2O_ROHF-HF_ENERGY.json", "6-31g*", "rohf", 3),
    ("examples/HF/H2O_RHF-HF_GRADIENT.json", "6-31g*", "rhf", 1),
    ("examples/HF/H2O_UHF-HF_GRADIENT.json", "6-31g*", "uhf", 3),
    ("examples/HF/H2O_ROHF-HF_GRADIENT.json", "6-31g*", "rohf", 3),
    ("examples/NMR/H2O_RHF-NMR.json", "sto-3g", "rhf", 1),
    ("examples/NMR/CH3_UHF-GIAO-NMR.json", "sto-3g", "uhf", 2),
    ("examples/NMR/CH3_ROHF-GIAO-NMR.json", "sto-3g", "rohf", 2),
    ("examples/TDHF/H2O_TDHF_ENERGY.json", "6-31g*", "rhf", 1),
]


def main(root):
    out = []
    for rel, basis, kind, mult in CASES:
        with open(os.path.join(root, rel)) as fh:
            d = json.load(fh)
        case = {"source": rel, "basis": basis, "scf": kind, "multiplicity": mult, "atoms": d["atoms"],
                "coord_bohr": d["coord"], "energy": d["energy"]}
        if "grad" in d:
            case["grad"] = d["grad"]
        if d.get("td_energies") and any(d["td_energies"]):
            case["td_energies"] = d["td_energies"]
        out.append(case)
    json.dump({"cases": out}, sys.stdout, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_golden.py <openqp checkout> > hf_golden.json")
    main(sys.argv[1])
