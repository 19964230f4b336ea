import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    oracle.build()
    return oracle


def h2o_basis(basis="6-31g*", spherical=None):
    import json
    import numpy as np
    from openqp_gb300.basis import build_basis
    g = json.load(open(os.path.join(ROOT, "tests", "golden", "hf_golden.json")))
    c = g["cases"][0]
    return build_basis(c["atoms"], np.array(c["coord_bohr"]).reshape(-1, 3), basis, spherical=spherical)
