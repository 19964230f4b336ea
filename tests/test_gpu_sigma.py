"""GPU parity of the MRSF sigma session (the reference's routec_sig seam)
against the oracle's restatement of the native sigma triple
(oracle/mrsf_sigma.py), and OpenQP's MRSF-TDHF golden excitation energies
through the session.

Tolerances: 1e-9 max-abs on sigma for unit-scale inputs (the 1e-10 Fock
parity gate carried through two orthonormal MO transforms); 1e-7 Eh on the
golden excitation energies (their Davidson converges them to ~1e-9).
"""
import json
import os

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("no CUDA device")
    from openqp_gb300 import build
    build.build()
    from openqp_gb300 import fock
    return fock


def _random_session_inputs(n, seed):
    rng = np.random.default_rng(seed)
    ca, _ = np.linalg.qr(rng.standard_normal((n, n)))
    cb, _ = np.linalg.qr(rng.standard_normal((n, n)))
    fa = rng.standard_normal((n, n))
    fb = rng.standard_normal((n, n))
    return ca, cb, 0.5 * (fa + fa.T), 0.5 * (fb + fb.T), rng


@pytest.mark.parametrize("kind", [1, 3])
def test_sigma_session_matches_oracle(gpu, oracle_lib, kind):
    """(H2O)4 / 6-31G(d), 21 alpha / 19 beta occupied, three trial vectors in
    one call, general orthonormal MO sets (alpha and beta different)."""
    from oracle import mrsf_sigma as ms
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(4, 6.0, seed=5, basis="6-31g(d)")
    n, na, nb = bas.nbf, 21, 19
    ca, cb, fa, fb, rng = _random_session_inputs(n, kind)
    bvec = rng.standard_normal((na * (n - nb), 3)) * 0.1
    o = oracle_lib.Oracle(bas)
    ref = ms.sigma(o.fock_mrsf, bvec, ca, cb, fa, fb, na, nb, kind, scale=0.5)
    assert gpu.routec_init(bas) == 0
    try:
        assert gpu.routec_sig_init(ca, cb, fa, fb, na, nb, kind) == 0
        gpu.routec_sig_set_scale(0.5)
        got, info = gpu.routec_sig_iter(bvec)
        assert info == 0
        assert np.abs(got - ref).max() < 1e-9 * max(1.0, np.abs(ref).max())
        # one vector at a time gives the same column up to the density
        # screening, which takes its bound over every vector of a call
        g1, info = gpu.routec_sig_iter(bvec[:, 1])
        assert info == 0 and np.abs(g1[:, 0] - got[:, 1]).max() < 1e-10 * max(1.0, np.abs(ref).max())
        gpu.routec_sig_free()
        _, info = gpu.routec_sig_iter(bvec)
        assert info == 1
    finally:
        gpu.routec_finalize()


@pytest.mark.parametrize("which", [0, 1], ids=["singlet", "triplet"])
def test_sigma_session_golden_mrsf(gpu, which):
    """OpenQP's h2o_rohf_mrsf-{s,t}_6-31g_hf through the GPU stack: ROHF by
    the GPU Fock build, then (A-B) over the whole active trial space from one
    routec_sig_iter call, diagonalised."""
    import mrsf
    from openqp_gb300.basis import build_basis
    case = json.load(open(os.path.join(ROOT, "tests", "golden", "mrsf_golden.json")))["cases"][which]
    bas = build_basis(case["atoms"], np.array(case["coord_bohr"]).reshape(-1, 3), case["basis"])
    fb_ = gpu.FockBuilder(bas)
    bas, r, C, fa, fbm, na, nb = mrsf.rohf_reference(case, lambda d: fb_.fock_jk(d))
    assert abs(r["energy"] - case["energy"]) < 1e-8
    mrst = case["mrsf_multiplicity"]
    assert gpu.routec_init(bas) == 0
    try:
        assert gpu.routec_sig_init(C, C, fa, fbm, na, nb, mrst) == 0

        def sigma(E):
            s, info = gpu.routec_sig_iter(E)
            assert info == 0
            return s

        w = mrsf.mrsf_energies(sigma, bas.nbf, na, nb, mrst, 6)
        assert np.abs(w - np.array(case["td_energies"])).max() < 1e-7
    finally:
        gpu.routec_finalize()


def test_sigma_session_declines(gpu):
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(1, workloads.cube_edge_like_c1(1), seed=0, basis="6-31g(d)")
    n = bas.nbf
    ca, cb, fa, fb, rng = _random_session_inputs(n, 0)
    gpu.routec_finalize()
    assert gpu.routec_sig_init(ca, cb, fa, fb, 6, 4, 1) == 1        # no seam context
    _, info = gpu.routec_sig_iter(np.zeros((6 * (n - 4), 1)))
    assert info == 1
    assert gpu.routec_init(bas) == 0
    try:
        assert gpu.routec_sig_init(ca, cb, fa, fb, 6, 5, 1) == 3    # not two open shells
        assert gpu.routec_sig_init(ca, cb, fa, fb, 6, 4, 2) == 3    # kind 1 or 3 only
        big = np.eye(n + 1)
        assert gpu.routec_sig_init(big, big, big, big, 6, 4, 1) == 1   # another basis
        assert gpu.routec_sig_init(ca, cb, fa, fb, 6, 4, 1) == 0
        b = rng.standard_normal((6 * (n - 4), 2))
        s1, info = gpu.routec_sig_iter(b)
        assert info == 0
        # the exchange scale enters linearly through the two-electron part
        gpu.routec_sig_set_scale(0.0)
        s0, _ = gpu.routec_sig_iter(b)
        gpu.routec_sig_set_scale(0.3)
        s3, _ = gpu.routec_sig_iter(b)
        assert np.abs(s3 - (s0 + 0.3 * (s1 - s0))).max() < 1e-11 * max(1.0, np.abs(s1).max())
        _, info = gpu.routec_sig_iter(np.zeros((6 * (n - 4), 0)))
        assert info == 0
    finally:
        gpu.routec_finalize()
    _, info = gpu.routec_sig_iter(b)
    assert info == 1        # routec_fock_finalize ended the session
