"""GPU parity of the response-type builds (general square densities) against
the oracle's restatement of OpenQP's int2_td_data_t / int2_tdgrd_data_t /
int2_rpagrd_data_t / int2_mrsf_data_t / int2_umrsf_data_t digestions.

Tolerance: 1e-10 max-abs (the plain-FP64 gate) on every output matrix;
the double-float mode is held to 1e-9.
"""
import json
import os

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.fixture(scope="module")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("no CUDA device")
    from openqp_gb300 import build
    build.build()
    from openqp_gb300 import fock
    return fock


def _flags(fl):
    return dict(apb=bool(fl & 1), amb=bool(fl & 2), tda=bool(fl & 4), tda_coulomb=bool(fl & 8))


@pytest.mark.parametrize("flags", [1, 2, 3, 4, 12])
@pytest.mark.parametrize("basis", ["6-31g(d)", "cc-pvdz"])
def test_td_water4(gpu, oracle_lib, flags, basis):
    """(H2O)4, 3 general densities, every combination of the TD flags."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(4, 6.0, seed=1, basis=basis)
    x = np.random.default_rng(flags).standard_normal((3, bas.nbf, bas.nbf)) * 0.2
    fb = gpu.FockBuilder(bas)
    pa, ma = fb.fock_td(x, scale_exch=0.8, scale_coul=1.1, **_flags(flags))
    rp, rm = oracle_lib.Oracle(bas).fock_td(x, flags, se=0.8, sc=1.1)
    assert np.abs(pa - rp).max() < TOL
    assert np.abs(ma - rm).max() < TOL
    if flags & 1:
        assert np.abs(pa - pa.transpose(0, 2, 1)).max() < 1e-12
    if flags == 2:
        assert np.abs(ma + ma.transpose(0, 2, 1)).max() < 1e-12


@pytest.mark.parametrize("nmat", [7, 11])
def test_mrsf_water2(gpu, oracle_lib, nmat):
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(2, workloads.cube_edge_like_c1(2), seed=4, basis="6-31g(d)")
    x = np.random.default_rng(nmat).standard_normal((2, nmat, bas.nbf, bas.nbf)) * 0.2
    f = gpu.FockBuilder(bas).fock_mrsf(x, scale_exch=0.5, scale_coul=1.0)
    ref = oracle_lib.Oracle(bas).fock_mrsf(x, se=0.5, sc=1.0)
    assert np.abs(f - ref).max() < TOL


def test_td_and_scf_builds_share_a_context(gpu, oracle_lib):
    """Response and SCF builds alternate on one context (shared list buffers)."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(4, 6.0, seed=2, basis="6-31g(d)")
    fb = gpu.FockBuilder(bas)
    o = oracle_lib.Oracle(bas)
    d = workloads.density(bas, 20, 2)
    x = np.random.default_rng(9).standard_normal((5, bas.nbf, bas.nbf))
    for _ in range(2):
        assert np.abs(fb.fock_jk(d) - o.fock_jk(d)).max() < TOL
        pa, ma = fb.fock_td(x, apb=True, amb=True)
        rp, rm = o.fock_td(x, 3)
        assert np.abs(pa - rp).max() < TOL and np.abs(ma - rm).max() < TOL


def test_td_device_and_routec(gpu, oracle_lib):
    """The torch-tensor entry point and the Fortran-style seam give the host result."""
    import torch
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(2, workloads.cube_edge_like_c1(2), seed=6, basis="6-31g(d)")
    n = bas.nbf
    x = np.random.default_rng(3).standard_normal((2, n, n))
    fb = gpu.FockBuilder(bas)
    pa, ma = fb.fock_td(x, apb=True, amb=True)
    tp, tm = fb.fock_td_device(torch.from_numpy(x).cuda(), apb=True, amb=True)
    assert np.abs(tp.cpu().numpy() - pa).max() < 1e-13 and np.abs(tm.cpu().numpy() - ma).max() < 1e-13
    assert gpu.routec_init(bas) == 0
    try:
        fx = np.ascontiguousarray(x.transpose(0, 2, 1))   # Fortran d2(nbf, nbf, nvec)
        ap, am, info = gpu.routec_fock_td(fx, n, 2, gpu.td_flags(True, True))
        assert info == 0
        assert np.abs(ap.reshape(2, n, n).transpose(0, 2, 1) - pa).max() < 1e-13
        assert np.abs(am.reshape(2, n, n).transpose(0, 2, 1) - ma).max() < 1e-13
        x3 = np.random.default_rng(4).standard_normal((1, 7, n, n))
        f3, info = gpu.routec_fock_mrsf(np.ascontiguousarray(x3.transpose(3, 2, 1, 0)), n, 1, 7)
        assert info == 0
        ref = oracle_lib.Oracle(bas).fock_mrsf(x3)
        assert np.abs(f3.reshape(n, n, 7, 1).transpose(3, 2, 1, 0) - ref).max() < TOL
        _, _, info = gpu.routec_fock_td(fx, n + 1, 2, 3)
        assert info == 1   # another basis: declined
    finally:
        gpu.routec_finalize()


def test_td_rejects_bad_input(gpu):
    from openqp_gb300 import workloads
    from openqp_gb300._lib import lib, ptr
    bas = workloads.water_cluster_basis(1, workloads.cube_edge_like_c1(1), seed=0, basis="6-31g(d)")
    fb = gpu.FockBuilder(bas)
    x = np.zeros((1, bas.nbf, bas.nbf))
    out1, out2 = np.zeros_like(x), np.zeros_like(x)
    assert lib().oqpg_fock_td(fb.h, ptr(x), ptr(out1), ptr(out2), 1, 16, 1.0, 1.0) == 3   # unknown flag
    assert lib().oqpg_fock_td(fb.h, ptr(x), ptr(out1), ptr(out2), 0, 1, 1.0, 1.0) == 3    # no vectors
    assert lib().oqpg_fock_mrsf(fb.h, ptr(x), ptr(out1), 1, 5, 1.0, 1.0) == 3            # nmat not 7 / 11
    pa, ma = fb.fock_td(x, apb=False, amb=False)
    assert not pa.any() and not ma.any()


def test_tdhf_golden_excitation_energies(gpu):
    """OpenQP's examples/TDHF/H2O_TDHF_ENERGY through the GPU TD build: full
    A+B / A-B over all 70 occupied-virtual unit vectors in one call."""
    import rpa
    from openqp_gb300 import onee, scf
    from openqp_gb300.basis import build_basis
    gold = json.load(open(os.path.join(ROOT, "tests", "golden", "hf_golden.json")))["cases"]
    case = [c for c in gold if "TDHF" in c["source"]][0]
    bas = build_basis(case["atoms"], np.array(case["coord_bohr"]).reshape(-1, 3), case["basis"])
    fb = gpu.FockBuilder(bas)
    S, T = onee.overlap_kinetic(bas)
    H = T + onee.nuclear(bas)
    r = scf.run_scf(bas.nbf, S, H, onee.nuclear_repulsion(bas), 5, 5, lambda d: fb.fock_jk(d), conv=1e-12,
                    dconv=1e-10)
    assert abs(r["energy"] - case["energy"]) < 1e-7
    e, C = rpa.canonical_orbitals(S, r["Fock"][0])

    def td(x, fl):
        return fb.fock_td(x, **_flags(fl))

    w, _, _ = rpa.rpa_energies(td, C, e, 5)
    assert np.abs(w[:3] - np.array(case["td_energies"])).max() < 5e-7


def test_td_double_float_mode(gpu, oracle_lib):
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(4, 6.0, seed=3, basis="cc-pvdz")
    x = np.random.default_rng(2).standard_normal((2, bas.nbf, bas.nbf)) * 0.2
    fb = gpu.FockBuilder(bas)
    fb.set_precision("df")
    pa, ma = fb.fock_td(x, apb=True, amb=True)
    rp, rm = oracle_lib.Oracle(bas).fock_td(x, 3)
    assert np.abs(pa - rp).max() < 1e-9 and np.abs(ma - rm).max() < 1e-9


def test_td_water16_properties(gpu):
    """(H2O)16 / 6-31G(d), 12 densities: linearity in the density (a sum of two
    builds equals the build of the sum) and the A+B / A-B symmetries."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(16, workloads.cube_edge_like_c1(16), seed=0, basis="6-31g(d)")
    n = bas.nbf
    rng = np.random.default_rng(0)
    x = rng.standard_normal((4, n, n)) * 0.05
    y = rng.standard_normal((4, n, n)) * 0.05
    fb = gpu.FockBuilder(bas)
    both = fb.fock_td(np.concatenate([x, y, x + y]), apb=True, amb=True)
    for m in both:
        assert np.abs(m[:4] + m[4:8] - m[8:]).max() < 1e-8 * max(1.0, np.abs(m).max())
    assert np.abs(both[0] - both[0].transpose(0, 2, 1)).max() < 1e-12
    assert np.abs(both[1] + both[1].transpose(0, 2, 1)).max() < 1e-12


@pytest.mark.parametrize("flags", [1, 2, 3])
def test_tdgrd_water4(gpu, oracle_lib, flags):
    """int2_tdgrd_data_t: two spin densities, (H2O)4 / cc-pVDZ; host form,
    device form and the Fortran-style seam."""
    import torch
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(4, 6.0, seed=7, basis="cc-pvdz")
    n = bas.nbf
    x = np.random.default_rng(20 + flags).standard_normal((2, n, n)) * 0.2
    fb = gpu.FockBuilder(bas)
    pa, ma = fb.fock_tdgrd(x, apb=bool(flags & 1), amb=bool(flags & 2), scale_exch=0.8, scale_coul=1.1)
    rp, rm = oracle_lib.Oracle(bas).fock_tdgrd(x, flags, se=0.8, sc=1.1)
    assert np.abs(pa - rp).max() < TOL and np.abs(ma - rm).max() < TOL
    assert not ma[1].any()
    from openqp_gb300._lib import lib
    fx = torch.from_numpy(np.ascontiguousarray(x.transpose(0, 2, 1))).cuda()
    tp, tm = torch.empty_like(fx), torch.empty_like(fx)
    rc = lib().oqpg_fock_tdgrd_device(fb.h, fx.data_ptr(), tp.data_ptr(), tm.data_ptr(), flags, 0.8, 1.1, None,
                                      torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    assert np.abs(tp.cpu().numpy().transpose(0, 2, 1) - pa).max() < 1e-13
    assert np.abs(tm.cpu().numpy().transpose(0, 2, 1) - ma).max() < 1e-13
    assert gpu.routec_init(bas) == 0
    try:
        ap, am, info = gpu.routec_fock_tdgrd(np.ascontiguousarray(x.transpose(0, 2, 1)), n, flags, 0.8, 1.1)
        assert info == 0
        assert np.abs(ap.reshape(2, n, n).transpose(0, 2, 1) - pa).max() < 1e-13
        assert np.abs(am.reshape(2, n, n).transpose(0, 2, 1) - ma).max() < 1e-13
    finally:
        gpu.routec_finalize()


@pytest.mark.parametrize("nspin", [1, 2])
def test_rpagrd_water4(gpu, oracle_lib, nspin):
    """int2_rpagrd_data_t: H+[X+Y], H+[T], H-[X-Y] with symmetric H+
    operands (as every reference caller passes) and a general X-Y; the
    xpy2-style layout (an extra operand slot read only by the screening)."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(4, 6.0, seed=8, basis="6-31g(d)")
    n = bas.nbf
    rng = np.random.default_rng(nspin)
    sym = lambda a: 0.5 * (a + a.swapaxes(-1, -2))
    xpy = sym(rng.standard_normal((2, nspin + 1, n, n)) * 0.2)
    t = sym(rng.standard_normal((1, nspin, n, n)) * 0.2)
    xmy = rng.standard_normal((2, nspin, n, n)) * 0.2
    fb = gpu.FockBuilder(bas)
    o = oracle_lib.Oracle(bas)
    got = fb.fock_rpagrd(xpy, xmy, t, nspin, scale_exch=0.6, scale_coul=1.2)
    ref = o.fock_rpagrd(xpy, xmy, t, nspin, se=0.6, sc=1.2)
    for g, r in zip(got, ref):
        assert np.abs(g - r).max() < TOL
    # the tdhf_z_vector.F90:341 call: t only
    _, ht, _ = fb.fock_rpagrd(t=t, nspin=nspin)
    assert np.abs(ht - o.fock_rpagrd(None, None, t, nspin)[1]).max() < TOL
    # X-Y alone is not screened in (init_screen): zero, as the reference
    _, _, hm = fb.fock_rpagrd(xmy=xmy, nspin=nspin)
    assert not hm.any()


def test_gradient_side_builds_reject_bad_input(gpu):
    from openqp_gb300 import workloads
    from openqp_gb300._lib import lib, ptr
    bas = workloads.water_cluster_basis(1, workloads.cube_edge_like_c1(1), seed=0, basis="6-31g(d)")
    fb = gpu.FockBuilder(bas)
    x = np.zeros((2, bas.nbf, bas.nbf))
    o1, o2 = np.zeros_like(x), np.zeros_like(x)
    assert lib().oqpg_fock_tdgrd(fb.h, ptr(x), ptr(o1), ptr(o2), 4, 1.0, 1.0, None) == 3   # TDA not defined
    v = x.ctypes.data
    assert lib().oqpg_fock_rpagrd(fb.h, v, 1, 1, None, 1, 0, None, 1, 0, 3, v, None, None, 1.0, 1.0, None) == 3
    assert lib().oqpg_fock_rpagrd(fb.h, v, 1, 1, None, 1, 0, None, 1, 0, 2, v, None, None, 1.0, 1.0, None) == 3
    assert lib().oqpg_fock_rpagrd(fb.h, None, 1, 1, None, 1, 0, None, 1, 0, 1, v, None, None, 1.0, 1.0, None) == 3
