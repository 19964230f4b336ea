"""GPU: the two-electron gradient (derivative-ERI kernels) against the grd2
restatement in the oracle and against central finite differences, the
golden OpenQP gradients through our two-electron part, the routec_grad2 seam,
and the backward of the torch.autograd.Function.

Tolerances: 1e-9 against the oracle (the same screens; only summation order
differs), 2e-7 against the golden gradients (SCF convergence), and for central
differences with h = 1e-4 Bohr 1e-6 at the default cutoff / 1e-7 at 1e-14
(O(h^2) truncation plus the screens of the displaced builds).
"""
import numpy as np
import pytest

from conftest import h2o_basis

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


def _full(d, n):
    from openqp_gb300.basis import unpack
    return unpack(d, n)


@pytest.mark.parametrize("basis", ["6-31g*", "cc-pvdz", "sto-3g"])
def test_grad2_matches_oracle_h2o(gpu, oracle_lib, basis):
    from openqp_gb300 import workloads
    bas = h2o_basis(basis)
    n = bas.nbf
    o = oracle_lib.Oracle(bas)
    fb = gpu.FockBuilder(bas)
    d = workloads.density(bas, 5, 0)
    g = fb.grad2(d)
    ref = o.grad2e(_full(d, n))
    assert np.abs(g - ref).max() < 1e-9
    du = workloads.density_open(bas, 6, 4, 1)
    g = fb.grad2(du, hfscale=0.7, coulscale=1.1)
    Da, Db = _full(du[0], n), _full(du[1], n)
    ref = o.grad2e(Da + Db, Da - Db, coulscale=1.1, hfscale=0.7)
    assert np.abs(g - ref).max() < 1e-9


@pytest.mark.parametrize("nw,basis", [(3, "6-31g(d)"), (2, "cc-pvdz")])
def test_grad2_matches_oracle_clusters(gpu, oracle_lib, nw, basis):
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(nw, workloads.cube_edge_like_c1(nw), seed=4, basis=basis)
    d = workloads.density(bas, 5 * nw, 4)
    fb = gpu.FockBuilder(bas)
    g = fb.grad2(d)
    ref = oracle_lib.Oracle(bas).grad2e(_full(d, bas.nbf))
    assert np.abs(g - ref).max() < 1e-9
    assert np.abs(g.sum(axis=0)).max() < 1e-10
    st = fb.grad_stats()
    assert st["quartets"] > 0 and st["prim_quartets"] > 0


@pytest.mark.parametrize("cutoff,tol", [(1e-10, 1e-6), (1e-14, 1e-7)])
def test_grad2_finite_difference(gpu, cutoff, tol):
    """dE2/dR at fixed AO density, E2 = 1/2 Tr D G(D) from GPU Fock builds.
    At the default cutoff the screens of the displaced builds drop slightly
    different elements (noise ~1e-10 / 2h); at 1e-14 that noise is gone."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(3, workloads.cube_edge_like_c1(3), seed=8, basis="6-31g(d)")
    d = workloads.density(bas, 15, 8)
    n = bas.nbf
    D = _full(d, n)
    g = gpu.FockBuilder(bas, cutoff=cutoff).grad2(d)

    def e2(xyz):
        f = gpu.FockBuilder(bas.with_geometry(xyz), cutoff=cutoff).fock_jk(d)[0]
        return 0.5 * np.sum(D * _full(f, n))

    h = 1e-4
    rng = np.random.default_rng(1)
    for at in rng.choice(bas.natom, 4, replace=False):
        for x in range(3):
            xp = bas.xyz.copy(); xp[at, x] += h
            xm = bas.xyz.copy(); xm[at, x] -= h
            fd = (e2(xp) - e2(xm)) / (2 * h)
            assert abs(fd - g[at, x]) < tol, (at, x, fd, g[at, x])


@pytest.mark.parametrize("case_idx", [3, 4, 5])
def test_golden_gradient_with_gpu_two_electron_part(gpu, oracle_lib, case_idx):
    import json
    import os
    from conftest import ROOT
    from openqp_gb300 import onee, scf
    from openqp_gb300.basis import build_basis
    case = json.load(open(os.path.join(ROOT, "tests", "golden", "hf_golden.json")))["cases"][case_idx]
    assert "GRADIENT" in case["source"]
    bas = build_basis(case["atoms"], np.array(case["coord_bohr"]).reshape(-1, 3), case["basis"])
    fb = gpu.FockBuilder(bas)
    S, T, V = onee.one_electron(bas)
    nel = int(sum(case["atoms"]))
    nunp = case["multiplicity"] - 1
    na, nb = (nel + nunp) // 2, (nel - nunp) // 2
    kind = case["scf"]
    r = scf.run_scf(bas.nbf, S, T + V, onee.nuclear_repulsion(bas), na, nb, fb.fock_jk, kind=kind, conv=1e-11,
                    dconv=1e-9)
    assert r["converged"]
    n = bas.nbf
    Dm = [_full(x, n) for x in r["D"]]
    Dt = Dm[0] if kind == "rhf" else Dm[0] + Dm[1]
    W = scf.energy_weighted_density(r, na, nb, kind)
    g2 = fb.grad2(r["D"])
    g = oracle_lib.nuclear_repulsion_gradient(bas) + oracle_lib.Oracle(bas).grad1e(Dt, W) + g2
    assert np.abs(g - np.array(case["grad"]).reshape(-1, 3)).max() < 2e-7


def test_routec_grad2_seam(gpu):
    from openqp_gb300 import workloads
    bas = h2o_basis("6-31g*")
    d = workloads.density(bas, 5, 2)
    assert gpu.routec_init(bas, 1e-10) == 0
    de0 = np.ones((bas.natom, 3))
    de, info = gpu.routec_grad2(d, bas.xyz, bas.nbf, bas.natom, de=de0)
    assert info == 0
    ref = gpu.FockBuilder(bas).grad2(d)
    assert np.abs(de - (1.0 + ref)).max() < 1e-10     # accumulated into de
    moved = bas.xyz.copy()
    moved[0, 0] += 0.01
    _, info = gpu.routec_grad2(d, moved, bas.nbf, bas.natom)
    assert info == 1                                  # another geometry: declined
    gpu.routec_finalize()


def test_autograd_backward(gpu):
    import torch
    from openqp_gb300 import autograd, workloads
    bas = workloads.water_cluster_basis(2, workloads.cube_edge_like_c1(2), seed=6, basis="6-31g(d)")
    n = bas.nbf
    d = workloads.density(bas, 10, 6)
    fb = gpu.FockBuilder(bas)
    dt = torch.from_numpy(d).cuda().requires_grad_(True)
    xyz = torch.from_numpy(bas.xyz.copy()).requires_grad_(True)
    e2 = autograd.two_electron_energy(dt, fb, xyz)
    e2.backward()
    # dE2/dD: G(D) on the diagonal, 2 G(D) off it
    f = fb.fock_jk(d)[0]
    w = np.full(d.shape, 2.0)
    idx = np.arange(n)
    w[idx * (idx + 1) // 2 + idx] = 1.0
    assert np.abs(dt.grad.cpu().numpy() - w * f).max() < 1e-10
    # dE2/dR: OpenQP's grd2 two-electron gradient
    assert np.abs(xyz.grad.numpy() - fb.grad2(d)).max() < 1e-10
    # a general upstream matrix: directional finite difference in D (exact: linear)
    rng = np.random.default_rng(0)
    gf = torch.from_numpy(rng.standard_normal(d.shape)).cuda()
    dt.grad = None
    out = autograd.fock_jk(dt, fb)
    (out * gf).sum().backward()
    v = rng.standard_normal(d.shape)
    lin = float((gf.cpu() * (torch.from_numpy(fb.fock_jk(v)[0]))).sum())
    assert abs(float((dt.grad.cpu() * torch.from_numpy(v)).sum()) - lin) < 1e-8 * max(1.0, abs(lin))


def test_autograd_geometry_fd_uhf(gpu):
    """d/dR of a general linear functional of the UHF Fock pair, by central differences."""
    import torch
    from openqp_gb300 import autograd, workloads
    bas = h2o_basis("6-31g*")
    du = workloads.density_open(bas, 6, 4, 3)
    rng = np.random.default_rng(3)
    gf = rng.standard_normal(du.shape)
    fb = gpu.FockBuilder(bas)
    xyz = torch.from_numpy(bas.xyz.copy()).requires_grad_(True)
    f = autograd.fock_jk(torch.from_numpy(du).cuda(), fb, xyz, scale_exch=0.9, scale_coul=1.05)
    (f * torch.from_numpy(gf).cuda()).sum().backward()

    def L(x):
        return float(np.sum(gpu.FockBuilder(bas.with_geometry(x)).fock_jk(du, 0.9, 1.05) * gf))

    h = 1e-4
    for at, x in ((0, 2), (1, 0), (2, 1)):
        xp = bas.xyz.copy(); xp[at, x] += h
        xm = bas.xyz.copy(); xm[at, x] -= h
        fd = (L(xp) - L(xm)) / (2 * h)
        assert abs(fd - float(xyz.grad[at, x])) < 1e-6 * max(1.0, abs(fd)), (at, x, fd, float(xyz.grad[at, x]))


@pytest.mark.parametrize("mode", ["mixed", "mixed-fast"])
def test_grad2_precision_split(gpu, mode):
    """FP32 derivative quartets below the bound: max gradient error against the
    FP64 gradient well inside 1e-5 Eh/Bohr."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(6, workloads.cube_edge_like_c1(6), seed=12, basis="6-31g(d)")
    d = workloads.density(bas, 30, 12)
    fb = gpu.FockBuilder(bas)
    g64 = fb.grad2(d)
    fb.set_precision(mode, 1e-6)
    g32 = fb.grad2(d)
    st = fb.grad_stats()
    assert st["f32_quartets_listed"] > 0
    assert np.abs(g32 - g64).max() < 1e-7
    fb.set_precision(mode, 1e-3)
    assert np.abs(fb.grad2(d) - g64).max() < 1e-5


def _mrsf_inputs(bas, seed):
    from openqp_gb300 import workloads
    n = bas.nbf
    nel = workloads.nelectrons(bas)
    du = workloads.density_open(bas, nel // 2 + 1, nel // 2 - 1, seed)
    d = np.stack([_full(du[0], n), _full(du[1], n)])
    rng = np.random.default_rng(seed)
    p = rng.standard_normal((2, n, n)) * 0.05
    p = 0.5 * (p + p.transpose(0, 2, 1))
    spc = rng.standard_normal((7, n, n)) * 0.05
    return d, p, spc


@pytest.mark.parametrize("mrst", [1, 3])
@pytest.mark.parametrize("nw,basis", [(2, "6-31g(d)"), (2, "cc-pvdz")])
def test_grad2_mrsf_matches_oracle(gpu, oracle_lib, mrst, nw, basis):
    """grd2 with the MRSF two-particle density of grd2_mrsf_compute_data_t
    (non-symmetric response densities, spin-pair scales apart from HFscale)."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(nw, workloads.cube_edge_like_c1(nw), seed=6, basis=basis)
    d, p, spc = _mrsf_inputs(bas, mrst)
    fb = gpu.FockBuilder(bas)
    o = oracle_lib.Oracle(bas)
    args = (0.5, 0.45, 1.0, (0.4, 0.3, 0.2), mrst)
    g = fb.grad2_mrsf(d, p, spc, *args)
    ref = o.grad2e_mrsf(d, p, spc, *args)
    assert np.abs(g - ref).max() < 1e-9 * max(1.0, np.abs(ref).max())
    assert np.abs(g.sum(axis=0)).max() < 1e-9 * max(1.0, np.abs(ref).max())
    # Coulomb only (every exchange-type branch off)
    g0 = fb.grad2_mrsf(d, p, spc, 0.0, 0.0, 1.0, (0.0, 0.0, 0.0), mrst)
    r0 = o.grad2e_mrsf(d, p, spc, 0.0, 0.0, 1.0, (0.0, 0.0, 0.0), mrst)
    assert np.abs(g0 - r0).max() < 1e-9 * max(1.0, np.abs(r0).max())


def test_grad2_mrsf_seam_and_precision(gpu):
    """routec_grad2_mrsf with the Fortran buffers of tdhf_mrsf_gradient (de
    accumulated, another geometry declined); the MRSF form stays FP64 when the
    context runs the precision split."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(2, workloads.cube_edge_like_c1(2), seed=1, basis="6-31g(d)")
    n = bas.nbf
    d, p, spc = _mrsf_inputs(bas, 5)
    fb = gpu.FockBuilder(bas)
    ref = fb.grad2_mrsf(d, p, spc, 0.5, 0.5, 1.0, (0.5, 0.5, 0.5), 1)
    fb.set_precision("mixed", 1e-6)
    assert np.abs(fb.grad2_mrsf(d, p, spc, 0.5, 0.5, 1.0, (0.5, 0.5, 0.5), 1) - ref).max() < 1e-12
    fd = np.ascontiguousarray(d.transpose(0, 2, 1))          # Fortran (nbf, nbf, 2)
    fp = np.ascontiguousarray(p.transpose(0, 2, 1))
    fs = np.ascontiguousarray(spc.transpose(2, 1, 0))        # Fortran (7, nbf, nbf)
    assert gpu.routec_init(bas, 1e-10) == 0
    try:
        de0 = np.ones((bas.natom, 3))
        de, info = gpu.routec_grad2_mrsf(fd, fp, fs, bas.xyz, n, bas.natom, 0.5, 0.5, 1.0, (0.5, 0.5, 0.5), 1,
                                         de=de0)
        assert info == 0
        assert np.abs(de - (1.0 + ref)).max() < 1e-10 * max(1.0, np.abs(ref).max())
        moved = bas.xyz.copy()
        moved[1, 2] += 0.01
        _, info = gpu.routec_grad2_mrsf(fd, fp, fs, moved, n, bas.natom, 0.5, 0.5, 1.0, (0.5, 0.5, 0.5), 1)
        assert info == 1
    finally:
        gpu.routec_finalize()


def test_grad2_sf_matches_oracle(gpu, oracle_lib):
    """grd2_sf_compute_data_t: the MRSF density with ball = v and no spin-pair
    coupling terms (the oracle's literal MRSF restatement with those inputs is
    the SF get_density term for term)."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(2, workloads.cube_edge_like_c1(2), seed=9, basis="cc-pvdz")
    d, p, spc = _mrsf_inputs(bas, 7)
    v = spc[0]
    g = gpu.FockBuilder(bas).grad2_sf(d, p, v, 0.5, 0.45)
    sp = np.zeros_like(spc)
    sp[6] = v
    ref = oracle_lib.Oracle(bas).grad2e_mrsf(d, p, sp, 0.5, 0.45, 1.0, (0.0, 0.0, 0.0), 1)
    assert np.abs(g - ref).max() < 1e-9 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("nw,basis", [(2, "6-31g(d)"), (2, "cc-pvdz")])
def test_grad2_cam_matches_oracle(gpu, oracle_lib, nw, basis):
    """grd2_driver's CAM branch: 1/r pass (alpha) + erf(mu r)/r pass (beta, no
    Coulomb) with its own Schwarz bounds, RHF and UHF; then the MRSF CAM form;
    a plain gradient on the same context afterwards is unaffected."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(nw, workloads.cube_edge_like_c1(nw), seed=11, basis=basis)
    n = bas.nbf
    fb = gpu.FockBuilder(bas)
    o = oracle_lib.Oracle(bas)
    cam = (0.19, 0.46, 0.33)
    d = workloads.density(bas, 5 * nw, 1)
    g = fb.grad2_cam(d, *cam)
    ref = o.grad2e_cam(_full(d, n), None, *cam)
    assert np.abs(g - ref).max() < 1e-9 * max(1.0, np.abs(ref).max())
    du = workloads.density_open(bas, 5 * nw + 1, 5 * nw - 1, 2)
    Da, Db = _full(du[0], n), _full(du[1], n)
    g = fb.grad2_cam(du, *cam)
    ref = o.grad2e_cam(Da + Db, Da - Db, *cam)
    assert np.abs(g - ref).max() < 1e-9 * max(1.0, np.abs(ref).max())
    dm, p, spc = _mrsf_inputs(bas, 3)
    c5 = (0.19, 0.46, 0.25, 0.5, 0.33)
    g = fb.grad2_mrsf(dm, p, spc, 0.0, 0.0, spcscale=(0.4, 0.3, 0.2), mrst=1, cam=c5)
    ref = o.grad2e_mrsf(dm, p, spc, 0.0, 0.0, 1.0, (0.4, 0.3, 0.2), 1, cam=c5)
    assert np.abs(g - ref).max() < 1e-9 * max(1.0, np.abs(ref).max())
    assert np.abs(fb.grad2(d) - o.grad2e(_full(d, n))).max() < 1e-9
