"""CPU tests that pin the oracle (the CPU restatement of OpenQP's Fock build)
before it is trusted as the checker of the GPU path.

Pins, in order of strength:
  * OpenQP's own golden HF energies (examples/HF, examples/NMR) reproduced by
    an SCF whose two-electron part is the oracle's fock_jk restatement;
  * J/K semantics of the restated storeints + digestion + scaling against a
    dense ERI contraction;
  * Rys ERIs against an independent McMurchie-Davidson code;
  * the Rys tables against 60-digit values;
  * the response digestions (int2_td_data_t, int2_mrsf_data_t,
    int2_umrsf_data_t) against dense J/K contractions of general matrices,
    and OpenQP's golden TDHF excitation energies (examples/TDHF) from full
    A+B / A-B matrices built with the restated int2_td_data_t;
  * the erf-attenuated integrals of the CAM pass (Rys with p + q -> p + q +
    pq/mu^2) against McMurchie-Davidson with the attenuated Hermite exponent,
    and the two-pass CAM builds against dense contractions.
"""
import json
import os

import numpy as np
import pytest

from conftest import ROOT, h2o_basis

GOLD = json.load(open(os.path.join(ROOT, "tests", "golden", "hf_golden.json")))["cases"]


def test_rys_tables_match_exact_values(oracle_lib):
    g = json.load(open(os.path.join(ROOT, "tests", "golden", "rys_exact.json")))
    worst = {}
    for c in g["cases"]:
        x, w = oracle_lib.rys(c["n"], c["X"])
        e = max(np.max(np.abs(x - c["x"]) / np.abs(c["x"])), np.max(np.abs(w - c["w"]) / np.abs(c["w"])))
        worst[c["n"]] = max(worst.get(c["n"], 0.0), e)
    assert sorted(worst) == list(range(1, 8))
    # degree-7 fits: ~5e-15 up to six roots; seven roots reach 1.8e-14 on the unit interval at X = 32
    assert all(worst[n] < 1e-14 for n in range(1, 7)) and worst[7] < 2.5e-14


@pytest.mark.parametrize("basis", ["6-31g*", "cc-pvdz"])
def test_rys_matches_mcmurchie_davidson(oracle_lib, basis):
    bas = h2o_basis(basis)
    o = oracle_lib.Oracle(bas)
    ns = len(bas.am)
    worst = 0.0
    rng = np.random.default_rng(3)
    for _ in range(250):
        i, j, k, l = (int(v) for v in rng.integers(0, ns, 4))
        worst = max(worst, np.abs(o.eri_quartet(i, j, k, l) - o.md_quartet(i, j, k, l)).max())
    assert worst < 1e-12


@pytest.mark.parametrize("basis", ["6-31g*", "cc-pvdz"])
def test_fock_jk_matches_dense_contraction(oracle_lib, basis):
    from openqp_gb300 import workloads
    from openqp_gb300.basis import unpack
    bas = h2o_basis(basis)
    o = oracle_lib.Oracle(bas, cutoff=1e-12)
    n = o.nbf
    eri = o.eri_dense()
    D = workloads.density(bas, 5, 0)
    Df = unpack(D, n)
    J = np.einsum("ijkl,kl->ij", eri, Df)
    K = np.einsum("ikjl,kl->ij", eri, Df)
    F = o.fock_jk(D)
    assert np.abs(unpack(F[0], n) - (J - 0.5 * K)).max() < 1e-11
    Dab = workloads.density_open(bas, 5, 4, 1)
    Da, Db = unpack(Dab[0], n), unpack(Dab[1], n)
    Jt = np.einsum("ijkl,kl->ij", eri, Da + Db)
    F2 = o.fock_jk(Dab, se=0.7, sc=0.9)
    assert np.abs(unpack(F2[0], n) - (0.9 * Jt - 0.7 * np.einsum("ikjl,kl->ij", eri, Da))).max() < 1e-11
    assert np.abs(unpack(F2[1], n) - (0.9 * Jt - 0.7 * np.einsum("ikjl,kl->ij", eri, Db))).max() < 1e-11


def test_one_electron_two_implementations_agree(oracle_lib):
    from openqp_gb300 import onee
    for basis in ("6-31g*", "cc-pvdz"):
        bas = h2o_basis(basis)
        o = oracle_lib.Oracle(bas)
        S, T = onee.overlap_kinetic(bas)
        assert np.abs(o.one_electron("S") - S).max() < 1e-13
        assert np.abs(o.one_electron("T") - T).max() < 1e-12
        assert np.abs(o.one_electron("V") - onee.nuclear(bas)).max() < 1e-12


@pytest.mark.parametrize("case", [c for c in GOLD if "GRADIENT" not in c["source"] and "TDHF" not in c["source"]],
                         ids=lambda c: c["source"].split("/")[-1])
def test_golden_hf_energy(oracle_lib, case):
    """OpenQP's own example energies; their CI gate is 4 decimals, we ask 1e-7."""
    from openqp_gb300 import onee, scf
    from openqp_gb300.basis import build_basis
    bas = build_basis(case["atoms"], np.array(case["coord_bohr"]).reshape(-1, 3), case["basis"])
    o = oracle_lib.Oracle(bas, cutoff=1e-10)
    S, T = onee.overlap_kinetic(bas)
    H = T + onee.nuclear(bas)
    nel = int(sum(case["atoms"]))
    nunp = case["multiplicity"] - 1
    na, nb = (nel + nunp) // 2, (nel - nunp) // 2
    kind = case["scf"]
    r = scf.run_scf(o.nbf, S, H, onee.nuclear_repulsion(bas), na, nb,
                    lambda d: o.fock_jk(d, urohf=(kind != "rhf")), kind=kind, conv=1e-11)
    assert r["converged"]
    assert abs(r["energy"] - case["energy"]) < 1e-7


def _scf_case(oracle_lib, case, conv=1e-11):
    from openqp_gb300 import onee, scf
    from openqp_gb300.basis import build_basis
    bas = build_basis(case["atoms"], np.array(case["coord_bohr"]).reshape(-1, 3), case["basis"])
    o = oracle_lib.Oracle(bas, cutoff=1e-10)
    S, T = onee.overlap_kinetic(bas)
    H = T + onee.nuclear(bas)
    nel = int(sum(case["atoms"]))
    nunp = case["multiplicity"] - 1
    na, nb = (nel + nunp) // 2, (nel - nunp) // 2
    kind = case["scf"]
    r = scf.run_scf(o.nbf, S, H, onee.nuclear_repulsion(bas), na, nb,
                    lambda d: o.fock_jk(d, urohf=(kind != "rhf")), kind=kind, conv=conv, dconv=1e-9)
    assert r["converged"]
    return bas, o, r, na, nb, kind


@pytest.mark.parametrize("case", [c for c in GOLD if "GRADIENT" in c["source"]], ids=lambda c: c["source"].split("/")[-1])
def test_golden_hf_gradient(oracle_lib, case):
    """OpenQP's example gradients: nuclear repulsion + one-electron part (oracle
    grad1e) + two-electron part (the grd2 restatement, oracle grad2e)."""
    from openqp_gb300 import scf
    from openqp_gb300.basis import unpack
    bas, o, r, na, nb, kind = _scf_case(oracle_lib, case)
    n = bas.nbf
    Ds = [unpack(d, n) for d in r["D"]]
    if kind == "rhf":
        Dt, Dsp = Ds[0], None
    else:
        Dt, Dsp = Ds[0] + Ds[1], Ds[0] - Ds[1]
    W = scf.energy_weighted_density(r, na, nb, kind)
    g = oracle_lib.nuclear_repulsion_gradient(bas) + o.grad1e(Dt, W) + o.grad2e(Dt, Dsp)
    ref = np.array(case["grad"]).reshape(-1, 3)
    assert np.abs(g - ref).max() < 2e-7
    assert np.abs(g.sum(axis=0)).max() < 1e-9   # translational invariance


def test_grad2e_matches_finite_difference_of_e2(oracle_lib):
    """At a fixed AO density, dE2/dR of E2 = 1/2 Tr D G(D) (the two-electron
    energy) by central differences (h = 1e-4 Bohr) against the grd2 restatement."""
    from openqp_gb300 import workloads
    from openqp_gb300.basis import unpack
    bas = workloads.water_cluster_basis(2, 4.0, seed=3, basis="6-31g*")
    d = workloads.density(bas, 10, 3)
    n = bas.nbf
    D = unpack(d, n)
    o = oracle_lib.Oracle(bas)
    g = o.grad2e(D)

    def e2(xyz):
        ob = oracle_lib.Oracle(bas.with_geometry(xyz))
        f = ob.fock_jk(d)[0]
        return 0.5 * np.sum(D * unpack(f, n))

    h = 1e-4
    for at, x in ((0, 2), (1, 0), (4, 1)):
        xp = bas.xyz.copy()
        xp[at, x] += h
        xm = bas.xyz.copy()
        xm[at, x] -= h
        fd = (e2(xp) - e2(xm)) / (2 * h)
        assert abs(fd - g[at, x]) < 2e-7, (at, x, fd, g[at, x])


def mrsf_gamma(d, p, spc, coul, x, x2, q, sgnk):
    """Dense AO two-particle density of grd2_mrsf_compute_data_t_get_density
    (modules/tdhf_mrsf_gradient.F90:404-601) in compact form: the eight-term
    sums of the reference regrouped by index pairing."""
    A, B = d[0] + d[1], d[0] - d[1]
    P, Q = p[0] + p[1], p[0] - p[1]
    bo2v, bo1v, bco1, bco2, o21v, co12, ball = spc
    e = np.einsum
    g = coul * (e("ij,kl->ijkl", A + P, A) + e("ij,kl->ijkl", A, P))

    def ex(X, Y):   # X_ik Y_jl + X_il Y_jk
        return e("ik,jl->ijkl", X, Y) + e("il,jk->ijkl", X, Y)

    g -= x * (ex(A + P, A) + ex(A, P) + ex(B + Q, B) + ex(B, Q))
    g -= 2 * x2 * (ex(ball, ball) + ex(ball.T, ball.T))

    def eight(X):
        return 2 * (e("ik,lj->ijkl", X, X) + e("il,kj->ijkl", X, X) + e("jk,li->ijkl", X, X) + e("jl,ki->ijkl", X, X))

    g += sgnk * (q[0] * eight(co12) + q[1] * eight(o21v))

    def dc(X, Y):
        return (e("ik,jl->ijkl", X, Y) + e("il,jk->ijkl", X, Y) + e("jk,il->ijkl", X, Y) + e("jl,ik->ijkl", X, Y)
                + e("lj,ki->ijkl", X, Y) + e("kj,li->ijkl", X, Y) + e("li,kj->ijkl", X, Y) + e("ki,lj->ijkl", X, Y))

    def dd(X, Y):
        return e("ij,kl->ijkl", X + X.T, Y + Y.T) + e("kl,ij->ijkl", X + X.T, Y + Y.T)

    g += sgnk * q[2] * (-dc(bco1, bo2v) - dc(bco2, bo1v) - dc(bo2v, bco1) - dc(bo1v, bco2)
                        + dd(bco1, bo2v) + dd(bco2, bo1v) + dd(bo2v, bco1) + dd(bo1v, bco2))
    return g


@pytest.mark.parametrize("mrst", [1, 3])
def test_grad2e_mrsf_matches_finite_difference(oracle_lib, mrst):
    """The MRSF two-electron gradient (grd2 with the MRSF two-particle density,
    general non-symmetric response densities) equals central differences
    (h = 1e-4 Bohr) of E2 = 1/8 sum_ijkl Gamma_ijkl (ij|kl) at fixed AO
    densities; Gamma (compact restatement) has the eightfold symmetry."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(1, workloads.cube_edge_like_c1(1), seed=2, basis="6-31g(d)")
    n = bas.nbf
    rng = np.random.default_rng(mrst)
    sym = lambda a: 0.5 * (a + a.swapaxes(-1, -2))
    d, p = sym(rng.standard_normal((2, n, n)) * 0.3), sym(rng.standard_normal((2, n, n)) * 0.3)
    spc = rng.standard_normal((7, n, n)) * 0.3
    x, x2, q = 0.5, 0.45, (0.4, 0.3, 0.2)
    sgnk = -1.0 if mrst == 3 else 1.0
    G = mrsf_gamma(d, p, spc, 4.0, x, x2, q, sgnk)
    for perm in ((1, 0, 2, 3), (0, 1, 3, 2), (2, 3, 0, 1)):
        assert np.abs(G - G.transpose(perm)).max() < 1e-12 * np.abs(G).max()
    o = oracle_lib.Oracle(bas)
    g = o.grad2e_mrsf(d, p, spc, x, x2, 1.0, q, mrst)

    def e2(xyz):
        eri = oracle_lib.Oracle(bas.with_geometry(xyz)).eri_dense().reshape(n, n, n, n)
        return np.sum(G * eri) / 8.0

    h = 1e-4
    for at, c in ((0, 2), (1, 0), (2, 1)):
        xp = bas.xyz.copy()
        xp[at, c] += h
        xm = bas.xyz.copy()
        xm[at, c] -= h
        fd = (e2(xp) - e2(xm)) / (2 * h)
        assert abs(fd - g[at, c]) < 2e-7 * max(1.0, abs(fd)), (at, c, fd, g[at, c])
    assert np.abs(g.sum(axis=0)).max() < 1e-9


def test_grad2e_cam_matches_finite_difference(oracle_lib):
    """grd2_driver's CAM branch (regular pass with hfscale alpha, erf(mu r)/r
    pass with hfscale beta and no Coulomb, its own Schwarz bounds and the
    attenuated primitive screens) against central differences of E2 =
    1/2 Tr D G_CAM(D) from the pinned CAM Fock build."""
    from openqp_gb300 import workloads
    from openqp_gb300.basis import unpack
    bas = workloads.water_cluster_basis(2, 4.0, seed=3, basis="6-31g*")
    d = workloads.density(bas, 10, 3)
    n = bas.nbf
    D = unpack(d, n)
    cam = (0.19, 0.46, 0.33)
    g = oracle_lib.Oracle(bas).grad2e_cam(D, None, *cam)

    def e2(xyz):
        f = oracle_lib.Oracle(bas.with_geometry(xyz)).fock_jk_cam(d, *cam)[0]
        return 0.5 * np.sum(D * unpack(f, n))

    h = 1e-4
    for at, x in ((0, 2), (1, 0), (4, 1)):
        xp = bas.xyz.copy()
        xp[at, x] += h
        xm = bas.xyz.copy()
        xm[at, x] -= h
        fd = (e2(xp) - e2(xm)) / (2 * h)
        assert abs(fd - g[at, x]) < 2e-7, (at, x, fd, g[at, x])


def _dense_jk(o, n):
    eri = o.eri_dense().reshape(n, n, n, n)
    return (lambda D: np.einsum("ijkl,kl->ij", eri, D)), (lambda D: np.einsum("ijkl,jl->ik", eri, D))


@pytest.mark.parametrize("flags", [1, 2, 3, 4, 12])
def test_td_digestion_matches_dense_contraction(oracle_lib, flags):
    """int2_td_data_t update + parallel_stop on general matrices X equals
    A+B = 4 sc J[X] - 2 se K[Xs], A-B = -2 se K[Xa], TDA = 2 sc J[X] - se K[X]."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(1, workloads.cube_edge_like_c1(1), seed=3, basis="6-31g(d)")
    o = oracle_lib.Oracle(bas, cutoff=1e-12)
    n = o.nbf
    J, K = _dense_jk(o, n)
    x = np.random.default_rng(flags).standard_normal((3, n, n)) * 0.3
    se, sc = 0.7, 1.3
    pa, ma = o.fock_td(x, flags, se, sc)
    for v in range(3):
        D = x[v]
        Ds, Da = 0.5 * (D + D.T), 0.5 * (D - D.T)
        ep = np.zeros((n, n))
        em = np.zeros((n, n))
        if flags & 4:
            em = -se * K(D) + (2 * sc * J(D) if flags & 8 else 0)
        else:
            if flags & 1:
                ep = 4 * sc * J(D) - 2 * se * K(Ds)
            if flags & 2:
                em = -2 * se * K(Da)
        assert np.abs(pa[v] - ep).max() < 1e-12
        assert np.abs(ma[v] - em).max() < 1e-12


@pytest.mark.parametrize("nmat", [7, 11])
def test_mrsf_digestion_matches_dense_contraction(oracle_lib, nmat):
    """int2_mrsf_data_t (7) / int2_umrsf_data_t (11) pass 1 equals
    sc J[X] - se K[X] on the Coulomb components, -se K[X] (UMRSF 8, 9: K[X^T])
    on the others."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(1, workloads.cube_edge_like_c1(1), seed=5, basis="6-31g(d)")
    o = oracle_lib.Oracle(bas, cutoff=1e-12)
    n = o.nbf
    J, K = _dense_jk(o, n)
    x = np.random.default_rng(nmat).standard_normal((2, nmat, n, n)) * 0.3
    se, sc = 0.6, 1.2
    f = o.fock_mrsf(x, se, sc)
    ncoul = 4 if nmat == 7 else 8
    for v in range(2):
        for m in range(nmat):
            D = x[v, m]
            ref = -se * K(D.T if (nmat == 11 and m in (8, 9)) else D)
            if m < ncoul:
                ref = ref + sc * J(D)
            assert np.abs(f[v, m] - ref).max() < 1e-12


@pytest.mark.parametrize("flags", [1, 2, 3])
def test_tdgrd_digestion_matches_dense_contraction(oracle_lib, flags):
    """int2_tdgrd_data_t update + the int2_td_data_t parallel_stop on two
    general spin densities equals A+B_s = 2 sc J[X1 + X2] - 2 se K[Xs_s],
    A-B_1 = -2 se K[X1a], A-B_2 = 0."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(1, workloads.cube_edge_like_c1(1), seed=3, basis="6-31g(d)")
    o = oracle_lib.Oracle(bas, cutoff=1e-12)
    n = o.nbf
    J, K = _dense_jk(o, n)
    x = np.random.default_rng(10 + flags).standard_normal((2, n, n)) * 0.3
    se, sc = 0.7, 1.3
    pa, ma = o.fock_tdgrd(x, flags, se, sc)
    for s in range(2):
        ep = 2 * sc * J(x[0] + x[1]) - 2 * se * K(0.5 * (x[s] + x[s].T)) if flags & 1 else 0 * x[s]
        assert np.abs(pa[s] - ep).max() < 1e-12
    em = -2 * se * K(0.5 * (x[0] - x[0].T)) if flags & 2 else 0 * x[0]
    assert np.abs(ma[0] - em).max() < 1e-12
    assert not ma[1].any()


@pytest.mark.parametrize("nspin", [1, 2])
def test_rpagrd_digestion_matches_dense_contraction(oracle_lib, nspin):
    """int2_rpagrd_data_t hplus / hminus + parallel_stop: for symmetric V,
    H+[V] = 4 sc J[V] - 2 se K[V] (nspin 1) or 2 sc J[V1 + V2] - 2 se K[V_s]
    (nspin 2); H-[V] = -2 se K[V1a] in spin 1, zero in spin 2.  A third
    operand slot beyond nspin (the reference's xpy2(:,:,2,:)) is read only by
    the screening."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(1, workloads.cube_edge_like_c1(1), seed=3, basis="6-31g(d)")
    o = oracle_lib.Oracle(bas, cutoff=1e-12)
    n = o.nbf
    J, K = _dense_jk(o, n)
    rng = np.random.default_rng(nspin)
    sym = lambda a: 0.5 * (a + a.swapaxes(-1, -2))
    xpy = sym(rng.standard_normal((2, nspin + 1, n, n)) * 0.3)
    t = sym(rng.standard_normal((1, nspin, n, n)) * 0.3)
    xmy = rng.standard_normal((2, nspin, n, n)) * 0.3
    se, sc = 0.7, 1.3
    hp, ht, hm = o.fock_rpagrd(xpy, xmy, t, nspin, se, sc)

    def hplus(v, s):
        if nspin == 1:
            return 4 * sc * J(v[0]) - 2 * se * K(v[0])
        return 2 * sc * J(v[0] + v[1]) - 2 * se * K(v[s])

    for i in range(2):
        for s in range(nspin):
            assert np.abs(hp[i, s] - hplus(xpy[i], s)).max() < 1e-11
        assert np.abs(hm[i, 0] + 2 * se * K(0.5 * (xmy[i, 0] - xmy[i, 0].T))).max() < 1e-12
        if nspin == 2:
            assert not hm[i, 1].any()
    for s in range(nspin):
        assert np.abs(ht[0, s] - hplus(t[0], s)).max() < 1e-11


def test_rpagrd_screens_xmy_only_with_xpy(oracle_lib):
    """The reference's init_screen adds X-Y to the shell density only when
    X+Y is present: with X-Y alone every quartet is screened out."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(1, workloads.cube_edge_like_c1(1), seed=3, basis="6-31g(d)")
    o = oracle_lib.Oracle(bas, cutoff=1e-12)
    xmy = np.random.default_rng(0).standard_normal((1, 1, o.nbf, o.nbf))
    _, _, hm = o.fock_rpagrd(None, xmy, None, 1)
    assert not hm.any()


@pytest.mark.parametrize("which", [0, 1], ids=["singlet", "triplet"])
def test_golden_mrsf_excitation_energies(oracle_lib, which):
    """OpenQP's h2o_rohf_mrsf-{s,t}_6-31g_hf: ROHF triplet energy and the six
    MRSF-TDHF excitation energies from the oracle's restatement of the native
    sigma triple (mrsfcbc -> int2_mrsf_data_t -> mrsfmntoia + mrsfesum) over
    the full active trial space (their Davidson converges them to ~1e-9)."""
    import mrsf
    from oracle import mrsf_sigma as ms
    from openqp_gb300.basis import build_basis
    case = json.load(open(os.path.join(ROOT, "tests", "golden", "mrsf_golden.json")))["cases"][which]
    o = oracle_lib.Oracle(build_basis(case["atoms"], np.array(case["coord_bohr"]).reshape(-1, 3), case["basis"]))
    bas, r, C, fa, fb, na, nb = mrsf.rohf_reference(case, o.fock_jk)
    assert abs(r["energy"] - case["energy"]) < 1e-8
    mrst = case["mrsf_multiplicity"]
    w = mrsf.mrsf_energies(lambda E: ms.sigma(o.fock_mrsf, E, C, C, fa, fb, na, nb, mrst), bas.nbf, na, nb, mrst, 6)
    assert np.abs(w - np.array(case["td_energies"])).max() < 1e-7


def test_golden_tdhf_excitation_energies(oracle_lib):
    """OpenQP's examples/TDHF/H2O_TDHF_ENERGY: RHF energy and the three RPA
    singlet excitation energies (their Davidson converges them to ~1e-7)."""
    import rpa
    from openqp_gb300 import onee, scf
    from openqp_gb300.basis import build_basis
    case = [c for c in GOLD if "TDHF" in c["source"]][0]
    bas = build_basis(case["atoms"], np.array(case["coord_bohr"]).reshape(-1, 3), case["basis"])
    o = oracle_lib.Oracle(bas, cutoff=1e-10)
    S, T = onee.overlap_kinetic(bas)
    H = T + onee.nuclear(bas)
    r = scf.run_scf(o.nbf, S, H, onee.nuclear_repulsion(bas), 5, 5, lambda d: o.fock_jk(d), conv=1e-12,
                    dconv=1e-10)
    assert abs(r["energy"] - case["energy"]) < 1e-7
    e, C = rpa.canonical_orbitals(S, r["Fock"][0])
    w, apb, amb = rpa.rpa_energies(lambda x, fl: o.fock_td(x, fl), C, e, 5)
    assert np.abs(apb - apb.T).max() < 1e-12 and np.abs(amb - amb.T).max() < 1e-12
    assert np.abs(w[:3] - np.array(case["td_energies"])).max() < 5e-7


@pytest.mark.parametrize("basis", ["6-31g*", "cc-pvdz"])
def test_attenuated_rys_matches_mcmurchie_davidson(oracle_lib, basis):
    bas = h2o_basis(basis)
    o = oracle_lib.Oracle(bas, cutoff=1e-14)
    ns = len(bas.am)
    rng = np.random.default_rng(1)
    for _ in range(60):
        i, j, k, l = (int(v) for v in rng.integers(0, ns, 4))
        for mu in (0.2, 0.33, 1.0, 4.0):
            a, b = o.eri_quartet(i, j, k, l, mu), o.md_quartet(i, j, k, l, mu)
            assert np.abs(a - b).max() < 1e-14 * max(1.0, np.abs(b).max())


def test_cam_builds_match_dense_contraction(oracle_lib):
    """int2_run_cam: pass 1 (1/r) with alpha, alpha_c, pass 2 (erf(mu r)/r,
    attenuated Schwarz) with beta, beta_c, for the RHF / UROHF Fock build, the
    TD build and the MRSF build (pass 2: last component, exchange only)."""
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(1, workloads.cube_edge_like_c1(1), seed=2, basis="6-31g(d)")
    o = oracle_lib.Oracle(bas, cutoff=1e-12)
    n = o.nbf
    e1, e2 = o.eri_dense(), o.eri_dense(mu=0.33)
    J1, K1 = (lambda D: np.einsum("ijkl,kl->ij", e1, D)), (lambda D: np.einsum("ijkl,jl->ik", e1, D))
    J2, K2 = (lambda D: np.einsum("ijkl,kl->ij", e2, D)), (lambda D: np.einsum("ijkl,jl->ik", e2, D))
    from openqp_gb300.basis import pack, unpack
    al, be, mu, ac, bc = 0.19, 0.46, 0.33, 1.0, 0.2
    d = workloads.density(bas, 5, 0)
    D = unpack(d, n)
    f = o.fock_jk_cam(d, al, be, mu, ac, bc)[0]
    ref = pack(ac * J1(D) - 0.5 * al * K1(D) + bc * J2(D) - 0.5 * be * K2(D))
    assert np.abs(f - ref).max() < 1e-11
    du = workloads.density_open(bas, 5, 4, 1)
    Da, Db = unpack(du[0], n), unpack(du[1], n)
    fu = o.fock_jk_cam(du, al, be, mu, ac, bc)
    for s, Ds in enumerate((Da, Db)):
        ref = pack(ac * J1(Da + Db) - al * K1(Ds) + bc * J2(Da + Db) - be * K2(Ds))
        assert np.abs(fu[s] - ref).max() < 1e-11
    x = np.random.default_rng(0).standard_normal((2, n, n)) * 0.3
    pa, ma = o.fock_td_cam(x, 3, al, be, mu, ac, bc)
    for v in range(2):
        X = x[v]
        Xs, Xa = 0.5 * (X + X.T), 0.5 * (X - X.T)
        assert np.abs(pa[v] - (4 * ac * J1(X) - 2 * al * K1(Xs) + 4 * bc * J2(X) - 2 * be * K2(Xs))).max() < 1e-11
        assert np.abs(ma[v] - (-2 * al * K1(Xa) - 2 * be * K2(Xa))).max() < 1e-11
    x3 = np.random.default_rng(1).standard_normal((1, 7, n, n)) * 0.3
    f3 = o.fock_mrsf_cam(x3, al, be, mu, ac, bc)
    for m in range(7):
        X = x3[0, m]
        ref = -al * K1(X) + (ac * J1(X) if m < 4 else 0) - (be * K2(X) if m == 6 else 0)
        assert np.abs(f3[0, m] - ref).max() < 1e-11


@pytest.mark.parametrize("spherical", [True, False])
def test_f_shells_rys_matches_md_and_dense_fock(oracle_lib, spherical):
    """cc-pVTZ water (one f shell on O): Rys f-shell ERIs against
    McMurchie-Davidson, and the Fock build against the dense contraction."""
    from openqp_gb300 import workloads
    from openqp_gb300.basis import pack, unpack
    bas = h2o_basis("cc-pvtz", spherical=spherical)
    o = oracle_lib.Oracle(bas, cutoff=1e-14)
    ns = len(bas.am)
    f = [i for i in range(ns) if bas.am[i] == 3][0]
    rng = np.random.default_rng(5)
    for _ in range(40):
        q = [int(v) for v in rng.integers(0, ns, 4)]
        q[int(rng.integers(0, 4))] = f
        a, b = o.eri_quartet(*q), o.md_quartet(*q)
        assert np.abs(a - b).max() < 1e-14 * max(1.0, np.abs(b).max())
    eri = o.eri_dense()
    d = workloads.density(bas, 5, 0)
    D = unpack(d, bas.nbf)
    ref = pack(np.einsum("ijkl,kl->ij", eri, D) - 0.5 * np.einsum("ijkl,jl->ik", eri, D))
    fk = oracle_lib.Oracle(bas, cutoff=1e-10).fock_jk(d)[0]
    assert np.abs(fk - ref).max() < 1e-10


@pytest.mark.parametrize("spherical", [True, False])
def test_grad2e_f_shells_matches_finite_difference(oracle_lib, spherical):
    """cc-pVTZ water (f on O, d on H): the grd2 restatement with f shells
    (raised g components) against central differences of E2 (h = 1e-4 Bohr)."""
    from openqp_gb300 import workloads
    from openqp_gb300.basis import unpack
    bas = h2o_basis("cc-pvtz", spherical=spherical)
    d = workloads.density(bas, 5, 4)
    n = bas.nbf
    D = unpack(d, n)
    g = oracle_lib.Oracle(bas).grad2e(D)

    def e2(xyz):
        f = oracle_lib.Oracle(bas.with_geometry(xyz), cutoff=1e-12).fock_jk(d)[0]
        return 0.5 * np.sum(D * unpack(f, n))

    h = 1e-4
    for at, x in ((0, 2), (1, 0), (2, 1)):
        xp = bas.xyz.copy()
        xp[at, x] += h
        xm = bas.xyz.copy()
        xm[at, x] -= h
        fd = (e2(xp) - e2(xm)) / (2 * h)
        assert abs(fd - g[at, x]) < 2e-7, (at, x, fd, g[at, x])
    assert np.abs(g.sum(axis=0)).max() < 1e-9


@pytest.mark.parametrize("basis,spherical", [("6-31g*", None), ("cc-pvdz", None), ("cc-pvdz", True)])
def test_rys_matches_mcmurchie_davidson_every_quartet(oracle_lib, basis, spherical):
    """Every canonical shell quartet of one water: the Rys engine (with the
    tables that the GPU kernels share) against the independent McMurchie-
    Davidson engine (Hermite expansion and Boys function, no Rys tables), so a
    table error cannot hide behind agreement between the GPU and the oracle."""
    bas = h2o_basis(basis, spherical=spherical)
    o = oracle_lib.Oracle(bas)
    ns = len(bas.am)
    worst = 0.0
    for i in range(ns):
        for j in range(i + 1):
            for k in range(i + 1):
                for l in range(k + 1):
                    if k == i and l > j:
                        continue
                    worst = max(worst, np.abs(o.eri_quartet(i, j, k, l) - o.md_quartet(i, j, k, l)).max())
    assert worst < 1e-12
