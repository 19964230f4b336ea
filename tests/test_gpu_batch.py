"""GPU: batched builds of many molecules of uneven size in one context, the
captured-graph replay, the batch seam and the per-class launch tuning.

Every molecule of a batch must get the Fock matrix the oracle gives it alone
(1e-10 max-abs, the plain-FP64 gate); graph replays and tuned launches must
agree with the direct build to 1e-12 (only the order of atomic additions
differs).
"""
import numpy as np
import pytest

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


def _batch(sizes, basis="6-31g", seed=7, open_shell=False):
    from openqp_gb300 import workloads
    from openqp_gb300.onee import one_electron
    bases, dens = [], []
    for k, n in enumerate(sizes):
        bas = workloads.water_cluster_basis(n, workloads.cube_edge_like_c1(n), seed * 1000 + k, basis)
        S = one_electron(bas)[0]
        ne = workloads.nelectrons(bas)
        if open_shell:
            d = workloads.density_open(bas, ne // 2 + 1, ne // 2 - 1, seed + k, S=S)
        else:
            d = workloads.density(bas, ne // 2, seed + k, S=S)[None]
        bases.append(bas)
        dens.append(d)
    return bases, dens


def test_batch_matches_oracle_per_molecule(gpu, oracle_lib):
    sizes = [1, 3, 2, 5, 4, 1]
    bases, dens = _batch(sizes)
    bb = gpu.BatchFockBuilder(bases)
    assert bb.nmol == len(sizes)
    assert bb.nbf == sum(b.nbf for b in bases)
    fs = bb.fock_jk(dens)
    for bas, d, f in zip(bases, dens, fs):
        ref = oracle_lib.Oracle(bas).fock_jk(d)
        assert np.abs(f - ref).max() < TOL
    st = bb.stats()
    assert st["quartets"] > 0 and st["launches"] > 0


def test_batch_uhf_and_scales_match_single_builds(gpu):
    sizes = [2, 1, 3]
    bases, dens = _batch(sizes, open_shell=True, seed=3)
    bb = gpu.BatchFockBuilder(bases)
    fs = bb.fock_jk(dens, scale_exch=0.7, scale_coul=1.2)
    for bas, d, f in zip(bases, dens, fs):
        ref = gpu.FockBuilder(bas).fock_jk(d, scale_exch=0.7, scale_coul=1.2)
        assert f.shape == (2, bas.nbf * (bas.nbf + 1) // 2)
        assert np.abs(f - ref).max() < 1e-12


def test_batch_pure_d(gpu, oracle_lib):
    bases, dens = _batch([2, 1], basis="cc-pvdz", seed=11)
    fs = gpu.BatchFockBuilder(bases).fock_jk(dens)
    for bas, d, f in zip(bases, dens, fs):
        assert np.abs(f - oracle_lib.Oracle(bas).fock_jk(d)).max() < TOL


def test_graph_replay_matches_direct(gpu):
    import torch
    bases, dens = _batch([3, 1, 4, 2], seed=5)
    bb = gpu.BatchFockBuilder(bases)
    d1 = torch.from_numpy(bb.pack(dens)[None]).cuda()
    # a second density on the same molecules: another seed of the random orbitals
    from openqp_gb300 import workloads
    from openqp_gb300.onee import one_electron
    alt = [workloads.density(b, workloads.nelectrons(b) // 2, 99 + k, S=one_electron(b)[0])[None]
           for k, b in enumerate(bases)]
    d2 = torch.from_numpy(bb.pack(alt)[None]).cuda()
    ref1 = bb.fock_jk_device(d1).clone()
    ref2 = bb.fock_jk_device(d2).clone()
    g1 = bb.fock_jk_graph(d1).clone()      # direct build + capture
    g2 = bb.fock_jk_graph(d2).clone()      # replay
    g1b = bb.fock_jk_graph(d1).clone()     # replay
    info = bb.graph_info()
    assert info["captures"] == 1 and info["replays"] >= 1 and info["kernels"] > 0
    for a, b in ((g1, ref1), (g2, ref2), (g1b, ref1)):
        assert float((a - b).abs().max()) < 1e-12


def test_graph_recaptures_when_lists_outgrow(gpu):
    """Capture on a weak density (few quartets survive the density screen),
    replay on the full one: the replay must notice and rebuild."""
    import torch
    bases, dens = _batch([4, 2], seed=9)
    bb = gpu.BatchFockBuilder(bases)
    d = torch.from_numpy(bb.pack(dens)[None]).cuda()
    weak = d * 1e-4
    bb.fock_jk_graph(weak)
    assert bb.graph_info()["captures"] == 1
    got = bb.fock_jk_graph(d).clone()
    ref = bb.fock_jk_device(d)
    assert float((got - ref).abs().max()) < 1e-12
    assert bb.graph_info()["captures"] == 2
    # and the weak density again, now from the larger capture
    got_w = bb.fock_jk_graph(weak).clone()
    assert float((got_w - bb.fock_jk_device(weak)).abs().max()) < 1e-14


def test_single_molecule_graph_matches_oracle(gpu, oracle_lib):
    import torch
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(4, 6.0, seed=1, basis="6-31g(d)")
    d = workloads.density(bas, 20, 1)
    fb = gpu.FockBuilder(bas)
    dt = torch.from_numpy(d[None]).cuda()
    fb.fock_jk_graph(dt)
    f = fb.fock_jk_graph(dt).cpu().numpy()[0]
    assert fb.graph_info()["replays"] == 1
    assert np.abs(f - oracle_lib.Oracle(bas).fock_jk(d)).max() < TOL


def test_batch_mixed_precision_graph(gpu):
    import torch
    bases, dens = _batch([4, 3, 5], seed=13)
    bb = gpu.BatchFockBuilder(bases)
    d = torch.from_numpy(bb.pack(dens)[None]).cuda()
    f64 = bb.fock_jk_device(d).clone()
    bb.set_precision("mixed-fast", 1e-6)
    bb.fock_jk_graph(d)
    fm = bb.fock_jk_graph(d).clone()
    assert bb.stats()["f32_quartets"] > 0
    df = (fm - f64).cpu().numpy()[0]
    assert np.abs(df).max() < 1e-7
    # two-electron energy error per molecule, 1/2 Tr(D dF)
    from openqp_gb300.basis import unpack
    for m, (bas, dm) in enumerate(zip(bases, dens)):
        o = bb.tri0[m]
        t = bas.nbf * (bas.nbf + 1) // 2
        de = 0.5 * np.sum(unpack(dm[0], bas.nbf) * unpack(df[o:o + t], bas.nbf))
        assert abs(de) < 1e-6


def test_routec_batch_seam(gpu):
    import ctypes
    from openqp_gb300._lib import lib, ptr, _i
    from openqp_gb300.fock import _batch_arrays
    bases, dens = _batch([2, 3], seed=17)
    nshell, natom, k = _batch_arrays(bases)
    rc = lib().routec_fock_init_batch(len(bases), ptr(nshell, _i), ptr(natom, _i), ptr(k[0], _i), ptr(k[1], _i),
                                      ptr(k[2], _i), ptr(k[3]), ptr(k[4]), ptr(k[5], _i), ptr(k[6]), 1e-10)
    assert rc == 0
    bb = gpu.BatchFockBuilder(bases)
    dflat = bb.pack(dens)
    f = np.zeros_like(dflat)
    info = ctypes.c_int(1)
    nm, nf = ctypes.c_int(len(bases)), ctypes.c_int(1)
    se, sc = ctypes.c_double(1.0), ctypes.c_double(1.0)
    for _ in range(2):  # capture, then replay
        lib().routec_fock_jk_batch(ptr(dflat), ptr(f), ctypes.byref(nm), ctypes.byref(nf), ctypes.byref(se),
                                   ctypes.byref(sc), ctypes.byref(info))
        assert info.value == 0
        ref = bb.pack(bb.fock_jk(dens))
        assert np.abs(f - ref).max() < 1e-12
    bad = ctypes.c_int(3)
    lib().routec_fock_jk_batch(ptr(dflat), ptr(f), ctypes.byref(bad), ctypes.byref(nf), ctypes.byref(se),
                               ctypes.byref(sc), ctypes.byref(info))
    assert info.value == 1
    gpu.routec_finalize()


def test_tuning_changes_launches_not_results(gpu):
    import torch
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(6, workloads.cube_edge_like_c1(6), seed=2, basis="6-31g(d)")
    d = workloads.density(bas, 30, 2)
    fb = gpu.FockBuilder(bas)
    ref = fb.fock_jk(d)
    nc = gpu.NCLASS
    for split, chunk, ctas in ((6, 64, 1), (64, 128, 2), (10, 32, 0)):
        fb.set_tuning([split] * nc, [chunk] * nc, [ctas] * nc)
        assert fb.get_tuning()["chunk"] == [chunk] * nc
        assert np.abs(fb.fock_jk(d) - ref).max() < 1e-12
    with pytest.raises(gpu.FockError):
        fb.set_tuning(chunk=[33] * nc)
    # the kernel family of the classes that have both (28-108 elements): thread
    # per quartet, warp per quartet, by list size -- the same matrices
    fam, avail = fb.get_kernel_family()
    assert fam == [0] * nc and 3 in avail and avail[0] == 1 and avail[20] == 2
    for f in (1, 2, 0):
        fb.set_kernel_family([f] * nc)
        assert np.abs(fb.fock_jk(d) - ref).max() < 1e-12
    with pytest.raises(gpu.FockError):
        fb.set_kernel_family([3] * nc)


def test_autotune_picks_and_persists(gpu, tmp_path):
    import torch
    from openqp_gb300 import autotune, workloads
    bas = workloads.water_cluster_basis(4, 6.0, seed=4, basis="6-31g(d)")
    d = workloads.density(bas, 20, 4)
    fb = gpu.FockBuilder(bas)
    ref = fb.fock_jk(d)
    dt = torch.from_numpy(d[None]).cuda()
    cache = str(tmp_path / "tune.json")
    t = autotune.autotune(fb, dt, "water4", cache=cache, reps=1)
    assert not t["cached"] and len(t["split_log2"]) == gpu.NCLASS
    assert np.abs(fb.fock_jk(d) - ref).max() < 1e-12
    fb2 = gpu.FockBuilder(bas)
    t2 = autotune.autotune(fb2, dt, "water4", cache=cache)
    assert t2["cached"] and fb2.get_tuning()["split_log2"] == t["split_log2"]
