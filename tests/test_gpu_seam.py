"""GPU tests of the seam entry points around routec_fock_jk, called through
the C ABI as OpenQP's bridge would call them, against the oracle:

* routec_fock_jk_inc: fock_jk's f_old branch (OpenQP scf_addons.F90:1207-1210,
  f = f + f_old; f_old = f), whose build runs on the difference density
  D - D_old (scf_addons.F90:2036-2043);
* routec_fock_set_cutoff / FockBuilder.set_cutoff: the run-time cutoff of
  int2_compute_t_set_cutoff (int2.F90:480-496) that the progressive-screening
  SCF changes before every build (scf.F90:721-734).

Tolerance: 1e-10 max-abs on the packed matrices (the plain-FP64 gate).
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


def _water4(seed):
    from openqp_gb300 import workloads
    return workloads.water_cluster_basis(4, 6.0, seed=seed, basis="6-31g(d)")


@pytest.mark.parametrize("open_shell", [False, True])
def test_routec_fock_jk_inc(gpu, oracle_lib, open_shell):
    """F = F_old + G(dD) through the seam, F_old overwritten with F.  The
    reference builds G(dD) with dD's own screening, so the oracle's
    G(D1) + G(D2 - D1) is the exact counterpart; G(D2) agrees to the
    screening error."""
    from openqp_gb300 import workloads
    bas = _water4(3)
    if open_shell:
        d1 = workloads.density_open(bas, 21, 19, 3)
        d2 = workloads.density_open(bas, 21, 19, 4)
        nf, se, sc = 2, 0.8, 1.1
    else:
        d1 = workloads.density(bas, 20, 3)[None]
        d2 = workloads.density(bas, 20, 4)[None]
        nf, se, sc = 1, 1.0, 1.0
    o = oracle_lib.Oracle(bas)
    g1 = o.fock_jk(d1, se=se, sc=sc).reshape(nf, -1)
    gdd = o.fock_jk(d2 - d1, se=se, sc=sc).reshape(nf, -1)
    assert gpu.routec_init(bas, 1e-10) == 0
    f_old = np.ascontiguousarray(g1.copy())
    f, info = gpu.routec_fock_jk_inc(d2 - d1, f_old, bas.nbf, nf, se=se, sc=sc)
    assert info == 0
    assert np.abs(f - (g1 + gdd)).max() < TOL
    assert np.array_equal(f_old, f)
    g2 = o.fock_jk(d2, se=se, sc=sc).reshape(nf, -1)
    assert np.abs(f - g2).max() < 1e-8
    # a second increment accumulates onto the updated f_old
    f2, info = gpu.routec_fock_jk_inc(d1 - d2, f_old, bas.nbf, nf, se=se, sc=sc)
    assert info == 0
    assert np.abs(f2 - (g1 + gdd - gdd)).max() < 2 * TOL
    assert np.array_equal(f_old, f2)
    gpu.routec_finalize()


def test_routec_set_cutoff_loosen_and_tighten(gpu, oracle_lib):
    """A loose build (tau = 1e-6) matches the oracle's build at that cutoff;
    re-tightening to the registered 1e-10 matches the tight oracle again;
    a cutoff below the registered one (1e-12) rebuilds the pair tables."""
    from openqp_gb300 import workloads
    bas = _water4(5)
    d = workloads.density(bas, 20, 5)
    ref = {t: oracle_lib.Oracle(bas, cutoff=t).fock_jk(d) for t in (1e-6, 1e-10, 1e-12)}
    assert np.abs(ref[1e-6] - ref[1e-10]).max() > 10 * TOL   # the cutoff matters for this case
    assert gpu.routec_init(bas, 1e-10) == 0
    for tau in (1e-6, 1e-10, 1e-12, 1e-6, 1e-10):
        assert gpu.routec_fock_set_cutoff(tau) == 0
        f, info = gpu.routec_fock_jk(d, bas.nbf, 1)
        assert info == 0
        assert np.abs(f - ref[tau]).max() < TOL, tau
    assert gpu.routec_fock_set_cutoff(0.0) == 3
    assert gpu.routec_fock_set_cutoff(float("nan")) == 3
    gpu.routec_finalize()
    assert gpu.routec_fock_set_cutoff(1e-10) == 1


def test_set_cutoff_device_and_graph_paths(gpu, oracle_lib):
    """The explicit-context API: device builds and captured-graph replays
    follow the cutoff (the graph is recaptured when it changes)."""
    import torch
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(6, workloads.cube_edge_like_c1(6), seed=7, basis="cc-pvdz")
    d = workloads.density(bas, 30, 7)
    fb = gpu.FockBuilder(bas, cutoff=1e-10)
    dt = torch.from_numpy(d[None]).cuda()
    for tau in (1e-10, 1e-7, 1e-10):
        fb.set_cutoff(tau)
        assert fb.get_cutoff() == tau and fb.cutoff == tau
        ref = oracle_lib.Oracle(bas, cutoff=tau).fock_jk(d)
        assert np.abs(fb.fock_jk_device(dt).cpu().numpy() - ref).max() < TOL
        for _ in range(2):
            assert np.abs(fb.fock_jk_graph(dt).cpu().numpy() - ref).max() < TOL
    with pytest.raises(gpu.FockError):
        fb.set_cutoff(-1.0)
