"""The allocation-free Fock build (oqpg_fock_jk_noalloc) against the regular
device entry point (oqpg_fock_jk_device), through the C ABI.

oqpg_fock_jk_noalloc exists for callers that cannot allocate device memory
while they build Fock matrices (a host whose pool allocator owns the device
memory, or a loop that cannot take cudaMalloc's synchronisation); its buffers
live in one static device array.  This file is collected last so that a run
that stops at the first failure has run every other test first; it also runs
alone in a fresh process, where its first call performs the one-time
device-address lookup of that array.
"""
import ctypes

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
    from openqp_gb300 import _lib, fock
    return torch, _lib.lib(), fock


def _noalloc(L, fb, d, torch):
    out = torch.full_like(d, float("nan"))
    st = torch.cuda.current_stream()
    rc = L.oqpg_fock_jk_noalloc(fb.h, ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(out.data_ptr()), d.shape[0],
                                1.0, 1.0, ctypes.c_void_p(st.cuda_stream))
    torch.cuda.synchronize()
    return rc, out


def test_noalloc_matches_device_entry_point_on_two_calls(gpu, oracle_lib):
    torch, L, fock = gpu
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(4, 6.0, seed=0, basis="6-31g(d)")
    fb = fock.FockBuilder(bas, cutoff=1e-10)
    o = oracle_lib.Oracle(bas, cutoff=1e-10)
    d_rhf = torch.from_numpy(workloads.density(bas, 20, 0)[None]).cuda()
    d_uhf = torch.from_numpy(workloads.density_open(bas, 21, 19, 1)).cuda()
    for d in (d_rhf, d_uhf):   # two calls in a row on the shared scratch array
        ref = fb.fock_jk_device(d).cpu().numpy()
        rc, out = _noalloc(L, fb, d, torch)
        assert rc == 0
        assert np.abs(out.cpu().numpy() - ref).max() < TOL
        assert np.abs(out.cpu().numpy() - o.fock_jk(d.cpu().numpy()).reshape(ref.shape)).max() < TOL
    rc, out = _noalloc(L, fb, d_rhf, torch)   # and once more after a different call
    assert rc == 0
    assert np.abs(out.cpu().numpy() - fb.fock_jk_device(d_rhf).cpu().numpy()).max() < TOL


def test_noalloc_builds_in_fp64_whatever_the_precision_split(gpu, oracle_lib):
    """The context's precision split does not apply: the result stays at the
    plain-FP64 gate against the oracle while the device entry point builds in
    the split mode."""
    torch, L, fock = gpu
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(5, workloads.cube_edge_like_c1(5), seed=3, basis="6-31g(d)")
    fb = fock.FockBuilder(bas, cutoff=1e-10)
    d = torch.from_numpy(workloads.density(bas, 25, 3)[None]).cuda()
    ref = oracle_lib.Oracle(bas, cutoff=1e-10).fock_jk(d.cpu().numpy()).reshape(1, -1)
    # a bound of 1: nearly every quartet in FP32 with FP32 roots, visibly off the FP64 result
    fb.set_precision("mixed-fast", 1.0)
    f_split = fb.fock_jk_device(d).cpu().numpy()
    assert fb.stats()["f32_quartets"] > 0 and np.abs(f_split - ref).max() > 100 * TOL
    rc, out = _noalloc(L, fb, d, torch)
    assert rc == 0
    assert np.abs(out.cpu().numpy() - ref).max() < TOL


def test_noalloc_rejects_molecules_beyond_its_limit(gpu):
    torch, L, fock = gpu
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(16, workloads.cube_edge_like_c1(16), seed=0, basis="6-31g(d)")
    assert bas.nbf > 128
    fb = fock.FockBuilder(bas, cutoff=1e-10)
    d = torch.zeros((1, fb.ntri), dtype=torch.float64, device="cuda")
    rc, _ = _noalloc(L, fb, d, torch)
    assert rc == 5


def test_noalloc_rejects_too_many_quartets_after_screening(gpu):
    """nbf and nshell within the limits (96 each) but ~1e7 screened quartets
    (48 hydrogen atoms on a compact 4 x 4 x 3 lattice, 2 bohr apart, 6-31G,
    cutoff 1e-12): status 5 from the screening pass, the caller's output
    untouched."""
    torch, L, fock = gpu
    from openqp_gb300 import workloads
    from openqp_gb300.basis import build_basis
    xyz = np.array([[2.0 * i, 2.0 * j, 2.0 * k] for i in range(4) for j in range(4) for k in range(3)])
    bas = build_basis([1] * len(xyz), xyz, "6-31g")
    assert bas.nbf <= 128 and len(bas.am) <= 128
    fb = fock.FockBuilder(bas, cutoff=1e-12)
    d = torch.from_numpy(workloads.density(bas, 24, 1)[None]).cuda()
    rc, out = _noalloc(L, fb, d, torch)
    assert rc == 5
    assert bool(torch.isnan(out).all())
    # the context stays usable for the regular entry point
    assert torch.isfinite(fb.fock_jk_device(d)).all()
