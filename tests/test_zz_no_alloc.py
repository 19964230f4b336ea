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


def test_noalloc_matches_device_entry_point_on_two_calls(gpu):
    torch, L, fock = gpu
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(4, 6.0, seed=0, basis="6-31g(d)")
    fb = fock.FockBuilder(bas, cutoff=1e-10)
    d_rhf = torch.from_numpy(workloads.density(bas, 20, 0)[None]).cuda()
    d_uhf = torch.from_numpy(workloads.density_open(bas, 21, 19, 1)).cuda()
    for d in (d_rhf, d_uhf):   # two calls in a row on the shared scratch array
        ref = fb.fock_jk_device(d).cpu().numpy()
        rc, out = _noalloc(L, fb, d, torch)
        assert rc == 0
        assert np.abs(out.cpu().numpy() - ref).max() < TOL
    rc, out = _noalloc(L, fb, d_rhf, torch)   # and once more after a different call
    assert rc == 0
    assert np.abs(out.cpu().numpy() - fb.fock_jk_device(d_rhf).cpu().numpy()).max() < TOL


def test_noalloc_rejects_molecules_beyond_its_limit(gpu):
    torch, L, fock = gpu
    from openqp_gb300 import workloads
    bas = workloads.water_cluster_basis(16, workloads.cube_edge_like_c1(16), seed=0, basis="6-31g(d)")
    assert bas.nbf > 128
    fb = fock.FockBuilder(bas, cutoff=1e-10)
    d = torch.zeros((1, fb.ntri), dtype=torch.float64, device="cuda")
    rc, _ = _noalloc(L, fb, d, torch)
    assert rc == 5
