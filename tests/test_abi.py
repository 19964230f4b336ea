"""CPU-side checks of the C ABI: the library builds and loads, it exports every
symbol the public header declares, and host-side input validation declines
unsupported inputs before touching a device."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def libgpu():
    from openqp_gb300 import build
    build.build()
    from openqp_gb300 import _lib
    return _lib.lib()


def test_exports_every_declared_symbol(libgpu):
    hdr = open(os.path.join(ROOT, "include", "openqp_gb300.h")).read()
    names = set(re.findall(r"^\s*(?:int|void|double)\s+\**\s*(\w+)\s*\(", hdr, re.M))
    assert {"routec_fock_jk", "routec_fock_init", "oqpg_create"} <= names
    for n in names:
        assert hasattr(libgpu, n), n


def test_unsupported_angular_momentum_is_declined(libgpu):
    from openqp_gb300.basis import build_basis
    from openqp_gb300.fock import _basis_arrays
    from openqp_gb300._lib import ptr, _i
    bas = build_basis([8], np.zeros((1, 3)), "6-31g*")
    k = _basis_arrays(bas)
    k[0] = k[0].copy()
    k[0][-1] = 4   # a g shell (s-f are supported)
    h = ctypes.c_void_p()
    rc = libgpu.oqpg_create(ctypes.byref(h), len(bas.am), ptr(k[0], _i), ptr(k[1], _i), ptr(k[2], _i), ptr(k[3]),
                            ptr(k[4]), ptr(k[5], _i), 1, ptr(k[6]), 1e-10)
    assert rc == 3 and not h.value


def test_seam_without_init_declines(libgpu):
    from openqp_gb300 import fock
    f, info = fock.routec_fock_jk(np.zeros(3), 2, 1)
    assert info == 1
    assert fock.routec_fock_set_cutoff(1e-8) == 1
    f, info = fock.routec_fock_jk_inc(np.zeros(3), np.zeros(3), 2, 1)
    assert info == 1
    eye = np.eye(4)
    assert fock.routec_sig_init(eye, eye, eye, eye, 3, 1, 1) == 1
    _, info = fock.routec_sig_iter(np.zeros((9, 1)))
    assert info == 1
    fock.routec_sig_free()


def test_class_table(libgpu):
    from openqp_gb300.fock import class_labels
    lab = class_labels()
    assert len(lab) == 55 and lab[0] == "(ss|ss)" and lab[20] == "(dd|dd)" and lab[-1] == "(ff|ff)"
    assert lab[21] == "(ss|sf)" and lab[27] == "(sf|sf)"
    # class index of every (bra type <= ket type) pair: the s-d block first, then the f block
    seen = set(lab)
    assert len(seen) == 55
