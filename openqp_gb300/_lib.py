"""Loader of libopenqp_gb300.so (the CUDA library behind the C ABI).

There is no CPU fallback: if the library is missing or no CUDA device is
usable, every entry point raises.
"""
import ctypes
import os

from . import build as _build

_lib = None
_d = ctypes.POINTER(ctypes.c_double)
_i = ctypes.POINTER(ctypes.c_int)

STATUS = {0: "ok", 1: "not initialised", 2: "out of device memory", 3: "unsupported input", 4: "device error"}


class FockError(RuntimeError):
    def __init__(self, code, what):
        super().__init__("%s failed: %s (status %d)" % (what, STATUS.get(code, "unknown"), code))
        self.code = code


def lib():
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            raise RuntimeError("libopenqp_gb300.so is not built (%s); run openqp_gb300.build.build() "
                               "or __graft_entry__.build() first" % path)
        L = ctypes.CDLL(path)
        L.oqpg_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, _i, _i, _i, _d, _d, _i, ctypes.c_int,
                                  _d, ctypes.c_double]
        L.oqpg_destroy.argtypes = [ctypes.c_void_p]
        L.oqpg_nbf.argtypes = [ctypes.c_void_p]
        L.oqpg_fock_jk.argtypes = [ctypes.c_void_p, _d, _d, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.oqpg_fock_jk_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_void_p]
        L.oqpg_fock_jk_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                           ctypes.c_double, ctypes.c_double, ctypes.c_void_p]
        L.oqpg_schwarz.argtypes = [ctypes.c_void_p, _d]
        L.oqpg_stats.argtypes = [ctypes.c_void_p, _d, ctypes.c_int]
        L.oqpg_class_l.argtypes = [ctypes.c_int, _i]
        L.oqpg_measure_fp64_peak.argtypes = [ctypes.c_int, _d]
        L.oqpg_math_check.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong]
        L.oqpg_set_precision.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double]
        L.routec_fock_set_precision.argtypes = [ctypes.c_int, ctypes.c_double]
        L.oqpg_set_cutoff.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.oqpg_get_cutoff.argtypes = [ctypes.c_void_p]
        L.oqpg_get_cutoff.restype = ctypes.c_double
        L.routec_fock_set_cutoff.argtypes = [_d, _i]
        L.routec_fock_set_cutoff.restype = None
        L.oqpg_set_symmetry.argtypes = [ctypes.c_void_p, ctypes.c_int, _i, _i, _d]
        L.oqpg_symmetry_info.argtypes = [ctypes.c_void_p, _i, _i]
        _ll = ctypes.POINTER(ctypes.c_longlong)
        L.routec_fock_set_symmetry.argtypes = [_i, _ll, _ll, _d, _i]
        L.routec_fock_set_symmetry.restype = None
        L.routec_fock_init.argtypes = [ctypes.c_int, _i, _i, _i, _d, _d, _i, ctypes.c_int, _d, ctypes.c_double]
        L.routec_fock_jk.argtypes = [_d, _d, _i, _i, _d, _d, _i]
        L.routec_fock_jk.restype = None
        L.routec_fock_jk_inc.argtypes = [_d, _d, _d, _i, _i, _d, _d, _i]
        L.routec_fock_jk_inc.restype = None
        L.routec_fock_finalize.restype = None
        L.oqpg_create_batch.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, _i, _i, _i, _i, _i, _d, _d, _i,
                                        _d, ctypes.c_double]
        L.oqpg_batch_info.argtypes = [ctypes.c_void_p, _i, ctypes.POINTER(ctypes.c_longlong)]
        L.oqpg_fock_jk_graph.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_void_p]
        L.oqpg_graph_info.argtypes = [ctypes.c_void_p, _i, _i, _i]
        L.oqpg_set_tuning.argtypes = [ctypes.c_void_p, _i, _i, _i]
        L.oqpg_get_tuning.argtypes = [ctypes.c_void_p, _i, _i, _i]
        L.oqpg_set_kernel_family.argtypes = [ctypes.c_void_p, _i]
        L.oqpg_get_kernel_family.argtypes = [ctypes.c_void_p, _i, _i]
        L.oqpg_set_shell_families.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.oqpg_shell_families_info.argtypes = [ctypes.c_void_p, _i, _i]
        L.routec_fock_init_batch.argtypes = [ctypes.c_int, _i, _i, _i, _i, _i, _d, _d, _i, _d, ctypes.c_double]
        L.routec_fock_jk_batch.argtypes = [_d, _d, _i, _i, _d, _d, _i]
        L.routec_fock_jk_batch.restype = None
        L.oqpg_grad2.argtypes = [ctypes.c_void_p, _d, ctypes.c_int, ctypes.c_double, ctypes.c_double, _d]
        L.oqpg_grad2_bilinear.argtypes = [ctypes.c_void_p, _d, _d, _d, _d, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_double, _d]
        L.oqpg_grad2_mrsf.argtypes = [ctypes.c_void_p, _d, _d, _d, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      _d, ctypes.c_int, _d]
        L.oqpg_grad2_cam.argtypes = [ctypes.c_void_p, _d, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_double, _d]
        L.oqpg_grad2_mrsf_cam.argtypes = [ctypes.c_void_p, _d, _d, _d, _d, _d, ctypes.c_int, _d]
        L.oqpg_grad2_sf.argtypes = [ctypes.c_void_p, _d, _d, _d, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                    _d]
        L.routec_grad2_mrsf.argtypes = [_d, _d, _d, _d, _d, _i, _i, _d, _d, _d, _d, _i, _i]
        L.routec_grad2_mrsf.restype = None
        L.oqpg_grad_stats.argtypes = [ctypes.c_void_p, _d, ctypes.c_int]
        L.routec_grad2.argtypes = [_d, _d, _d, _i, _i, _d, _d, _i]
        L.routec_grad2.restype = None
        L.oqpg_one_electron.argtypes = [ctypes.c_int, _i, _i, _i, _d, _d, _i, ctypes.c_int, _d, _d, ctypes.c_int, _d]
        L.oqpg_fock_td.argtypes = [ctypes.c_void_p, _d, _d, _d, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                   ctypes.c_double]
        L.oqpg_fock_td_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_void_p]
        L.oqpg_fock_mrsf.argtypes = [ctypes.c_void_p, _d, _d, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_double]
        L.oqpg_fock_mrsf_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_void_p]
        L.routec_fock_td.argtypes = [_d, _d, _d, _i, _i, _i, _d, _d, _i]
        L.routec_fock_td.restype = None
        L.routec_fock_mrsf.argtypes = [_d, _d, _i, _i, _i, _d, _d, _i]
        L.routec_fock_mrsf.restype = None
        L.oqpg_fock_jk_cam.argtypes = [ctypes.c_void_p, _d, _d, ctypes.c_int, _d]
        L.oqpg_fock_jk_cam_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, _d,
                                              ctypes.c_void_p]
        L.oqpg_fock_td_cam.argtypes = [ctypes.c_void_p, _d, _d, _d, ctypes.c_int, ctypes.c_int, _d]
        L.oqpg_fock_mrsf_cam.argtypes = [ctypes.c_void_p, _d, _d, ctypes.c_int, ctypes.c_int, _d]
        L.routec_fock_jk_cam.argtypes = [_d, _d, _i, _i, _d, _i]
        L.routec_fock_jk_cam.restype = None
        L.oqpg_fock_tdgrd.argtypes = [ctypes.c_void_p, _d, _d, _d, ctypes.c_int, ctypes.c_double, ctypes.c_double, _d]
        L.oqpg_fock_tdgrd_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                             ctypes.c_int, ctypes.c_double, ctypes.c_double, _d, ctypes.c_void_p]
        _rpa = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                ctypes.c_double, ctypes.c_double, _d]
        L.oqpg_fock_rpagrd.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + _rpa
        L.oqpg_fock_rpagrd_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + _rpa + [ctypes.c_void_p]
        L.routec_fock_tdgrd.argtypes = [_d, _d, _d, _i, _i, _d, _d, _d, _i]
        L.routec_fock_tdgrd.restype = None
        L.routec_fock_rpagrd.argtypes = [_d, _i, _i, _d, _i, _i, _d, _i, _i, _i, _i, _d, _d, _d, _d, _d, _d, _i]
        L.routec_fock_rpagrd.restype = None
        L.routec_sig_init.argtypes = [_i, _d, _d, _d, _d, _i, _i, _i]
        L.routec_sig_set_scale.argtypes = [_d]
        L.routec_sig_set_scale.restype = None
        L.routec_sig_iter.argtypes = [_d, _i, _d, _i]
        L.routec_sig_iter.restype = None
        L.oqpg_sig_iter_device.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.routec_sig_free.argtypes = []
        L.routec_sig_free.restype = None
        _lib = L
    return _lib


def ptr(a, t=_d):
    return a.ctypes.data_as(t)
