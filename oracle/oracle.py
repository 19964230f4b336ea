"""ctypes wrapper of the oracle (test infrastructure only).

The oracle is a CPU restatement of OpenQP's direct two-electron Fock build
(see oracle_core.cpp / oracle_fock.cpp for the function-by-function citations)
plus an independent McMurchie-Davidson integral code.  Only the tests, the
smoke check and the CPU-baseline leg of bench.py load it, and only as the
checker: the product never routes through it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboqp_oracle.so")
_lib = None

_d = ctypes.POINTER(ctypes.c_double)
_i = ctypes.POINTER(ctypes.c_int)


def build():
    subprocess.check_call(["make", "-s", "-C", HERE])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.c_int, _i, _i, _i, _d, _d, _i, ctypes.c_int, _d, ctypes.c_double]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_nbf.argtypes = [ctypes.c_void_p]
        L.orc_fock_jk.argtypes = [ctypes.c_void_p, _d, _d, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_int, ctypes.c_int, _d, _d]
        L.orc_fock_jk_sample.argtypes = [ctypes.c_void_p, _d, _d, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_int, ctypes.c_int, _d, ctypes.c_int, ctypes.c_int, _d]
        L.orc_schwarz.argtypes = [ctypes.c_void_p, _d, ctypes.c_int]
        L.orc_shlden.argtypes = [ctypes.c_void_p, _d, ctypes.c_int, _d]
        L.orc_eri_quartet.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 4 + [_d]
        L.orc_md_quartet.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 4 + [_d]
        L.orc_eri_quartet_att.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 4 + [ctypes.c_double, _d]
        L.orc_md_quartet_att.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 4 + [ctypes.c_double, _d]
        L.orc_eri_dense.argtypes = [ctypes.c_void_p, _d]
        L.orc_eri_dense_att.argtypes = [ctypes.c_void_p, ctypes.c_double, _d]
        L.orc_one_electron.argtypes = [ctypes.c_void_p, ctypes.c_int, _d, _d]
        L.orc_rys.argtypes = [ctypes.c_int, ctypes.c_double, _d, _d]
        L.orc_boys.argtypes = [ctypes.c_int, ctypes.c_double, _d]
        L.orc_grad2e_mrsf.restype = ctypes.c_longlong
        L.orc_grad2e_mrsf.argtypes = [ctypes.c_void_p, _d, _d, _d, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      _d, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      _d, _d]
        L.orc_grad2e_cam.restype = ctypes.c_longlong
        L.orc_grad2e_cam.argtypes = [ctypes.c_void_p, _d, _d, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_int, _d]
        L.orc_grad2e.restype = ctypes.c_longlong
        L.orc_grad2e.argtypes = [ctypes.c_void_p, _d, _d, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                 ctypes.c_int, ctypes.c_int, ctypes.c_int, _d]
        L.orc_grad1e.argtypes = [ctypes.c_void_p, _d, _d, _d, _d]
        L.orc_fock_td.argtypes = [ctypes.c_void_p, _d, _d, _d, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                  ctypes.c_double, ctypes.c_int]
        L.orc_fock_mrsf.argtypes = [ctypes.c_void_p, _d, _d, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_int]
        L.orc_fock_tdgrd.argtypes = [ctypes.c_void_p, _d, _d, _d, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_int]
        L.orc_fock_rpagrd.argtypes = [ctypes.c_void_p, _d, ctypes.c_int, ctypes.c_int, _d, ctypes.c_int, ctypes.c_int,
                                      _d, ctypes.c_int, ctypes.c_int, ctypes.c_int, _d, _d, _d, ctypes.c_double,
                                      ctypes.c_double, _d, ctypes.c_int]
        L.orc_fock_mrsf_sample.argtypes = [ctypes.c_void_p, _d, _d, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, _d]
        L.orc_fock_tdgrd_cam.argtypes = [ctypes.c_void_p, _d, _d, _d, ctypes.c_int, _d, ctypes.c_int]
        L.orc_fock_jk_cam.argtypes = [ctypes.c_void_p, _d, _d, ctypes.c_int, ctypes.c_int, _d, ctypes.c_int]
        L.orc_fock_jk_cam_sample.argtypes = [ctypes.c_void_p, _d, _d, ctypes.c_int, ctypes.c_int, _d, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_int, _d]
        L.orc_fock_td_cam.argtypes = [ctypes.c_void_p, _d, _d, _d, ctypes.c_int, ctypes.c_int, _d, ctypes.c_int]
        L.orc_fock_mrsf_cam.argtypes = [ctypes.c_void_p, _d, _d, ctypes.c_int, ctypes.c_int, _d, ctypes.c_int]
        L.orc_schwarz_att.argtypes = [ctypes.c_void_p, _d, ctypes.c_int, ctypes.c_double]
        L.orc_fock_td_sample.argtypes = [ctypes.c_void_p, _d, _d, _d, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int, _d]
        _lib = L
    return _lib


def _p(a, t=_d):
    return a.ctypes.data_as(t)


class Oracle:
    """One basis/geometry registered with the oracle."""

    def __init__(self, bas, cutoff=1e-10):
        self.bas = bas
        self._keep = [np.ascontiguousarray(bas.am, dtype=np.int32), np.ascontiguousarray(bas.ncontr, dtype=np.int32),
                      np.ascontiguousarray(bas.origin, dtype=np.int32), np.ascontiguousarray(bas.ex),
                      np.ascontiguousarray(bas.cc), np.ascontiguousarray(bas.harmonic, dtype=np.int32),
                      np.ascontiguousarray(bas.xyz.reshape(-1))]
        k = self._keep
        self.h = lib().orc_create(len(bas.am), _p(k[0], _i), _p(k[1], _i), _p(k[2], _i), _p(k[3]), _p(k[4]),
                                  _p(k[5], _i), int(bas.natom), _p(k[6]), float(cutoff))
        self.nbf = lib().orc_nbf(self.h)
        self.ntri = self.nbf * (self.nbf + 1) // 2

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def fock_jk(self, d, se=1.0, sc=1.0, urohf=None, nthreads=None, schwarz=None):
        """Two-electron Fock part in OpenQP's packed convention.

        d: (ntri,) or (nfocks, ntri).  nfocks == 1 -> RHF consumer, 2 -> UROHF
        consumer (unless urohf is given)."""
        d = np.ascontiguousarray(np.atleast_2d(d), dtype=np.float64)
        nf = d.shape[0]
        if urohf is None:
            urohf = nf == 2
        f = np.zeros_like(d)
        st = np.zeros(8)
        nt = nthreads or os.cpu_count()
        q = None if schwarz is None else _p(np.ascontiguousarray(schwarz))
        lib().orc_fock_jk(self.h, _p(d), _p(f), nf, se, sc, int(urohf), nt, q, _p(st))
        self.last_stats = dict(t_init=st[0], t_schwarz=st[1], t_twoei=st[2], t_total=st[3], quartets=int(st[4]),
                               screened=int(st[5]), prim_quartets=int(st[6]), stored=int(st[7]))
        return f

    def fock_jk_sample(self, d, stride, offset=0, se=1.0, sc=1.0, urohf=None, nthreads=None, schwarz=None):
        """fock_jk over the shell pairs p (cost-sorted order) with p % stride == offset:
        one rank of the reference's round-robin split.  Returns (f, stats)."""
        d = np.ascontiguousarray(np.atleast_2d(d), dtype=np.float64)
        nf = d.shape[0]
        if urohf is None:
            urohf = nf == 2
        f = np.zeros_like(d)
        st = np.zeros(8)
        q = None if schwarz is None else _p(np.ascontiguousarray(schwarz))
        lib().orc_fock_jk_sample(self.h, _p(d), _p(f), nf, se, sc, int(urohf), nthreads or os.cpu_count(), q,
                                 int(stride), int(offset), _p(st))
        return f, dict(t_init=st[0], t_schwarz=st[1], t_twoei=st[2], t_total=st[3], quartets=int(st[4]),
                       screened=int(st[5]), prim_quartets=int(st[6]), stored=int(st[7]))

    def fock_td(self, x, flags, se=1.0, sc=1.0, nthreads=None):
        """int2_td_data_t build: x (nvec, nbf, nbf) natural indexing -> (apb, amb)
        in the same indexing (flags: 1 A+B, 2 A-B, 4 TDA, 8 TDA Coulomb)."""
        x = np.asarray(x, dtype=np.float64)
        fx = np.ascontiguousarray(x.transpose(0, 2, 1))
        pa, ma = np.zeros_like(fx), np.zeros_like(fx)
        lib().orc_fock_td(self.h, _p(fx), _p(pa), _p(ma), fx.shape[0], int(flags), se, sc, nthreads or os.cpu_count())
        return pa.transpose(0, 2, 1), ma.transpose(0, 2, 1)

    def fock_td_sample(self, x, flags, stride, offset=0, se=1.0, sc=1.0, nthreads=None):
        """fock_td over the bra pairs p (cost-sorted) with p % stride == offset.
        Returns (apb, amb, stats) with set-up and loop seconds and the quartet count."""
        x = np.asarray(x, dtype=np.float64)
        fx = np.ascontiguousarray(x.transpose(0, 2, 1))
        pa, ma = np.zeros_like(fx), np.zeros_like(fx)
        st = np.zeros(3)
        lib().orc_fock_td_sample(self.h, _p(fx), _p(pa), _p(ma), fx.shape[0], int(flags), se, sc,
                                 nthreads or os.cpu_count(), int(stride), int(offset), _p(st))
        return pa.transpose(0, 2, 1), ma.transpose(0, 2, 1), dict(t_setup=st[0], t_twoei=st[1], quartets=int(st[2]))

    def fock_tdgrd(self, x, flags, se=1.0, sc=1.0, nthreads=None):
        """int2_tdgrd_data_t build: x (2, nbf, nbf) spin densities, natural
        indexing -> (apb, amb) (2, nbf, nbf) (flags: 1 A+B, 2 A-B)."""
        x = np.asarray(x, dtype=np.float64)
        fx = np.ascontiguousarray(x.transpose(0, 2, 1))
        pa, ma = np.zeros_like(fx), np.zeros_like(fx)
        lib().orc_fock_tdgrd(self.h, _p(fx), _p(pa), _p(ma), int(flags), se, sc, nthreads or os.cpu_count())
        return pa.transpose(0, 2, 1), ma.transpose(0, 2, 1)

    def fock_tdgrd_cam(self, x, flags, alpha, beta, mu, alpha_c=1.0, beta_c=0.0, nthreads=None):
        x = np.asarray(x, dtype=np.float64)
        fx = np.ascontiguousarray(x.transpose(0, 2, 1))
        pa, ma = np.zeros_like(fx), np.zeros_like(fx)
        c = self._cam(alpha, beta, mu, alpha_c, beta_c)
        lib().orc_fock_tdgrd_cam(self.h, _p(fx), _p(pa), _p(ma), int(flags), _p(c), nthreads or os.cpu_count())
        return pa.transpose(0, 2, 1), ma.transpose(0, 2, 1)

    def fock_rpagrd(self, xpy, xmy, t, nspin, se=1.0, sc=1.0, cam=None, nthreads=None):
        """int2_rpagrd_data_t build.  xpy / xmy / t: (nvec, ld, nbf, nbf)
        natural indexing (or None), ld >= nspin -> (hpp, hpt, hmm), each
        (nvec, nspin, nbf, nbf) or None.  cam = (alpha, beta, mu, alpha_c,
        beta_c) runs the two-pass CAM form."""
        n = self.nbf

        def fort(x):
            if x is None:
                return np.zeros((0, 1, n, n)), 1, 0
            x = np.asarray(x, dtype=np.float64)
            return np.ascontiguousarray(x.transpose(0, 1, 3, 2)), x.shape[1], x.shape[0]

        (fp, ldp, np_), (fm, ldm, nm), (ft, ldt, nt) = fort(xpy), fort(xmy), fort(t)
        hp, ht, hm = (np.zeros((k, nspin, n, n)) for k in (np_, nt, nm))
        c = self._cam(*cam) if cam is not None else None
        lib().orc_fock_rpagrd(self.h, _p(fp), ldp, np_, _p(fm), ldm, nm, _p(ft), ldt, nt, int(nspin), _p(hp), _p(ht),
                              _p(hm), se, sc, _p(c) if c is not None else None, nthreads or os.cpu_count())
        out = [h.transpose(0, 1, 3, 2) if k else None for h, k in ((hp, np_), (ht, nt), (hm, nm))]
        return tuple(out)

    def fock_mrsf(self, x, se=1.0, sc=1.0, nthreads=None):
        """int2_mrsf_data_t (nmat 7) / int2_umrsf_data_t (nmat 11) first pass:
        x (nvec, nmat, nbf, nbf) natural indexing -> f3 in the same indexing."""
        x = np.asarray(x, dtype=np.float64)
        fx = np.ascontiguousarray(x.transpose(3, 2, 1, 0))
        out = np.zeros_like(fx)
        rc = lib().orc_fock_mrsf(self.h, _p(fx), _p(out), x.shape[0], x.shape[1], se, sc, nthreads or os.cpu_count())
        if rc:
            raise ValueError("nmat must be 7 or 11")
        return out.transpose(3, 2, 1, 0)

    def fock_mrsf_sample(self, x, stride, offset=0, se=1.0, sc=1.0, nthreads=None):
        """fock_mrsf over the bra pairs p (cost-sorted) with p % stride == offset.
        Returns (f3, stats) with set-up and loop seconds and the quartet count."""
        x = np.asarray(x, dtype=np.float64)
        fx = np.ascontiguousarray(x.transpose(3, 2, 1, 0))
        out = np.zeros_like(fx)
        st = np.zeros(3)
        lib().orc_fock_mrsf_sample(self.h, _p(fx), _p(out), x.shape[0], x.shape[1], se, sc,
                                   nthreads or os.cpu_count(), int(stride), int(offset), _p(st))
        return out.transpose(3, 2, 1, 0), dict(t_setup=st[0], t_twoei=st[1], quartets=int(st[2]))

    # ---- CAM (int2_run_cam): regular pass + erf-attenuated pass ---------------
    @staticmethod
    def _cam(alpha, beta, mu, alpha_c, beta_c):
        return np.array([alpha, beta, mu, alpha_c, beta_c], dtype=np.float64)

    def fock_jk_cam(self, d, alpha, beta, mu, alpha_c=1.0, beta_c=0.0, urohf=None, nthreads=None):
        d = np.ascontiguousarray(np.atleast_2d(d), dtype=np.float64)
        if urohf is None:
            urohf = d.shape[0] == 2
        f = np.zeros_like(d)
        c = self._cam(alpha, beta, mu, alpha_c, beta_c)
        lib().orc_fock_jk_cam(self.h, _p(d), _p(f), d.shape[0], int(urohf), _p(c), nthreads or os.cpu_count())
        return f

    def fock_jk_cam_sample(self, d, alpha, beta, mu, stride, offset=0, alpha_c=1.0, beta_c=0.0, urohf=None,
                           nthreads=None):
        """fock_jk_cam over the bra pairs p with p % stride == offset (both passes). Returns (f, stats)."""
        d = np.ascontiguousarray(np.atleast_2d(d), dtype=np.float64)
        if urohf is None:
            urohf = d.shape[0] == 2
        f = np.zeros_like(d)
        st = np.zeros(8)
        c = self._cam(alpha, beta, mu, alpha_c, beta_c)
        lib().orc_fock_jk_cam_sample(self.h, _p(d), _p(f), d.shape[0], int(urohf), _p(c), nthreads or os.cpu_count(),
                                     int(stride), int(offset), _p(st))
        return f, dict(t_init=st[0], t_schwarz=st[1], t_twoei=st[2], t_total=st[3], quartets=int(st[4]))

    def fock_td_cam(self, x, flags, alpha, beta, mu, alpha_c=1.0, beta_c=0.0, nthreads=None):
        x = np.asarray(x, dtype=np.float64)
        fx = np.ascontiguousarray(x.transpose(0, 2, 1))
        pa, ma = np.zeros_like(fx), np.zeros_like(fx)
        c = self._cam(alpha, beta, mu, alpha_c, beta_c)
        lib().orc_fock_td_cam(self.h, _p(fx), _p(pa), _p(ma), fx.shape[0], int(flags), _p(c),
                              nthreads or os.cpu_count())
        return pa.transpose(0, 2, 1), ma.transpose(0, 2, 1)

    def fock_mrsf_cam(self, x, alpha, beta, mu, alpha_c=1.0, beta_c=0.0, nthreads=None):
        x = np.asarray(x, dtype=np.float64)
        fx = np.ascontiguousarray(x.transpose(3, 2, 1, 0))
        out = np.zeros_like(fx)
        c = self._cam(alpha, beta, mu, alpha_c, beta_c)
        lib().orc_fock_mrsf_cam(self.h, _p(fx), _p(out), x.shape[0], x.shape[1], _p(c), nthreads or os.cpu_count())
        return out.transpose(3, 2, 1, 0)

    def schwarz_att(self, mu, nthreads=None):
        ns = len(self.bas.am)
        q = np.zeros(ns * ns)
        lib().orc_schwarz_att(self.h, _p(q), nthreads or os.cpu_count(), float(mu))
        return q.reshape(ns, ns)

    def schwarz(self, nthreads=None):
        ns = len(self.bas.am)
        q = np.zeros(ns * ns)
        lib().orc_schwarz(self.h, _p(q), nthreads or os.cpu_count())
        return q.reshape(ns, ns)

    def shlden(self, d):
        d = np.ascontiguousarray(np.atleast_2d(d))
        ns = len(self.bas.am)
        out = np.zeros(ns * ns)
        lib().orc_shlden(self.h, _p(d), d.shape[0], _p(out))
        return out.reshape(ns, ns)

    def _shape(self, i, j, k, l):
        return tuple(int(self.bas.naos[s]) for s in (i, j, k, l))

    def eri_quartet(self, i, j, k, l, mu=0.0):
        """Rys block; mu > 0: the erf(mu r)/r operator."""
        sh = self._shape(i, j, k, l)
        out = np.zeros(int(np.prod(sh)))
        lib().orc_eri_quartet_att(self.h, i, j, k, l, float(mu), _p(out))
        return out.reshape(sh)

    def md_quartet(self, i, j, k, l, mu=0.0):
        """McMurchie-Davidson block; mu > 0: the erf(mu r)/r operator."""
        sh = self._shape(i, j, k, l)
        out = np.zeros(int(np.prod(sh)))
        lib().orc_md_quartet_att(self.h, i, j, k, l, float(mu), _p(out))
        return out.reshape(sh)

    def eri_dense(self, mu=0.0):
        """Unscreened (nbf,)*4 tensor; mu > 0: the erf(mu r)/r operator."""
        n = self.nbf
        out = np.zeros(n ** 4)
        lib().orc_eri_dense_att(self.h, float(mu), _p(out))
        return out.reshape(n, n, n, n)

    def one_electron(self, which, charges=None):
        n = self.nbf
        out = np.zeros(n * n)
        z = np.ascontiguousarray(self.bas.charges if charges is None else charges, dtype=np.float64)
        lib().orc_one_electron(self.h, {"S": 0, "T": 1, "V": 2}[which], _p(z), _p(out))
        return out.reshape(n, n)


    def grad2e(self, dt, ds=None, coulscale=1.0, hfscale=1.0, cutoff=1e-10, nthreads=None, stride=1, offset=0):
        """Two-electron HF gradient (natom, 3) of OpenQP's grd2 for the full AO
        total density dt (and spin density ds for UHF/ROHF); stride > 1: only
        the bra shell pairs with index % stride == offset (timing samples)."""
        n = self.nbf
        dt = np.ascontiguousarray(dt, dtype=np.float64).reshape(n, n)
        dsp = None if ds is None else np.ascontiguousarray(ds, dtype=np.float64).reshape(n, n)
        de = np.zeros(3 * self.bas.natom)
        nt = nthreads or os.cpu_count()
        nq = lib().orc_grad2e(self.h, _p(dt), None if dsp is None else _p(dsp), 4.0 * coulscale, hfscale, cutoff,
                              nt, int(stride), int(offset), _p(de))
        self.last_grad2e_quartets = int(nq)
        return de.reshape(-1, 3)

    def grad2e_cam(self, dt, ds, alpha, beta, mu, cutoff=1e-10, nthreads=None):
        """CAM two-electron gradient (natom, 3) of grd2_driver: regular pass with
        hfscale alpha, erf(mu r)/r pass with hfscale beta and no Coulomb."""
        n = self.nbf
        dt = np.ascontiguousarray(dt, dtype=np.float64).reshape(n, n)
        dsp = None if ds is None else np.ascontiguousarray(ds, dtype=np.float64).reshape(n, n)
        de = np.zeros(3 * self.bas.natom)
        lib().orc_grad2e_cam(self.h, _p(dt), None if dsp is None else _p(dsp), alpha, beta, mu, cutoff,
                             nthreads or os.cpu_count(), _p(de))
        return de.reshape(-1, 3)

    def grad2e_mrsf(self, d, p, spc, hfscale, hfscale2, coulscale=1.0, spcscale=(1.0, 1.0, 1.0), mrst=1,
                    cutoff=1e-10, nthreads=None, stride=1, offset=0, cam=None):
        """MRSF two-electron gradient (natom, 3) of grd2 with the two-particle
        density of grd2_mrsf_compute_data_t: d, p (2, nbf, nbf) raw alpha / beta
        SCF and relaxed difference densities, spc (7, nbf, nbf) the response
        densities (bo2v, bo1v, bco1, bco2, o21v, co12, ball), natural indexing."""
        n = self.nbf
        fd = np.ascontiguousarray(np.asarray(d, dtype=np.float64).transpose(0, 2, 1))
        fp = np.ascontiguousarray(np.asarray(p, dtype=np.float64).transpose(0, 2, 1))
        fs = np.ascontiguousarray(np.asarray(spc, dtype=np.float64).transpose(2, 1, 0))   # Fortran (7, n, n)
        sc = np.asarray(spcscale, dtype=np.float64)
        de = np.zeros(3 * self.bas.natom)
        nq = lib().orc_grad2e_mrsf(self.h, _p(fd), _p(fp), _p(fs), hfscale, hfscale2, coulscale, _p(sc), int(mrst),
                                   cutoff, nthreads or os.cpu_count(), int(stride), int(offset), _p(de),
                                   None if cam is None else _p(np.asarray(cam, dtype=np.float64)))
        self.last_grad2e_quartets = int(nq)
        return de.reshape(-1, 3)

    def grad1e(self, d, w, charges=None):
        """One-electron gradient (natom, 3): sum D dH/dR - W dS/dR."""
        n = self.nbf
        d = np.ascontiguousarray(d, dtype=np.float64).reshape(n, n)
        w = np.ascontiguousarray(w, dtype=np.float64).reshape(n, n)
        z = np.ascontiguousarray(self.bas.charges if charges is None else charges, dtype=np.float64)
        de = np.zeros(3 * self.bas.natom)
        lib().orc_grad1e(self.h, _p(d), _p(w), _p(z), _p(de))
        return de.reshape(-1, 3)


def nuclear_repulsion_gradient(bas):
    g = np.zeros((bas.natom, 3))
    for i in range(bas.natom):
        for j in range(bas.natom):
            if i != j:
                r = bas.xyz[i] - bas.xyz[j]
                g[i] -= bas.charges[i] * bas.charges[j] * r / np.linalg.norm(r) ** 3
    return g


def rys(n, X):
    x = np.zeros(n)
    w = np.zeros(n)
    lib().orc_rys(n, float(X), _p(x), _p(w))
    return x, w


def boys(m, T):
    F = np.zeros(m + 1)
    lib().orc_boys(m, float(T), _p(F))
    return F
