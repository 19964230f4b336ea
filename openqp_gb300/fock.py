"""Python front end of the GB300 Fock build.

``FockBuilder`` mirrors OpenQP's operator for this path,
``fock_jk(basis, d, f, infos, scale_exch, nschwz, f_old, scale_coul)``
(``source/scf_addons.F90:1063-1214``): the same packed-triangle density in,
the same ready-to-use packed two-electron Fock matrix out (``nfocks = 1``:
RHF, F = sc J - se/2 K; ``nfocks = 2``: UHF/ROHF, F_s = sc J[Da+Db] - se K[D_s]).
Every call goes through the C ABI of ``libopenqp_gb300.so``; there is no CPU
path.  ``routec_*`` wrap the reference-facing seam itself.
"""
import ctypes

import numpy as np

from ._lib import FockError, lib, ptr, _i

NCLASS = 55


def class_labels():
    names = "spdf"
    out = []
    for c in range(NCLASS):
        l4 = (ctypes.c_int * 4)()
        lib().oqpg_class_l(c, l4)
        out.append("(%s%s|%s%s)" % tuple(names[v] for v in l4))
    return out


def _basis_arrays(bas):
    return [np.ascontiguousarray(bas.am, dtype=np.int32), np.ascontiguousarray(bas.ncontr, dtype=np.int32),
            np.ascontiguousarray(bas.origin, dtype=np.int32), np.ascontiguousarray(bas.ex, dtype=np.float64),
            np.ascontiguousarray(bas.cc, dtype=np.float64), np.ascontiguousarray(bas.harmonic, dtype=np.int32),
            np.ascontiguousarray(bas.xyz.reshape(-1), dtype=np.float64)]


def _batch_arrays(bases):
    """Per-molecule counts and the concatenated basis arrays of a batch."""
    parts = [_basis_arrays(b) for b in bases]
    cat = [np.ascontiguousarray(np.concatenate([p[k] for p in parts])) for k in range(7)]
    nshell = np.array([len(b.am) for b in bases], dtype=np.int32)
    natom = np.array([b.natom for b in bases], dtype=np.int32)
    return nshell, natom, cat


class FockBuilder:
    """Direct J/K builder for one basis and geometry (one device context)."""

    def __init__(self, bas, cutoff=1e-10):
        self.bas = bas
        self.cutoff = cutoff
        k = _basis_arrays(bas)
        self._keep = k
        h = ctypes.c_void_p()
        rc = lib().oqpg_create(ctypes.byref(h), len(bas.am), ptr(k[0], _i), ptr(k[1], _i), ptr(k[2], _i), ptr(k[3]),
                               ptr(k[4]), ptr(k[5], _i), int(bas.natom), ptr(k[6]), float(cutoff))
        if rc != 0:
            raise FockError(rc, "oqpg_create")
        self.h = h
        self._layout()

    def _layout(self):
        n = lib().oqpg_batch_info(self.h, None, None)
        nbf = (ctypes.c_int * n)()
        tri0 = (ctypes.c_longlong * n)()
        lib().oqpg_batch_info(self.h, nbf, tri0)
        self.nmol = n
        self.nbf_mol = [int(v) for v in nbf]
        self.tri0 = [int(v) for v in tri0]
        self.nbf = lib().oqpg_nbf(self.h)
        self.ntri = sum(v * (v + 1) // 2 for v in self.nbf_mol)

    def close(self):
        if getattr(self, "h", None):
            lib().oqpg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def fock_jk(self, d, scale_exch=1.0, scale_coul=1.0):
        """d: (ntri,) or (nfocks, ntri) packed densities (host) -> packed F, same shape as 2-D."""
        d = np.ascontiguousarray(np.atleast_2d(d), dtype=np.float64)
        if d.shape[1] != self.ntri:
            raise ValueError("density has %d packed elements, basis needs %d" % (d.shape[1], self.ntri))
        f = np.empty_like(d)
        rc = lib().oqpg_fock_jk(self.h, ptr(d), ptr(f), d.shape[0], float(scale_exch), float(scale_coul))
        if rc != 0:
            raise FockError(rc, "oqpg_fock_jk")
        return f

    def fock_jk_cam(self, d, alpha, beta, mu, alpha_coul=1.0, beta_coul=0.0):
        """CAM build (OpenQP's int2_run_cam, int2.F90:538-584) of packed
        densities: sc = alpha_coul, se = alpha over 1/r plus sc = beta_coul,
        se = beta over erf(mu r)/r; same packing and scaling as fock_jk."""
        d = np.ascontiguousarray(np.atleast_2d(d), dtype=np.float64)
        if d.shape[1] != self.ntri:
            raise ValueError("density has %d packed elements, basis needs %d" % (d.shape[1], self.ntri))
        f = np.empty_like(d)
        rc = lib().oqpg_fock_jk_cam(self.h, ptr(d), ptr(f), d.shape[0], ptr(cam_array(alpha, beta, mu, alpha_coul,
                                                                                      beta_coul)))
        if rc != 0:
            raise FockError(rc, "oqpg_fock_jk_cam")
        return f

    def fock_jk_device(self, d, scale_exch=1.0, scale_coul=1.0, out=None, stream=None):
        """d: torch CUDA tensor (nfocks, ntri) float64 -> torch tensor, no host copies."""
        import torch
        if not (d.is_cuda and d.dtype == torch.float64 and d.is_contiguous()):
            raise ValueError("d must be a contiguous float64 CUDA tensor")
        d2 = d if d.dim() == 2 else d.unsqueeze(0)
        if out is None:
            out = torch.empty_like(d2)
        st = stream if stream is not None else torch.cuda.current_stream(d.device)
        rc = lib().oqpg_fock_jk_device(self.h, ctypes.c_void_p(d2.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                       d2.shape[0], float(scale_exch), float(scale_coul),
                                       ctypes.c_void_p(st.cuda_stream))
        if rc != 0:
            raise FockError(rc, "oqpg_fock_jk_device")
        return out

    def fock_jk_graph(self, d, scale_exch=1.0, scale_coul=1.0, out=None, stream=None):
        """As fock_jk_device, replayed from the context's captured CUDA graph
        (captured on the first call; rebuilt and recaptured when needed)."""
        import torch
        if not (d.is_cuda and d.dtype == torch.float64 and d.is_contiguous()):
            raise ValueError("d must be a contiguous float64 CUDA tensor")
        d2 = d if d.dim() == 2 else d.unsqueeze(0)
        if out is None:
            out = torch.empty_like(d2)
        st = stream if stream is not None else torch.cuda.current_stream(d.device)
        rc = lib().oqpg_fock_jk_graph(self.h, ctypes.c_void_p(d2.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                      d2.shape[0], float(scale_exch), float(scale_coul),
                                      ctypes.c_void_p(st.cuda_stream))
        if rc != 0:
            raise FockError(rc, "oqpg_fock_jk_graph")
        return out

    # ---- response-type builds (general square densities) ---------------------
    def fock_td(self, x, apb=True, amb=False, tda=False, tda_coulomb=False, scale_exch=1.0, scale_coul=1.0,
                cam=None):
        """TDHF-type build of OpenQP's int2_td_data_t (tdhf_lib.F90:140-224).

        x: (nvec, nbf, nbf) or (nbf, nbf) general square densities (host,
        natural indexing x[v][r, c]).  Returns (apb, amb), each (nvec, nbf, nbf):
          A+B: 4 sc J[X] - 2 se K[(X + X^T)/2]        (apb=True)
          A-B: -2 se K[(X - X^T)/2]                    (amb=True)
          TDA, into amb: 2 sc J[X] (tda_coulomb) - se K[X]
        with J[X]_ij = sum (ij|kl) X_kl and K[X]_ik = sum (ij|kl) X_jl.
        cam = (alpha, beta, mu[, alpha_coul, beta_coul]): the two-pass CAM build
        (scale_exch / scale_coul are then replaced by the pass scales)."""
        x = np.asarray(x, dtype=np.float64)
        squeeze = x.ndim == 2
        x3 = x[None] if squeeze else x
        nv, n = x3.shape[0], self.nbf
        if x3.shape[1:] != (n, n):
            raise ValueError("densities must be (nvec, %d, %d)" % (n, n))
        fx = np.ascontiguousarray(x3.transpose(0, 2, 1))  # Fortran (nbf, nbf, nvec)
        pa, ma = np.empty_like(fx), np.empty_like(fx)
        fl = td_flags(apb, amb, tda, tda_coulomb)
        if cam is not None:
            rc = lib().oqpg_fock_td_cam(self.h, ptr(fx), ptr(pa), ptr(ma), nv, fl, ptr(cam_array(*cam)))
        else:
            rc = lib().oqpg_fock_td(self.h, ptr(fx), ptr(pa), ptr(ma), nv, fl, float(scale_exch), float(scale_coul))
        if rc != 0:
            raise FockError(rc, "oqpg_fock_td")
        pa, ma = pa.transpose(0, 2, 1), ma.transpose(0, 2, 1)
        return (pa[0], ma[0]) if squeeze else (pa, ma)

    def fock_td_device(self, x, apb=True, amb=False, tda=False, tda_coulomb=False, scale_exch=1.0,
                       scale_coul=1.0, stream=None):
        """fock_td on torch CUDA tensors: x (nvec, nbf, nbf) float64 -> (apb, amb)."""
        import torch
        if not (x.is_cuda and x.dtype == torch.float64):
            raise ValueError("x must be a float64 CUDA tensor")
        x3 = x if x.dim() == 3 else x.unsqueeze(0)
        fx = x3.transpose(1, 2).contiguous()
        pa, ma = torch.empty_like(fx), torch.empty_like(fx)
        st = stream if stream is not None else torch.cuda.current_stream(x.device)
        rc = lib().oqpg_fock_td_device(self.h, ctypes.c_void_p(fx.data_ptr()), ctypes.c_void_p(pa.data_ptr()),
                                       ctypes.c_void_p(ma.data_ptr()), x3.shape[0],
                                       td_flags(apb, amb, tda, tda_coulomb), float(scale_exch), float(scale_coul),
                                       ctypes.c_void_p(st.cuda_stream))
        if rc != 0:
            raise FockError(rc, "oqpg_fock_td_device")
        pa, ma = pa.transpose(1, 2), ma.transpose(1, 2)
        return (pa[0], ma[0]) if x.dim() == 2 else (pa, ma)

    def fock_tdgrd(self, x, apb=True, amb=False, scale_exch=1.0, scale_coul=1.0, cam=None):
        """Spin-adapted response build of OpenQP's int2_tdgrd_data_t
        (tdhf_lib.F90:228-295), the operator of the SF / MRSF Z-vector solvers.

        x: (2, nbf, nbf) alpha / beta densities (host, natural indexing).
        Returns (apb, amb), each (2, nbf, nbf):
          A+B, spin s: 2 sc J[X1 + X2] - 2 se K[(Xs + Xs^T)/2]      (apb=True)
          A-B: spin 1 -2 se K[(X1 - X1^T)/2], spin 2 zero           (amb=True)
        cam = (alpha, beta, mu[, alpha_coul, beta_coul]): the two-pass CAM build."""
        x = np.asarray(x, dtype=np.float64)
        n = self.nbf
        if x.shape != (2, n, n):
            raise ValueError("densities must be (2, %d, %d)" % (n, n))
        fx = np.ascontiguousarray(x.transpose(0, 2, 1))
        pa, ma = np.empty_like(fx), np.empty_like(fx)
        fl = td_flags(apb, amb)
        c = cam_array(*cam) if cam is not None else None
        rc = lib().oqpg_fock_tdgrd(self.h, ptr(fx), ptr(pa), ptr(ma), fl, float(scale_exch), float(scale_coul),
                                   ptr(c) if c is not None else None)
        if rc != 0:
            raise FockError(rc, "oqpg_fock_tdgrd")
        return pa.transpose(0, 2, 1), ma.transpose(0, 2, 1)

    def fock_rpagrd(self, xpy=None, xmy=None, t=None, nspin=1, scale_exch=1.0, scale_coul=1.0, cam=None):
        """H+ / H- build of OpenQP's int2_rpagrd_data_t (tdhf_lib.F90:1068-1322),
        used by the TDHF / TDDFT gradient.

        xpy, xmy, t: (nvec, ld, nbf, nbf) host arrays (ld >= nspin) or None.
        Returns (hpp, hpt, hmm), each (nvec, nspin, nbf, nbf) or None:
          nspin 1: H+[V] = 4 sc J[V] - 2 se K[V]
          nspin 2: H+[V]_s = 2 sc J[V1 + V2] - 2 se K[V_s]
          H-[V]: spin 1 -2 se K[(V1 - V1^T)/2], other spin zero
        (H+ of the symmetric part of V, the operand every reference caller
        passes)."""
        n = self.nbf

        def fort(x):
            if x is None:
                return None, 1, 0
            x = np.asarray(x, dtype=np.float64)
            if x.ndim != 4 or x.shape[2:] != (n, n) or x.shape[1] < nspin:
                raise ValueError("operands must be (nvec, ld >= nspin, %d, %d)" % (n, n))
            return np.ascontiguousarray(x.transpose(0, 1, 3, 2)), x.shape[1], x.shape[0]

        (fp, ldp, np_), (fm, ldm, nm), (ft, ldt, nt) = fort(xpy), fort(xmy), fort(t)
        outs = [np.empty((k, nspin, n, n)) if k else None for k in (np_, nt, nm)]
        vp = lambda a: a.ctypes.data if a is not None else None
        c = cam_array(*cam) if cam is not None else None
        rc = lib().oqpg_fock_rpagrd(self.h, vp(fp), ldp, np_, vp(fm), ldm, nm, vp(ft), ldt, nt, int(nspin),
                                    vp(outs[0]), vp(outs[1]), vp(outs[2]), float(scale_exch), float(scale_coul),
                                    ptr(c) if c is not None else None)
        if rc != 0:
            raise FockError(rc, "oqpg_fock_rpagrd")
        return tuple(o.transpose(0, 1, 3, 2) if o is not None else None for o in outs)

    def fock_mrsf(self, x, scale_exch=1.0, scale_coul=1.0, cam=None):
        """MRSF (nmat 7) / UMRSF (nmat 11) sigma-vector build of OpenQP's
        int2_mrsf_data_t / int2_umrsf_data_t, first pass (tdhf_mrsf_lib.F90:218-426).

        x: (nvec, nmat, nbf, nbf) host, natural indexing x[v, m][r, c].
        Returns f of the same shape:
          MRSF:  m < 4: sc J[X] - se K[X];  m >= 4: -se K[X]
          UMRSF: m < 8: sc J[X] - se K[X];  m = 8, 9: -se K[X^T];  m = 10: -se K[X].
        cam = (alpha, beta, mu[, alpha_coul, beta_coul]): pass 1 with (alpha,
        alpha_coul), pass 2 over erf(mu r)/r adds -beta K[X] to the last component."""
        x = np.asarray(x, dtype=np.float64)
        nv, nm, n = x.shape[0], x.shape[1], self.nbf
        if x.shape[2:] != (n, n) or nm not in (7, 11):
            raise ValueError("densities must be (nvec, 7 or 11, %d, %d)" % (n, n))
        fx = np.ascontiguousarray(x.transpose(3, 2, 1, 0))  # Fortran (nvec, nmat, nbf, nbf)
        out = np.empty_like(fx)
        if cam is not None:
            rc = lib().oqpg_fock_mrsf_cam(self.h, ptr(fx), ptr(out), nv, nm, ptr(cam_array(*cam)))
        else:
            rc = lib().oqpg_fock_mrsf(self.h, ptr(fx), ptr(out), nv, nm, float(scale_exch), float(scale_coul))
        if rc != 0:
            raise FockError(rc, "oqpg_fock_mrsf")
        return out.transpose(3, 2, 1, 0)

    def graph_info(self):
        c, r, k = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        lib().oqpg_graph_info(self.h, ctypes.byref(c), ctypes.byref(r), ctypes.byref(k))
        return dict(captures=c.value, replays=r.value, kernels=k.value)

    def set_tuning(self, split_log2=None, chunk=None, ctas_per_sm=None):
        arrs = [None if v is None else np.ascontiguousarray(v, dtype=np.int32) for v in (split_log2, chunk, ctas_per_sm)]
        for a in arrs:
            if a is not None and a.shape != (NCLASS,):
                raise ValueError("tuning arrays have one entry per class (%d)" % NCLASS)
        rc = lib().oqpg_set_tuning(self.h, *[None if a is None else ptr(a, _i) for a in arrs])
        if rc != 0:
            raise FockError(rc, "oqpg_set_tuning")

    def get_tuning(self):
        arrs = [np.zeros(NCLASS, dtype=np.int32) for _ in range(3)]
        lib().oqpg_get_tuning(self.h, *[ptr(a, _i) for a in arrs])
        return dict(split_log2=arrs[0].tolist(), chunk=arrs[1].tolist(), ctas_per_sm=arrs[2].tolist())

    def set_kernel_family(self, family):
        """Per class: 0 by list size (default), 1 thread per quartet, 2 warp
        per quartet (classes with both kernels; ignored elsewhere)."""
        a = np.ascontiguousarray(family, dtype=np.int32)
        if a.shape != (NCLASS,):
            raise ValueError("one entry per class (%d)" % NCLASS)
        rc = lib().oqpg_set_kernel_family(self.h, ptr(a, _i))
        if rc != 0:
            raise FockError(rc, "oqpg_set_kernel_family")

    def get_kernel_family(self):
        """(family per class, available families per class: 1 thread, 2 warp, 3 both)"""
        f, av = np.zeros(NCLASS, dtype=np.int32), np.zeros(NCLASS, dtype=np.int32)
        lib().oqpg_get_kernel_family(self.h, ptr(f, _i), ptr(av, _i))
        return f.tolist(), av.tolist()

    def set_shell_families(self, on):
        """Share the primitive integrals of two s shells on one atom whose
        exponents are equal or nested (cc-pVXZ's generally contracted shells)
        in the s-rich classes ((ss|ss) .. (ss|pd), (sp|sp), (sp|sd), (sp|pp))
        of SCF builds in every precision mode (default on); off: every shell
        quartet on its own."""
        rc = lib().oqpg_set_shell_families(self.h, 1 if on else 0)
        if rc != 0:
            raise FockError(rc, "oqpg_set_shell_families")

    def shell_families_info(self):
        """(on, family pairs with more than one member shell pair)"""
        on, n = ctypes.c_int(0), ctypes.c_int(0)
        lib().oqpg_shell_families_info(self.h, ctypes.byref(on), ctypes.byref(n))
        return bool(on.value), n.value

    def set_precision(self, mode, threshold=1e-6):
        """mode "fp64": plain path; mode "mixed": quartets whose screening value
        (Schwarz bound x shell density) is below threshold run in FP32 with their
        Rys roots/weights in FP64; "mixed-fast": the same with FP32 roots;
        "df": the thread-per-quartet classes in double-float arithmetic
        (FP32 pairs, ~1e-13 relative) with FP64 digestion, no split;
        "mixed-df": FP32 below the threshold (as mixed-fast), double-float above.  The
        gradient (grad2) splits the same way on the bound of its two-particle
        density."""
        m = {"fp64": 0, "mixed": 1, "mixed-fast": 2, "df": 3, "mixed-df": 4}[mode]
        rc = lib().oqpg_set_precision(self.h, m, float(threshold))
        if rc != 0:
            raise FockError(rc, "oqpg_set_precision")

    def set_cutoff(self, cutoff):
        """Two-electron cutoff of the following builds, as OpenQP's
        int2_compute_t_set_cutoff (the progressive-screening SCF changes it per
        build)."""
        rc = lib().oqpg_set_cutoff(self.h, float(cutoff))
        if rc != 0:
            raise FockError(rc, "oqpg_set_cutoff")
        self.cutoff = float(cutoff)

    def set_symmetry(self, sym=None):
        """Petite list of the following SCF builds: sym = (nops, shell_map,
        ao_target, ao_sign) as openqp_gb300.symmetry.abelian_symmetry returns
        (0-based); None or nops <= 1 switches it off.  The builds still return
        the complete Fock matrix."""
        if sym is None or int(sym[0]) <= 1:
            rc = lib().oqpg_set_symmetry(self.h, 0, None, None, None)
        else:
            nops, sm, at, sg = sym
            self._sym = (np.ascontiguousarray(sm, dtype=np.int32), np.ascontiguousarray(at, dtype=np.int32),
                         np.ascontiguousarray(sg, dtype=np.float64))
            rc = lib().oqpg_set_symmetry(self.h, int(nops), ptr(self._sym[0], _i), ptr(self._sym[1], _i),
                                         ptr(self._sym[2]))
        if rc != 0:
            raise FockError(rc, "oqpg_set_symmetry")

    def symmetry_info(self):
        """(group order, whether the last direct build used the reduction)"""
        n, r = ctypes.c_int(0), ctypes.c_int(0)
        rc = lib().oqpg_symmetry_info(self.h, ctypes.byref(n), ctypes.byref(r))
        if rc != 0:
            raise FockError(rc, "oqpg_symmetry_info")
        return n.value, bool(r.value)

    def get_cutoff(self):
        """The cutoff the library applies to the next build."""
        return lib().oqpg_get_cutoff(self.h)

    def grad2(self, d, hfscale=1.0, coulscale=1.0):
        """Two-electron gradient (natom, 3) for packed densities d ((ntri,) or
        (nfocks, ntri): total RHF density, or alpha and beta)."""
        d = np.ascontiguousarray(np.atleast_2d(d), dtype=np.float64)
        de = np.zeros(3 * self.bas.natom)
        rc = lib().oqpg_grad2(self.h, ptr(d), d.shape[0], float(hfscale), float(coulscale), ptr(de))
        if rc != 0:
            raise FockError(rc, "oqpg_grad2")
        return de.reshape(-1, 3)

    def grad2_bilinear(self, x, y, xs=None, ys=None, cj=4.0, ckt=1.0, cks=1.0):
        """Gradient (natom, 3) of the symmetric bilinear two-particle density of
        full AO matrices (see oqpg_grad2_bilinear)."""
        n = self.nbf
        mats = [None if m is None else np.ascontiguousarray(m, dtype=np.float64).reshape(n, n) for m in (x, y, xs, ys)]
        de = np.zeros(3 * self.bas.natom)
        rc = lib().oqpg_grad2_bilinear(self.h, *[None if m is None else ptr(m) for m in mats], float(cj), float(ckt),
                                       float(cks), ptr(de))
        if rc != 0:
            raise FockError(rc, "oqpg_grad2_bilinear")
        return de.reshape(-1, 3)

    def grad2_cam(self, d, alpha, beta, mu):
        """CAM two-electron gradient (natom, 3) of grd2_driver's CAM branch:
        1/r pass with hfscale alpha, erf(mu r)/r pass with hfscale beta and no
        Coulomb.  d as in grad2."""
        d = np.ascontiguousarray(np.atleast_2d(d), dtype=np.float64)
        de = np.zeros(3 * self.bas.natom)
        rc = lib().oqpg_grad2_cam(self.h, ptr(d), d.shape[0], float(alpha), float(beta), float(mu), ptr(de))
        if rc != 0:
            raise FockError(rc, "oqpg_grad2_cam")
        return de.reshape(-1, 3)

    def grad2_mrsf(self, d, p, spc, hfscale, hfscale2, coulscale=1.0, spcscale=(1.0, 1.0, 1.0), mrst=1, cam=None):
        """MRSF two-electron gradient (natom, 3) of OpenQP's
        grd2_mrsf_compute_data_t (modules/tdhf_mrsf_gradient.F90:341-601).
        d, p: (2, nbf, nbf) raw alpha / beta SCF and relaxed difference
        densities; spc: (7, nbf, nbf) response densities (bo2v, bo1v, bco1,
        bco2, o21v, co12, ball), natural indexing; spcscale = (spc_coco,
        spc_ovov, spc_coov)."""
        n = self.nbf
        fd, fp = (np.ascontiguousarray(np.asarray(m, dtype=np.float64).reshape(2, n, n).transpose(0, 2, 1))
                  for m in (d, p))
        fs = np.ascontiguousarray(np.asarray(spc, dtype=np.float64).reshape(7, n, n).transpose(2, 1, 0))
        sc = np.asarray(spcscale, dtype=np.float64)
        de = np.zeros(3 * self.bas.natom)
        if cam is not None:   # (reference alpha, reference beta, response alpha, response beta, mu)
            c5 = np.asarray(cam, dtype=np.float64)
            rc = lib().oqpg_grad2_mrsf_cam(self.h, ptr(fd), ptr(fp), ptr(fs), ptr(c5), ptr(sc), int(mrst), ptr(de))
        else:
            rc = lib().oqpg_grad2_mrsf(self.h, ptr(fd), ptr(fp), ptr(fs), float(hfscale), float(hfscale2),
                                       float(coulscale), ptr(sc), int(mrst), ptr(de))
        if rc != 0:
            raise FockError(rc, "oqpg_grad2_mrsf")
        return de.reshape(-1, 3)

    def grad2_sf(self, d, p, v, hfscale, hfscale2, coulscale=1.0):
        """SF-TDDFT two-electron gradient (natom, 3) of OpenQP's
        grd2_sf_compute_data_t (modules/tdhf_sf_gradient.F90:277-502): d, p
        (2, nbf, nbf) raw alpha / beta densities, v (nbf, nbf) the transition
        density, natural indexing."""
        n = self.nbf
        fd, fp = (np.ascontiguousarray(np.asarray(m, dtype=np.float64).reshape(2, n, n).transpose(0, 2, 1))
                  for m in (d, p))
        fv = np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(n, n).T)
        de = np.zeros(3 * self.bas.natom)
        rc = lib().oqpg_grad2_sf(self.h, ptr(fd), ptr(fp), ptr(fv), float(hfscale), float(hfscale2), float(coulscale),
                                 ptr(de))
        if rc != 0:
            raise FockError(rc, "oqpg_grad2_sf")
        return de.reshape(-1, 3)

    def grad_stats(self):
        s = np.zeros(5)
        lib().oqpg_grad_stats(self.h, ptr(s), 5)
        return dict(quartets_listed=int(s[0]), quartets=int(s[1]), prim_quartets=int(s[2]), ms=float(s[3]),
                    f32_quartets_listed=int(s[4]))

    def schwarz(self):
        ns = len(self.bas.am)
        q = np.zeros(ns * ns)
        rc = lib().oqpg_schwarz(self.h, ptr(q))
        if rc != 0:
            raise FockError(rc, "oqpg_schwarz")
        return q.reshape(ns, ns)

    def stats(self):
        s = np.zeros(10 + 4 * NCLASS)
        lib().oqpg_stats(self.h, ptr(s), len(s))
        return dict(quartets=int(s[0]), prim_quartets=int(s[1]), list_ms=s[2], eri_ms=s[3], total_ms=s[4],
                    nbf=int(s[5]), npair=int(s[6]), per_class=[int(v) for v in s[7:7 + NCLASS]],
                    prim_per_class=[int(v) for v in s[7 + NCLASS:7 + 2 * NCLASS]],
                    ms_per_class=[float(v) for v in s[7 + 2 * NCLASS:7 + 3 * NCLASS]],
                    launches=int(s[7 + 3 * NCLASS]), f32_quartets=int(s[8 + 3 * NCLASS]),
                    f32_prim_quartets=int(s[9 + 3 * NCLASS]),
                    ms_per_class_f32=[float(v) for v in s[10 + 3 * NCLASS:10 + 4 * NCLASS]])


class BatchFockBuilder(FockBuilder):
    """One context over many molecules: every build builds all of them (one
    launch per class for the whole batch).  Matrices go in and out as the
    molecules' packed blocks one after the other; pack / unpack convert from and
    to lists of per-molecule (nfocks, ntri_m) arrays."""

    def __init__(self, bases, cutoff=1e-10):
        self.bases = list(bases)
        self.cutoff = cutoff
        nshell, natom, k = _batch_arrays(self.bases)
        self._keep = (nshell, natom, k)
        h = ctypes.c_void_p()
        rc = lib().oqpg_create_batch(ctypes.byref(h), len(self.bases), ptr(nshell, _i), ptr(natom, _i),
                                     ptr(k[0], _i), ptr(k[1], _i), ptr(k[2], _i), ptr(k[3]), ptr(k[4]), ptr(k[5], _i),
                                     ptr(k[6]), float(cutoff))
        if rc != 0:
            raise FockError(rc, "oqpg_create_batch")
        self.h = h
        self._layout()

    def pack(self, ds):
        """List of per-molecule (nfocks, ntri_m) densities -> (ntotal,) vector."""
        return np.ascontiguousarray(np.concatenate([np.atleast_2d(d).reshape(-1) for d in ds]))

    def unpack(self, flat, nfocks=1):
        out = []
        for m, n in enumerate(self.nbf_mol):
            t = n * (n + 1) // 2
            o = nfocks * self.tri0[m]
            out.append(np.asarray(flat[o:o + nfocks * t]).reshape(nfocks, t))
        return out

    def fock_jk(self, ds, scale_exch=1.0, scale_coul=1.0):
        """ds: list of per-molecule densities -> list of packed Fock matrices."""
        nfocks = np.atleast_2d(ds[0]).shape[0]
        d = self.pack(ds)
        if d.size != nfocks * self.ntri:
            raise ValueError("densities do not match the batch")
        f = np.empty_like(d)
        rc = lib().oqpg_fock_jk(self.h, ptr(d), ptr(f), nfocks, float(scale_exch), float(scale_coul))
        if rc != 0:
            raise FockError(rc, "oqpg_fock_jk")
        return self.unpack(f, nfocks)


def fp64_peak_tflops(iters=20000):
    v = ctypes.c_double(0)
    rc = lib().oqpg_measure_fp64_peak(int(iters), ctypes.byref(v))
    if rc != 0:
        raise FockError(rc, "oqpg_measure_fp64_peak")
    return v.value


def class_flops(c, nprim, nquart, nk=1, pure=False, nj=1):
    """Algorithmic FP64 flops of class c: assembly 3 R N_c per primitive
    quartet (x*y, then FMA with z, per Rys root) plus digestion per
    contracted quartet, 2 FMA per element and Coulomb density plus 4 FMA per
    element and exchange density (12 flops for RHF)."""
    l4 = (ctypes.c_int * 4)()
    lib().oqpg_class_l(c, l4)
    L = list(l4)
    R = sum(L) // 2 + 1
    nc = 1
    nao = 1
    for l in L:
        nc *= (l + 1) * (l + 2) // 2
        nao *= (2 * l + 1 if (pure and l >= 2) else (l + 1) * (l + 2) // 2)
    dig = 2 * (2 * nj + 4 * nk)
    return 3.0 * R * nc * nprim + dig * nao * nquart


# ---- the reference-facing seam ------------------------------------------------

def routec_init(bas, cutoff=1e-10):
    k = _basis_arrays(bas)
    rc = lib().routec_fock_init(len(bas.am), ptr(k[0], _i), ptr(k[1], _i), ptr(k[2], _i), ptr(k[3]), ptr(k[4]),
                                ptr(k[5], _i), int(bas.natom), ptr(k[6]), float(cutoff))
    return rc


def routec_fock_jk(d, nbf, nfocks, se=1.0, sc=1.0):
    """Calls routec_fock_jk exactly as OpenQP's bridge does (all by reference).
    Returns (f, info)."""
    d = np.ascontiguousarray(d, dtype=np.float64).reshape(-1)
    f = np.zeros_like(d)
    n = ctypes.c_int(nbf)
    nf = ctypes.c_int(nfocks)
    se_ = ctypes.c_double(se)
    sc_ = ctypes.c_double(sc)
    info = ctypes.c_int(1)
    lib().routec_fock_jk(ptr(d), ptr(f), ctypes.byref(n), ctypes.byref(nf), ctypes.byref(se_), ctypes.byref(sc_),
                         ctypes.byref(info))
    return f.reshape(nfocks, -1), info.value


def routec_fock_jk_inc(dd, f_old, nbf, nfocks, se=1.0, sc=1.0):
    """Calls routec_fock_jk_inc (all by reference): F = F_old + G(dD) with
    F_old overwritten by F, as fock_jk's f_old branch.  f_old is updated in
    place (a float64 C-contiguous array).  Returns (f, info)."""
    dd = np.ascontiguousarray(dd, dtype=np.float64).reshape(-1)
    if not (isinstance(f_old, np.ndarray) and f_old.dtype == np.float64 and f_old.flags.c_contiguous
            and f_old.size == dd.size):
        raise ValueError("f_old must be a C-contiguous float64 array of the density's size")
    f = np.zeros_like(dd)
    n, nf = ctypes.c_int(nbf), ctypes.c_int(nfocks)
    se_, sc_ = ctypes.c_double(se), ctypes.c_double(sc)
    info = ctypes.c_int(1)
    lib().routec_fock_jk_inc(ptr(dd), ptr(f), ptr(f_old), ctypes.byref(n), ctypes.byref(nf), ctypes.byref(se_),
                             ctypes.byref(sc_), ctypes.byref(info))
    return f.reshape(nfocks, -1), info.value


def routec_fock_set_cutoff(cutoff):
    """Calls routec_fock_set_cutoff by reference; returns info."""
    c = ctypes.c_double(cutoff)
    info = ctypes.c_int(1)
    lib().routec_fock_set_cutoff(ctypes.byref(c), ctypes.byref(info))
    return info.value


def routec_fock_set_symmetry(nops, shell_map=None, ao_target=None, ao_sign=None):
    """Calls routec_fock_set_symmetry with OpenQP's staged layout: 1-based
    integer(8) images, shell or AO index fastest.  Takes the 0-based arrays of
    openqp_gb300.symmetry.abelian_symmetry.  Returns info."""
    n = ctypes.c_int(int(nops))
    info = ctypes.c_int(1)
    if int(nops) <= 1:
        lib().routec_fock_set_symmetry(ctypes.byref(n), None, None, None, ctypes.byref(info))
        return info.value
    sm = np.ascontiguousarray(np.asarray(shell_map).reshape(-1) + 1, dtype=np.int64)
    at = np.ascontiguousarray(np.asarray(ao_target).reshape(-1) + 1, dtype=np.int64)
    sg = np.ascontiguousarray(np.asarray(ao_sign).reshape(-1), dtype=np.float64)
    ll = ctypes.POINTER(ctypes.c_longlong)
    lib().routec_fock_set_symmetry(ctypes.byref(n), sm.ctypes.data_as(ll), at.ctypes.data_as(ll), ptr(sg),
                                   ctypes.byref(info))
    return info.value


def routec_grad2(d, xyz, nbf, natom, hfscale=1.0, coulscale=1.0, de=None):
    """Calls routec_grad2 as OpenQP's bridge does; de (natom, 3) is accumulated."""
    d = np.ascontiguousarray(d, dtype=np.float64).reshape(-1)
    x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
    de = np.zeros(3 * natom) if de is None else np.ascontiguousarray(de, dtype=np.float64).reshape(-1)
    n, na = ctypes.c_int(nbf), ctypes.c_int(natom)
    hf, cs = ctypes.c_double(hfscale), ctypes.c_double(coulscale)
    info = ctypes.c_int(1)
    lib().routec_grad2(ptr(d), ptr(x), ptr(de), ctypes.byref(n), ctypes.byref(na), ctypes.byref(hf), ctypes.byref(cs),
                       ctypes.byref(info))
    return de.reshape(-1, 3), info.value


def routec_grad2_mrsf(d, p, spc, xyz, nbf, natom, hfscale, hfscale2, coulscale=1.0, spcscale=(1.0, 1.0, 1.0), mrst=1,
                      de=None):
    """Calls routec_grad2_mrsf as OpenQP's bridge does: d, p the Fortran
    (nbf, nbf, 2) arrays and spc the Fortran (7, nbf, nbf) array as flat
    buffers; de (natom, 3) is accumulated.  Returns (de, info)."""
    bufs = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1) for a in (d, p, spc, xyz)]
    de = np.zeros(3 * natom) if de is None else np.ascontiguousarray(de, dtype=np.float64).reshape(-1)
    sc = np.asarray(spcscale, dtype=np.float64)
    n, na, ms = ctypes.c_int(nbf), ctypes.c_int(natom), ctypes.c_int(mrst)
    hf, hf2, cs = ctypes.c_double(hfscale), ctypes.c_double(hfscale2), ctypes.c_double(coulscale)
    info = ctypes.c_int(1)
    lib().routec_grad2_mrsf(*[ptr(b) for b in bufs], ptr(de), ctypes.byref(n), ctypes.byref(na), ctypes.byref(hf),
                            ctypes.byref(hf2), ctypes.byref(cs), ptr(sc), ctypes.byref(ms), ctypes.byref(info))
    return de.reshape(-1, 3), info.value


def cam_array(alpha, beta, mu, alpha_coul=1.0, beta_coul=0.0):
    """The cam[5] argument of the C ABI (int2_run_cam's parameters)."""
    if not mu > 0:
        raise ValueError("CAM needs mu > 0")
    return np.array([alpha, beta, mu, alpha_coul, beta_coul], dtype=np.float64)


def routec_fock_jk_cam(d, nbf, nfocks, alpha, beta, mu, alpha_coul=1.0, beta_coul=0.0):
    """Calls routec_fock_jk_cam with all arguments by reference. Returns (f, info)."""
    d = np.ascontiguousarray(d, dtype=np.float64).reshape(-1)
    f = np.zeros_like(d)
    n, nf = ctypes.c_int(nbf), ctypes.c_int(nfocks)
    info = ctypes.c_int(1)
    lib().routec_fock_jk_cam(ptr(d), ptr(f), ctypes.byref(n), ctypes.byref(nf),
                             ptr(cam_array(alpha, beta, mu, alpha_coul, beta_coul)), ctypes.byref(info))
    return f.reshape(nfocks, -1), info.value


def td_flags(apb=True, amb=False, tda=False, tda_coulomb=False):
    """OQPG_TD_* flags of the TD build (include/openqp_gb300.h)."""
    return (1 if apb else 0) | (2 if amb else 0) | (4 if tda else 0) | (8 if tda_coulomb else 0)


def routec_fock_td(d2, nbf, nvec, flags, se=1.0, sc=1.0):
    """Calls routec_fock_td as a Fortran caller would: d2 the Fortran-ordered
    (nbf, nbf, nvec) array as a flat buffer.  Returns (apb, amb, info), flat."""
    d2 = np.ascontiguousarray(d2, dtype=np.float64).reshape(-1)
    apb, amb = np.zeros_like(d2), np.zeros_like(d2)
    n, nv, fl = ctypes.c_int(nbf), ctypes.c_int(nvec), ctypes.c_int(flags)
    se_, sc_ = ctypes.c_double(se), ctypes.c_double(sc)
    info = ctypes.c_int(1)
    lib().routec_fock_td(ptr(d2), ptr(apb), ptr(amb), ctypes.byref(n), ctypes.byref(nv), ctypes.byref(fl),
                         ctypes.byref(se_), ctypes.byref(sc_), ctypes.byref(info))
    return apb, amb, info.value


def routec_fock_tdgrd(d2, nbf, flags, se=1.0, sc=1.0, cam=None):
    """Calls routec_fock_tdgrd with the Fortran-ordered (nbf, nbf, 2) array as a
    flat buffer.  Returns (apb, amb, info), flat."""
    d2 = np.ascontiguousarray(d2, dtype=np.float64).reshape(-1)
    apb, amb = np.zeros_like(d2), np.zeros_like(d2)
    n, fl = ctypes.c_int(nbf), ctypes.c_int(flags)
    se_, sc_ = ctypes.c_double(se), ctypes.c_double(sc)
    c = cam_array(*cam) if cam is not None else None
    info = ctypes.c_int(1)
    lib().routec_fock_tdgrd(ptr(d2), ptr(apb), ptr(amb), ctypes.byref(n), ctypes.byref(fl), ctypes.byref(se_),
                            ctypes.byref(sc_), ptr(c) if c is not None else None, ctypes.byref(info))
    return apb, amb, info.value


def routec_sig_init(mo_a, mo_b, fmo_a, fmo_b, nocca, noccb, kind):
    """Begins the MRSF sigma session as routec_sig_begin does
    (modules/routec_sig.F90): (nbf, nbf) natural-indexed host matrices, kind 1
    singlet / 3 triplet.  Returns the status (0: ready)."""
    mats = [np.asfortranarray(np.asarray(m, dtype=np.float64)) for m in (mo_a, mo_b, fmo_a, fmo_b)]
    n = ctypes.c_int(mats[0].shape[0])
    na, nb, k = ctypes.c_int(nocca), ctypes.c_int(noccb), ctypes.c_int(kind)
    flat = [np.ascontiguousarray(m.T).reshape(-1) for m in mats]   # column-major buffers
    return lib().routec_sig_init(ctypes.byref(n), *[ptr(f) for f in flat], ctypes.byref(na), ctypes.byref(nb),
                                 ctypes.byref(k))


def routec_sig_set_scale(s):
    v = ctypes.c_double(s)
    lib().routec_sig_set_scale(ctypes.byref(v))


def routec_sig_iter(bvec):
    """bvec (ntrial, nv) -> (sigma (ntrial, nv), info): the Fortran
    bvec_mo(:, ist:iend) slice as a column-major buffer."""
    b = np.asarray(bvec, dtype=np.float64)
    if b.ndim == 1:
        b = b[:, None]
    fb = np.ascontiguousarray(b.T)           # column v contiguous
    out = np.zeros_like(fb)
    nv, info = ctypes.c_int(b.shape[1]), ctypes.c_int(1)
    lib().routec_sig_iter(ptr(fb), ctypes.byref(nv), ptr(out), ctypes.byref(info))
    return out.T, info.value


def routec_sig_free():
    lib().routec_sig_free()


def routec_fock_mrsf(d3, nbf, nvec, nmat, se=1.0, sc=1.0):
    """Calls routec_fock_mrsf with the Fortran-ordered (nvec, nmat, nbf, nbf)
    array as a flat buffer.  Returns (f3, info), flat."""
    d3 = np.ascontiguousarray(d3, dtype=np.float64).reshape(-1)
    f3 = np.zeros_like(d3)
    n, nv, nm = ctypes.c_int(nbf), ctypes.c_int(nvec), ctypes.c_int(nmat)
    se_, sc_ = ctypes.c_double(se), ctypes.c_double(sc)
    info = ctypes.c_int(1)
    lib().routec_fock_mrsf(ptr(d3), ptr(f3), ctypes.byref(n), ctypes.byref(nv), ctypes.byref(nm),
                           ctypes.byref(se_), ctypes.byref(sc_), ctypes.byref(info))
    return f3, info.value


def routec_finalize():
    lib().routec_fock_finalize()
