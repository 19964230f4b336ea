"""Minimal direct SCF driver around the two-electron Fock build.

The loop follows OpenQP's ``scf_driver`` (``source/scf.F90:46-1364``) in the
parts that touch the Fock build: every iteration forms the packed two-electron
part G(D) through a caller-supplied builder (the GPU C-ABI in production, the
oracle in the tests), optionally incrementally -- F_n = F_{n-1} + G(D_n - D_{n-1})
with a full rebuild every ``refresh`` iterations or once the DIIS error drops
below ``refresh_err`` (``source/scf.F90:758-773``, ``source/scf_addons.F90:2036-2043``)
-- adds the core Hamiltonian and evaluates E = 1/2 tr D (F + H) + E_nuc
(``source/scf_addons.F90:2049-2065``).  Convergence acceleration is plain
Pulay DIIS on the commutator FDS - SDF (OpenQP's convergers in
``source/scf_converger.F90`` are out of scope).

RHF, UHF and ROHF are supported.  ROHF uses the effective Fock matrix of the
closed/open/virtual partition (closed-open block from F_beta, open-virtual
block from F_alpha, everything else from (F_alpha + F_beta)/2).
"""
import numpy as np

from .basis import pack, unpack


class DIIS:
    def __init__(self, nvec=8):
        self.nvec = nvec
        self.F, self.E = [], []

    def push(self, F, err):
        self.F.append(F)
        self.E.append(err)
        if len(self.F) > self.nvec:
            self.F.pop(0)
            self.E.pop(0)

    def extrapolate(self):
        n = len(self.F)
        if n < 2:
            return self.F[-1]
        B = -np.ones((n + 1, n + 1))
        B[n, n] = 0
        for i in range(n):
            for j in range(n):
                B[i, j] = sum(np.vdot(a, b) for a, b in zip(self.E[i], self.E[j]))
        rhs = np.zeros(n + 1)
        rhs[n] = -1
        try:
            c = np.linalg.solve(B, rhs)[:n]
        except np.linalg.LinAlgError:
            return self.F[-1]
        return [sum(c[i] * self.F[i][s] for i in range(n)) for s in range(len(self.F[-1]))]


def run_scf(nbf, S, H, enuc, nalpha, nbeta, fock2e, kind="rhf", conv=1e-9, maxit=100, incremental=False,
            refresh=10, refresh_err=1e-4, dconv=1e-7, guess=None, log=None):
    """Returns dict(energy, iterations, D (packed, per spin), F (packed 2e part),
    builds, C (alpha, beta orbitals of D), Fock (full AO Fock matrices of D))."""
    w, U = np.linalg.eigh(S)
    X = U / np.sqrt(w)
    Hp = pack(H)
    nspin = 1 if kind == "rhf" else 2

    def diag(F):
        e, Cp = np.linalg.eigh(X.T @ F @ X)
        return e, X @ Cp

    if guess is None:
        _, C = diag(H)
        Ca = Cb = C
    else:
        Ca, Cb = guess

    def dens(Ca, Cb):
        if kind == "rhf":
            return [2.0 * Ca[:, :nalpha] @ Ca[:, :nalpha].T]
        return [Ca[:, :nalpha] @ Ca[:, :nalpha].T, Cb[:, :nbeta] @ Cb[:, :nbeta].T]

    Dm = dens(Ca, Cb)
    Cc = (Ca, Cb)   # orbitals of the current density
    diis = DIIS()
    e_old = 0.0
    Gp_prev = None
    Dp_prev = None
    builds = 0
    since_full = 0
    err_norm = 1.0
    for it in range(1, maxit + 1):
        Dp = np.stack([pack(d) for d in Dm])
        full = (not incremental) or Gp_prev is None or since_full >= refresh or err_norm < refresh_err
        if full:
            Gp = fock2e(Dp)
            since_full = 0
        else:
            Gp = Gp_prev + fock2e(Dp - Dp_prev)
            since_full += 1
        builds += 1
        Gp_prev, Dp_prev = Gp, Dp
        Fs = [unpack(Hp + Gp[s], nbf) for s in range(nspin)]
        if kind == "rhf":
            E = 0.5 * np.sum(Dm[0] * (H + Fs[0])) + enuc
        else:
            E = 0.5 * sum(np.sum(Dm[s] * (H + Fs[s])) for s in range(2)) + enuc
        if kind == "rohf":
            Fa, Fb = Fs
            Fc = 0.5 * (Fa + Fb)
            C = Ca
            Fm = [C.T @ M @ C for M in (Fa, Fb, Fc)]
            R = Fm[2].copy()
            nc, no = nbeta, nalpha
            R[:nc, nc:no] = Fm[1][:nc, nc:no]
            R[nc:no, :nc] = Fm[1][nc:no, :nc]
            R[nc:no, no:] = Fm[0][nc:no, no:]
            R[no:, nc:no] = Fm[0][no:, nc:no]
            SC = S @ C
            Feff = SC @ R @ SC.T
            Dtot = Dm[0] + Dm[1]
            err = [Feff @ (0.5 * Dtot) @ S - S @ (0.5 * Dtot) @ Feff]
            diis.push([Feff], err)
            (Fx,) = diis.extrapolate()
            _, Ca = diag(Fx)
            Cb = Ca
        else:
            errs = [Fs[s] @ Dm[s] @ S - S @ Dm[s] @ Fs[s] for s in range(nspin)]
            diis.push(Fs, errs)
            Fx = diis.extrapolate()
            _, Ca = diag(Fx[0])
            Cb = Ca if kind == "rhf" else diag(Fx[1])[1]
            err = errs
        err_norm = max(np.abs(e).max() for e in err)
        Dm_new = dens(Ca, Cb)
        dD = max(np.abs(a - b).max() for a, b in zip(Dm_new, Dm))
        if log:
            log("iter %3d  E = %.12f  dE = %.3e  err = %.3e  %s" % (it, E, E - e_old, err_norm,
                                                                   "full" if full else "inc"))
        if abs(E - e_old) < conv and err_norm < 1e-6 and dD < dconv:
            return dict(energy=E, iterations=it, D=Dp, F=Gp, builds=builds, converged=True, C=Cc, Fock=Fs)
        e_old = E
        Dm = Dm_new
        Cc = (Ca, Cb)
    return dict(energy=E, iterations=maxit, D=Dp, F=Gp, builds=builds, converged=False, C=Cc, Fock=Fs)


def energy_weighted_density(res, nalpha, nbeta, kind="rhf"):
    """W of the gradient's overlap term, -sum W dS/dR, for the orbitals of a
    converged run: W = C lam C^T with the orbital Lagrangian
    lam_pq = (C^T Fa C)_pq n^a_q + (C^T Fb C)_pq n^b_q (symmetrised).  For
    RHF / UHF canonical orbitals this is sum_occ eps c c^T per spin."""
    Ca, Cb = res["C"]
    Fs = res["Fock"]
    if kind == "rhf":
        Fa = Fb = Fs[0]
    else:
        Fa, Fb = Fs
    n = Ca.shape[1]
    na = np.zeros(n)
    na[:nalpha] = 1.0
    nb_ = np.zeros(n)
    nb_[:nbeta] = 1.0
    if kind == "uhf":
        Wa = (Ca * na) @ (Ca.T @ Fa @ Ca) @ (Ca * na).T
        Wb = (Cb * nb_) @ (Cb.T @ Fb @ Cb) @ (Cb * nb_).T
        return Wa + Wb
    C = Ca
    lam = (C.T @ Fa @ C) * na[None, :] + (C.T @ Fb @ C) * nb_[None, :]
    lam = 0.5 * (lam + lam.T)
    return C @ lam @ C.T
