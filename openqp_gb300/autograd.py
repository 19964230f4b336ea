"""torch.autograd.Function over the GB300 Fock build.

``FockJK.apply(d, xyz, builder, scale_exch, scale_coul)`` returns the packed
two-electron Fock matrices of ``builder.fock_jk`` for the packed densities d
((nfocks, ntri), float64).  Its backward is hand-written:

* dL/dD reapplies the same J/K build to the upstream matrix.  The build is
  linear and self-adjoint on symmetric matrices, so for the packed lower
  triangles: S = gF with its off-diagonal elements halved (the symmetric
  matrix whose packing gives back the upstream weights), then
  dL/dD = 2 G(S) off the diagonal and G(S) on it.
* dL/dR (when xyz requires grad) is the derivative-ERI contraction of the
  same pairing: with S and D unpacked, the two-particle density of the
  bilinear kernel is cj = 8 sc, ckt = cks = 2 se over (S_total, D_total) and,
  for UHF/ROHF, the spin pair (S_a - S_b, D_a - D_b).  For the energy
  E2 = 1/2 Tr D G(D) this is OpenQP's grd2 gradient.

Integrals are recomputed, never stored.  xyz is the geometry the builder was
made for (Bohr, (natom, 3)); it only carries the gradient.
"""
import torch

from .basis import unpack


def _tri_weights(nbf, device):
    """1 on the packed diagonal, 0.5 elsewhere."""
    w = torch.full((nbf * (nbf + 1) // 2,), 0.5, dtype=torch.float64, device=device)
    idx = torch.arange(nbf, device=device)
    w[idx * (idx + 1) // 2 + idx] = 1.0
    return w


class FockJK(torch.autograd.Function):
    @staticmethod
    def forward(ctx, d, xyz, builder, scale_exch=1.0, scale_coul=1.0):
        if d.dtype != torch.float64:
            raise ValueError("FockJK works in float64")
        d2 = d if d.dim() == 2 else d.unsqueeze(0)
        if xyz is not None:
            ref = torch.as_tensor(builder.bas.xyz, dtype=torch.float64)
            if float((xyz.detach().cpu().reshape(-1, 3) - ref).abs().max()) > 1e-10:
                raise ValueError("xyz differs from the geometry the builder was made for")
        if d2.is_cuda:
            f = builder.fock_jk_device(d2.contiguous(), scale_exch, scale_coul)
        else:
            f = torch.from_numpy(builder.fock_jk(d2.detach().numpy(), scale_exch, scale_coul))
        ctx.builder = builder
        ctx.se, ctx.sc = float(scale_exch), float(scale_coul)
        ctx.squeeze = d.dim() == 1
        ctx.save_for_backward(d2.detach())
        return f[0] if ctx.squeeze else f

    @staticmethod
    def backward(ctx, gf):
        (d2,) = ctx.saved_tensors
        b = ctx.builder
        g2 = gf if gf.dim() == 2 else gf.unsqueeze(0)
        w = _tri_weights(b.nbf, g2.device)
        s = (g2 * w).contiguous()
        gd = gxyz = None
        if ctx.needs_input_grad[0]:
            if s.is_cuda:
                gs = b.fock_jk_device(s, ctx.se, ctx.sc)
            else:
                gs = torch.from_numpy(b.fock_jk(s.numpy(), ctx.se, ctx.sc))
            gd = gs / w
            if ctx.squeeze:
                gd = gd[0]
        if ctx.needs_input_grad[1]:
            n = b.nbf
            S = [unpack(x, n) for x in s.detach().cpu().numpy()]
            D = [unpack(x, n) for x in d2.cpu().numpy()]
            if len(S) == 1:
                de = b.grad2_bilinear(S[0], D[0], None, None, 8.0 * ctx.sc, 2.0 * ctx.se, 0.0)
            else:
                de = b.grad2_bilinear(S[0] + S[1], D[0] + D[1], S[0] - S[1], D[0] - D[1], 8.0 * ctx.sc,
                                      2.0 * ctx.se, 2.0 * ctx.se)
            gxyz = torch.from_numpy(de)
        return gd, gxyz, None, None, None


def fock_jk(d, builder, xyz=None, scale_exch=1.0, scale_coul=1.0):
    """Differentiable packed Fock matrices of the packed densities d."""
    return FockJK.apply(d, xyz, builder, scale_exch, scale_coul)


def two_electron_energy(d, builder, xyz=None):
    """E2 = 1/2 Tr D G(D) for RHF packed D (1-D) or sum over spins of
    1/2 Tr D_s F_s for (2, ntri) UHF densities, differentiable in d and xyz."""
    f = fock_jk(d, builder, xyz)
    w = 1.0 / _tri_weights(builder.nbf, d.device)   # full-matrix weight of each packed element
    return 0.5 * torch.sum(d * f * w)
