"""openqp_gb300: GB300-native direct two-electron Fock build for OpenQP.

Schwarz- and density-screened (ab|cd) shell quartets over s, p and d shells,
evaluated with Rys quadrature in hand-written sm_103a CUDA kernels and
contracted on the fly into Coulomb J and exchange K for RHF, UHF and ROHF
densities, behind OpenQP's own route-C seam (``routec_fock_jk``).
"""
from .basis import build_basis, pack, unpack  # noqa: F401

__all__ = ["build_basis", "pack", "unpack", "FockBuilder"]


def __getattr__(name):
    if name == "FockBuilder":
        from .fock import FockBuilder
        return FockBuilder
    raise AttributeError(name)
