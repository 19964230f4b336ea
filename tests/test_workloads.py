"""The seeded synthetic workloads follow the stated construction rules (CPU):
water geometry (O-H 0.9572 A, HOH 104.52 deg, oxygens uniform in the cube with
O-O >= 2.7 A, each molecule rotated), the all-trans alkane (C-C 1.54 A, C-H
1.09 A, tetrahedral angles, +-0.02 A jitter per coordinate), the RHF density
D = 2 C C^T with S-orthonormal columns, and the basis sizes of the configurations."""
import math

import numpy as np
import pytest

from openqp_gb300 import workloads
from openqp_gb300.basis import build_basis, unpack
from openqp_gb300.onee import overlap_kinetic

BOHR = 1.0 / workloads.ANGSTROM   # Angstrom per bohr


def _dist(a, b):
    return float(np.linalg.norm(a - b)) * BOHR


def _angle(a, c, b):
    u, v = a - c, b - c
    return math.degrees(math.acos(float(u @ v) / float(np.linalg.norm(u) * np.linalg.norm(v))))


@pytest.mark.parametrize("nwater,edge,seed", [(4, 6.0, 0), (32, 14.0, 0), (16, 9.52, 3)])
def test_water_cluster_rules(nwater, edge, seed):
    z, xyz = workloads.water_cluster(nwater, edge, seed)
    assert list(z) == [8.0, 1.0, 1.0] * nwater
    ox = xyz[0::3]
    for k in range(nwater):
        o, h1, h2 = xyz[3 * k], xyz[3 * k + 1], xyz[3 * k + 2]
        assert _dist(o, h1) == pytest.approx(0.9572, abs=1e-10)
        assert _dist(o, h2) == pytest.approx(0.9572, abs=1e-10)
        assert _angle(h1, o, h2) == pytest.approx(104.52, abs=1e-8)
        assert np.all(o * BOHR >= 0.0) and np.all(o * BOHR <= edge)
    d = [_dist(ox[i], ox[j]) for i in range(nwater) for j in range(i)]
    assert min(d) >= 2.7
    # molecules are rotated independently (not all H-O-H planes parallel)
    normals = [np.cross(xyz[3 * k + 1] - xyz[3 * k], xyz[3 * k + 2] - xyz[3 * k]) for k in range(nwater)]
    assert len({tuple(np.round(n / np.linalg.norm(n), 6)) for n in normals}) == nwater
    # seeded: the same seed gives the same cluster, another seed another one
    assert np.array_equal(workloads.water_cluster(nwater, edge, seed)[1], xyz)
    assert not np.allclose(workloads.water_cluster(nwater, edge, seed + 1)[1], xyz)


def test_alkane_rules():
    n = 40
    z, xyz = workloads.alkane(n, 0)
    assert list(z).count(6.0) == n and list(z).count(1.0) == 2 * n + 2
    C, H = xyz[:n], xyz[n:]
    tol = 2.0 * math.sqrt(3.0) * 0.02 + 1e-9   # two atoms, each displaced by <= 0.02 A per coordinate
    for k in range(n - 1):
        assert abs(_dist(C[k], C[k + 1]) - 1.54) <= tol
    for h in H:
        dch = min(_dist(h, c) for c in C)
        assert abs(dch - 1.09) <= tol
    for k in range(1, n - 1):
        assert abs(_angle(C[k - 1], C[k], C[k + 1]) - math.degrees(workloads.TETRA)) < 3.0
    # jitter within +-0.02 A of the ideal chain: the unjittered chain is the jitter-0 call
    _, ideal = workloads.alkane(n, 0, jitter=0.0)
    assert np.abs(xyz - ideal).max() * BOHR <= 0.02 + 1e-12


def test_density_is_rhf_idempotent():
    bas = workloads.water_cluster_basis(2, workloads.cube_edge_like_c1(2), 5, "6-31g(d)")
    S, _ = overlap_kinetic(bas)
    nocc = workloads.nelectrons(bas) // 2
    D = unpack(workloads.density(bas, nocc, 5, S=S), bas.nbf)
    assert np.abs(D - D.T).max() < 1e-12
    assert np.trace(D @ S) == pytest.approx(2 * nocc, abs=1e-9)
    assert np.abs(D @ S @ D - 2.0 * D).max() < 1e-9


@pytest.mark.parametrize("case,nbf", [("water4_631gd", 76), ("water32_ccpvdz", 768), ("alkane40_631gd", 764)])
def test_configuration_basis_sizes(case, nbf):
    if case == "water4_631gd":
        bas = workloads.water_cluster_basis(4, 6.0, 0, "6-31g(d)")
    elif case == "water32_ccpvdz":
        bas = workloads.water_cluster_basis(32, 14.0, 0, "cc-pvdz", spherical=True)
    else:
        z, xyz = workloads.alkane(40, 0)
        bas = build_basis(z, xyz, "6-31g(d)")
    assert bas.nbf == nbf
