"""CPU: the C ABI library (loads, exports what include/occ_xc.h declares) and
the host-side set-up (basis normalisation, molecular grid, oracle build
properties).  No compute call needs a GPU here."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import occ_gb300 as og
import oracle
from occ_gb300 import workloads as wl
from occ_gb300.xc import ERR_ARG
from helpers import host_grid, water_case

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol():
    with open(os.path.join(ROOT, "include", "occ_xc.h")) as f:
        header = f.read()
    names = set(re.findall(r"\b(occ_xc_\w+)\s*\(", header))
    assert len(names) >= 15
    lib = og.library()
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_cosx_entry_points_refuse_null_arguments():
    """The COSX entry points (restricted and unrestricted, host and device
    buffers) return OCC_XC_ERR_ARG for missing handles or buffers before any
    device work."""
    lib = og.library()
    four = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    for name in ("occ_xc_cosx_exchange", "occ_xc_cosx_exchange_unrestricted"):
        fn = getattr(lib, name)
        fn.argtypes = four
        assert fn(None, None, None, None) == ERR_ARG
    for name in ("occ_xc_cosx_exchange_device", "occ_xc_cosx_exchange_unrestricted_device"):
        fn = getattr(lib, name)
        fn.argtypes = four + [C.c_void_p]
        assert fn(None, None, None, None, None) == ERR_ARG


def test_normalised_shell_has_unit_self_overlap():
    """Shell::incorporate_shell_norm (src/gto/shell.cpp:180-186): the
    contracted radial function is normalised to one."""
    from math import gamma
    lib = og.library()
    exps = np.array([5484.67166, 825.234946, 188.046958, 52.9645, 16.8975704, 5.79963534])
    for l in range(4):
        c = np.array([0.00183107443, 0.0139501722, 0.0684450781, 0.232714336, 0.470192898,
                      0.358520853])
        assert lib.occ_xc_normalize_shell(l, len(exps), exps.ctypes.data_as(og.xc._dp),
                                          c.ctypes.data_as(og.xc._dp)) == 0
        n = l * 2 + 2
        S = sum(ci * cj * gamma((n + 1) / 2) / (2 * (ai + aj) ** ((n + 1) / 2))
                for ci, ai in zip(c, exps) for cj, aj in zip(c, exps))
        assert abs(S - 1.0) < 1e-13


def test_basis_sizes():
    mol = wl.water()
    assert wl.basis_for(mol, "6-31g").nbf() == 13
    assert wl.basis_for(mol, "def2-svp").nbf() == 24
    assert wl.basis_for(mol, "def2-svp", pure=False).nbf() == 25
    assert wl.basis_for(wl.alkane(30), "def2-tzvp").nbf() == 1302


def test_molecular_grid_integrates_gaussians():
    mol, b, _ = water_case("6-31g")
    P, W = host_grid(b)
    assert len(W) == 28590
    for atom in b.atoms():
        A = np.array([atom.x, atom.y, atom.z])
        for a in (0.5, 5.0):
            f = (a / np.pi) ** 1.5 * np.exp(-a * ((P - A) ** 2).sum(1))
            assert abs((W * f).sum() - 1.0) < 1e-5


def test_becke_weights_partition_unity():
    """Becke weights of all atoms at a point sum to one, so the molecular grid
    integrates as accurately as the atom grids do.  (Weights may be negative:
    the published 230-point Lebedev rule has a negative weight, and so does
    the reference's grid.)"""
    mol = wl.water_cluster(3, box=5.0, seed=2)
    b = wl.basis_for(mol, "6-31g")
    P, W = host_grid(b)
    for atom in b.atoms()[:3]:
        A = np.array([atom.x, atom.y, atom.z])
        f = np.exp(-((P - A) ** 2).sum(1))
        assert abs((W * f).sum() - np.pi ** 1.5) < 1e-5


def test_reduced_hydrogen_grid_settings():
    mol, b, _ = water_case("6-31g")
    full = og.GridSettings(reduced_first_row_element_grid=False)
    P1, _ = host_grid(b)
    P2, _ = host_grid(b, full)
    assert len(P2) > len(P1)


def test_oracle_build_properties():
    mol, b, D = water_case("6-31g")
    P, W = host_grid(b)
    e, V, ne = oracle.xc_build(b, P, W, D, "pbe")
    assert np.max(np.abs(V - V.T)) < 1e-14
    # screened vs (nearly) unscreened agree within the reference's own bar
    # for screening (tests/dft_tests.cpp:904-931)
    e2, V2, _ = oracle.xc_build(b, P, W, D, "pbe", screen=1e-16)
    assert abs(e - e2) < 1e-8
    assert np.max(np.abs(V - V2)) < 1e-8
    # the leaf stride of the CPU baseline sample processes a subset only
    e3, _, _ = oracle.xc_build(b, P, W, D, "pbe", leaf_stride=4)
    assert abs(e3) < abs(e)


def test_oracle_lda_potential_is_functional_derivative():
    """V_xc is the derivative of E_xc with respect to the density matrix:
    E(D + hX) - E(D - hX) = 2h tr(V X)."""
    mol, b, D = water_case("6-31g")
    P, W = host_grid(b)
    rng = np.random.default_rng(9)
    X = rng.standard_normal(D.shape)
    X = 0.5 * (X + X.T)
    h = 1e-5
    _, V, _ = oracle.xc_build(b, P, W, D, "lda")
    ep, _, _ = oracle.xc_build(b, P, W, D + h * X, "lda")
    em, _, _ = oracle.xc_build(b, P, W, D - h * X, "lda")
    # OCC's V multiplies D2 = 2 D: dE/dD = 2 V
    assert abs((ep - em) / (2 * h) - 2 * np.sum(V * X)) < 1e-6


@pytest.mark.parametrize("method", ["pbe", "blyp"])
def test_oracle_gga_potential_is_functional_derivative(method):
    mol, b, D = water_case("6-31g")
    P, W = host_grid(b)
    rng = np.random.default_rng(11)
    X = rng.standard_normal(D.shape)
    X = 0.5 * (X + X.T)
    h = 1e-5
    _, V, _ = oracle.xc_build(b, P, W, D, method)
    ep, _, _ = oracle.xc_build(b, P, W, D + h * X, method)
    em, _, _ = oracle.xc_build(b, P, W, D - h * X, method)
    assert abs((ep - em) / (2 * h) - 2 * np.sum(V * X)) < 1e-6


def test_morton_leaves_match_reference_rules():
    """Leaf sizes (include/occ/numint/spatial_grid_hierarchy.h:26-30): 128
    points each, the last leaf takes what remains when at most 256 are left;
    every point is in exactly one leaf."""
    mol, b, _ = water_case("6-31g")
    P, W = host_grid(b)
    perm, off, cnt, cen, rad = oracle.morton_leaves(P)
    assert sorted(perm.tolist()) == list(range(len(P)))
    assert np.all(cnt[:-1] == 128) and 128 < cnt[-1] <= 256 or len(P) <= 256
    assert off[-1] + cnt[-1] == len(P)
    for i in range(0, len(off), 37):
        pts = P[perm[off[i]:off[i] + cnt[i]]]
        assert np.allclose(cen[i], pts.mean(0))
        assert abs(rad[i] - np.linalg.norm(pts - cen[i], axis=1).max()) < 1e-12
