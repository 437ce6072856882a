"""GPU parity: the CUDA XC build through the C ABI against the CPU oracle on
the same grid, basis and density (the oracle restates
include/occ/dft/dft.h:192-388)."""
import numpy as np
import pytest

import occ_gb300 as og
import oracle
from occ_gb300 import workloads as wl
from helpers import TOL_E_FP64, TOL_E_MIXED, TOL_V_FP64, TOL_V_MIXED, water_case

pytestmark = pytest.mark.gpu


def _run(method, basis, D, precision=og.FP64, build=None):
    dft = og.DFT(method, basis, build_settings=build)
    V = dft.compute_vxc(D, precision)
    P, W = dft.grid()
    kw = {}
    if build is not None:
        kw = dict(screen=build.xc_screening_threshold, density_threshold=build.density_threshold,
                  leaf=(build.leaf_target, build.leaf_min, build.leaf_max))
    e_ref, V_ref, n_ref = oracle.xc_build(basis, P, W, D, method, **kw)
    return dft, V, V_ref, e_ref, n_ref


@pytest.mark.parametrize("method", ["lda", "svwn5", "pbe", "blyp", "b3lyp", "b3lyp5", "bpbe",
                                    "pbeh", "bhandh", "bhandhlyp", "vwn5"])
@pytest.mark.parametrize("basis_name", ["6-31g", "3-21g"])
def test_water_fp64(method, basis_name):
    mol, b, D = water_case(basis_name)
    dft, V, V_ref, e_ref, n_ref = _run(method, b, D)
    assert abs(dft.exchange_correlation_energy() - e_ref) <= TOL_E_FP64
    assert np.max(np.abs(V - V_ref)) <= TOL_V_FP64
    assert abs(dft.integrated_density() - n_ref) <= 1e-9
    assert np.max(np.abs(V - V.T)) <= 1e-12


@pytest.mark.parametrize("method", ["pbe", "lda"])
def test_water_dimer_svp_fp64(method):
    mol = wl.water_cluster(2, box=4.0, seed=3)
    b = wl.basis_for(mol, "def2-svp")
    D = wl.random_density(b.nbf(), 10, seed=1)
    dft, V, V_ref, e_ref, _ = _run(method, b, D)
    assert abs(dft.exchange_correlation_energy() - e_ref) <= TOL_E_FP64
    assert np.max(np.abs(V - V_ref)) <= TOL_V_FP64


def test_cartesian_d_shells_fp64():
    """Cartesian (OCC's default) d shells: common_fac 1, CCA order."""
    mol = wl.water()
    b = wl.basis_for(mol, "6-31g(d,p)", pure=False)
    D = wl.random_density(b.nbf(), 5, seed=2)
    dft, V, V_ref, e_ref, _ = _run("pbe", b, D)
    assert abs(dft.exchange_correlation_energy() - e_ref) <= TOL_E_FP64
    assert np.max(np.abs(V - V_ref)) <= TOL_V_FP64


def test_f_shells_fp64():
    """def2-TZVP carbon carries f shells (l = 3)."""
    mol = og.Molecule([6, 1, 1, 1, 1], [[0, 0, 0], [0.63, 0.63, 0.63], [-0.63, -0.63, 0.63],
                                        [-0.63, 0.63, -0.63], [0.63, -0.63, -0.63]])
    b = wl.basis_for(mol, "def2-tzvp")
    D = wl.random_density(b.nbf(), 5, seed=4)
    dft, V, V_ref, e_ref, _ = _run("b3lyp", b, D)
    assert abs(dft.exchange_correlation_energy() - e_ref) <= TOL_E_FP64
    assert np.max(np.abs(V - V_ref)) <= TOL_V_FP64


def test_screening_off_matches_dense_limit():
    """Tighter screening moves the result by less than the reference's own
    screened-vs-dense bar (tests/dft_tests.cpp:904-931)."""
    mol, b, D = water_case("6-31g")
    d1 = og.DFT("pbe", b)
    d1.compute_vxc(D)
    d2 = og.DFT("pbe", b, build_settings=og.BuildSettings(xc_screening_threshold=1e-14))
    d2.compute_vxc(D)
    assert abs(d1.exchange_correlation_energy() - d2.exchange_correlation_energy()) < 1e-8


@pytest.mark.parametrize("method", ["lda", "pbe", "blyp", "b3lyp"])
@pytest.mark.parametrize("basis_name", ["6-31g", "def2-svp"])
def test_water_mixed(method, basis_name):
    mol, b, D = water_case(basis_name)
    dft, V, V_ref, e_ref, n_ref = _run(method, b, D, precision=og.MIXED)
    assert abs(dft.exchange_correlation_energy() - e_ref) <= TOL_E_MIXED
    assert np.max(np.abs(V - V_ref)) <= TOL_V_MIXED
    assert abs(dft.integrated_density() - n_ref) <= 1e-6


def test_water_hexamer_svp_mixed_vs_fp64():
    mol = wl.water_cluster(6, box=6.0, seed=5)
    b = wl.basis_for(mol, "def2-svp")
    D = wl.random_density(b.nbf(), 30, seed=5)
    dft = og.DFT("pbe", b)
    V64 = dft.compute_vxc(D, og.FP64)
    e64 = dft.exchange_correlation_energy()
    Vm = dft.compute_vxc(D, og.MIXED)
    em = dft.exchange_correlation_energy()
    assert abs(em - e64) <= TOL_E_MIXED
    assert np.max(np.abs(Vm - V64)) <= TOL_V_MIXED


def test_repeat_builds_identical_energy():
    mol, b, D = water_case("6-31g")
    dft = og.DFT("pbe", b)
    dft.compute_vxc(D)
    e1 = dft.exchange_correlation_energy()
    dft.compute_vxc(D)
    assert dft.exchange_correlation_energy() == e1
