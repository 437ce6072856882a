"""Edge cases of the build, the unrestricted build, the gradient and VV10:
a single atom (all shells on one centre; an inversion-symmetric grid), the
hydrogen atom as a fully polarised doublet (rho_b = 0 everywhere), a basis
with g functions (l = 4), and an LDA / GGA pair on the same molecule."""
import numpy as np
import pytest

import occ_gb300 as og
import oracle
from occ_gb300 import workloads as wl
from helpers import host_grid


def _atom(Z, basis_name, pure=True):
    mol = og.Molecule([Z], [[0.3, -0.2, 0.1]])
    return wl.basis_for(mol, basis_name, pure)


def test_oracle_single_atom_gradient_vanishes():
    """On an atom-centred grid (the Lebedev rules are inversion-symmetric) the
    fixed-grid XC gradient of a spherically symmetric atomic density (s
    functions only) is zero to rounding."""
    b = _atom(1, "6-31g")
    D = wl.random_density(b.nbf(), 1, seed=2)
    P, W = host_grid(b)
    g = oracle.xc_gradient(b, P, W, D, "pbe")
    assert np.max(np.abs(g)) < 1e-12


def test_oracle_hydrogen_atom_fully_polarised():
    b = _atom(1, "6-31g")
    nbf = b.nbf()
    Q, _ = np.linalg.qr(np.random.default_rng(3).standard_normal((nbf, nbf)))
    D = np.zeros((2 * nbf, nbf))
    D[:nbf] = 0.5 * np.outer(Q[:, 0], Q[:, 0])
    P, W = host_grid(b)
    for method in ("lda", "pbe", "blyp"):
        e, V, n = oracle.xc_build_unrestricted(b, P, W, D, method)
        assert np.isfinite(e) and np.all(np.isfinite(V))
        assert abs(n[1]) < 1e-15  # no beta density
        assert np.max(np.abs(V[:nbf] - V[:nbf].T)) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["lda", "pbe", "b3lyp"])
def test_single_atom_gpu(method):
    b = _atom(8, "def2-tzvp")
    D = wl.random_density(b.nbf(), 4, seed=5)
    dft = og.DFT(method, b)
    P, W = dft.grid()
    e_ref, V_ref, _ = oracle.xc_build(b, P, W, D, method)
    V = dft.compute_vxc(D, og.FP64)
    assert abs(dft.exchange_correlation_energy() - e_ref) <= 1e-8
    assert np.max(np.abs(V - V_ref)) <= 1e-9
    Vm = dft.compute_vxc(D, og.MIXED)
    assert abs(dft.exchange_correlation_energy() - e_ref) <= 1e-6
    assert np.max(np.abs(Vm - V_ref)) <= 1e-5
    g = dft.compute_xc_gradient(D)
    g_ref = oracle.xc_gradient(b, P, W, D, method)
    assert np.max(np.abs(g - g_ref)) <= 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_hydrogen_atom_fully_polarised_gpu(precision):
    prec = og.FP64 if precision == "fp64" else og.MIXED
    b = _atom(1, "def2-svp")
    nbf = b.nbf()
    Q, _ = np.linalg.qr(np.random.default_rng(3).standard_normal((nbf, nbf)))
    D = np.zeros((2 * nbf, nbf))
    D[:nbf] = 0.5 * np.outer(Q[:, 0], Q[:, 0])
    dft = og.DFT("pbe", b)
    V = dft.compute_vxc(D, prec)
    P, W = dft.grid()
    e_ref, V_ref, n_ref = oracle.xc_build_unrestricted(b, P, W, D, "pbe")
    tol_e, tol_v = (1e-8, 1e-9) if precision == "fp64" else (1e-6, 1e-5)
    assert abs(dft.exchange_correlation_energy() - e_ref) <= tol_e
    assert np.max(np.abs(V - V_ref)) <= tol_v
    assert abs(dft.integrated_spin_densities()[1]) < 1e-12


@pytest.mark.gpu
def test_g_functions_gpu():
    """A shell with l = 4 (Cartesian and pure) through both paths."""
    for pure in (True, False):
        mol = og.Molecule([8, 1], [[0.0, 0.0, 0.0], [0.97, 0.0, 0.0]])
        b = wl.basis_for(mol, "def2-svp", pure)
        # add a g shell on O (one primitive, normalised as OCC would)
        import ctypes as C
        from occ_gb300.xc import _ptr
        e = np.array([1.1])
        c = np.array([1.0])
        assert og.library().occ_xc_normalize_shell(4, 1, _ptr(e), _ptr(c)) == 0
        b.shells.append(og.Shell(4, 0, np.array(b.shells[0].origin), e, c))
        D = wl.random_density(b.nbf(), 5, seed=7)
        dft = og.DFT("pbe", b)
        P, W = dft.grid()
        e_ref, V_ref, _ = oracle.xc_build(b, P, W, D, "pbe")
        V = dft.compute_vxc(D, og.FP64)
        assert abs(dft.exchange_correlation_energy() - e_ref) <= 1e-8
        assert np.max(np.abs(V - V_ref)) <= 1e-9
        Vm = dft.compute_vxc(D, og.MIXED)
        assert np.max(np.abs(Vm - V_ref)) <= 1e-5
        g = dft.compute_xc_gradient(D)
        assert np.max(np.abs(g - oracle.xc_gradient(b, P, W, D, "pbe"))) <= 1e-9


@pytest.mark.gpu
def test_single_atom_vv10_and_grid():
    b = _atom(7, "def2-svp")
    D = wl.random_density(b.nbf(), 3, seed=9)
    dft = og.DFT("pbe", b)
    e, V = dft.nlc_vv10(D)
    P, W = dft.nlc_grid()
    e_ref, V_ref = oracle.nlc_vv10(b, P, W, D)
    assert abs(e - e_ref) <= 1e-10 * max(1.0, abs(e_ref))
    assert np.max(np.abs(V - V_ref)) <= 1e-9
    Pd, Wd = og.molecular_grid(b, device=0)
    Ph, Wh = og.molecular_grid(b)
    assert np.array_equal(Pd, Ph) and np.max(np.abs(Wd - Wh)) <= 1e-13 * np.max(Wh)
