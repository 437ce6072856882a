"""End-to-end pins against the values the reference's own tests assert.

* tests/qm_tests.cpp:527-549 ("Water RHF SCF energy"): RHF energies of water
  in STO-3G and 3-21G.  The small s/p RHF of tests/golden/make_hf_density.py
  reproduces them, which pins the integrals, the basis normalisation and the
  SCF that produce the density fixture below.
* tests/isolated_xc_tests.cpp:28-200: water HF/3-21G density, then E_xc and
  the XC gradient of LDA, PBE and BLYP.  The reference asserts E_xc against
  PySCF values at 1e-8 and the gradient at 1e-4.  E_xc moves by ~1e-6 Ha
  between reasonable grids (LMG precision 1e-10 .. 1e-14 here), so the
  PySCF numbers pin the grid only to that level: the bar here is 3e-6 Ha for
  E_xc, the reference's own 1e-4 Ha/Bohr for the gradient, and its 1e-10 for
  the gradient's symmetry (x components zero, H y components opposite)."""
import os

import numpy as np
import pytest

import occ_gb300 as og
import oracle
from helpers import host_grid

HERE = os.path.dirname(os.path.abspath(__file__))

# tests/isolated_xc_tests.cpp:94, 138, 182 and the gradients beside them
EXC = {"lda": -8.786388687644, "pbe": -9.262866622721, "blyp": -9.325386381715}
GRAD = {  # O z, H1 y, H1 z (Ha/Bohr)
    "lda": (-0.3433120725, -0.2038702847, 0.1716549224),
    "pbe": (-0.3409121608, -0.2022757063, 0.1704560022),
    "blyp": (-0.3356949358, -0.1988199134, 0.1678460822),
}
TOL_EXC_PUBLISHED = 3e-6
TOL_GRAD_PUBLISHED = 1e-4


def water_hf_case():
    f = np.load(os.path.join(HERE, "golden", "water_hf_321g.npz"))
    mol = og.Molecule([8, 1, 1], [[0.0, 0.0, 0.0], [0.0, -0.757, 0.587], [0.0, 0.757, 0.587]])
    b = og.AOBasis.load(mol.atoms(), "3-21g")
    b.set_pure(True)
    return b, f["D"]


def test_small_rhf_reproduces_reference_hf_energies():
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_hf_density as hf
    atoms = [og.Atom(8, -1.32695761, -0.10593856, 0.01878821),
             og.Atom(1, -1.93166418, 1.60017351, -0.02171049),
             og.Atom(1, 0.48664409, 0.07959806, 0.00986248)]
    Z = np.array([8.0, 1.0, 1.0])
    xyz = np.array([[a.x, a.y, a.z] for a in atoms])
    enuc = sum(Z[a] * Z[c] / np.linalg.norm(xyz[a] - xyz[c]) for a in range(3) for c in range(a))
    for name, ref in (("sto-3g", -74.963706080054), ("3-21g", -75.585325673488)):
        aos = hf.ao_list(og.AOBasis.load(atoms, name))
        S, T, V = hf.one_electron(aos, Z, xyz)
        E, D, _ = hf.rhf(S, T + V, hf.eri(aos), 5, enuc)
        assert abs(E - ref) < 1e-7, (name, E, ref)
        assert abs(np.sum(2 * D * S) - 10.0) < 1e-10


def _check_gradient(g, method):
    assert np.max(np.abs(g[:, 0])) < 1e-10
    assert abs(g[1, 1] + g[2, 1]) < 1e-10
    ref = GRAD[method]
    assert abs(g[0, 2] - ref[0]) < TOL_GRAD_PUBLISHED
    assert abs(g[1, 1] - ref[1]) < TOL_GRAD_PUBLISHED
    assert abs(g[1, 2] - ref[2]) < TOL_GRAD_PUBLISHED


@pytest.mark.parametrize("method", ["lda", "pbe", "blyp"])
def test_oracle_matches_reference_isolated_xc_values(method):
    b, D = water_hf_case()
    P, W = host_grid(b)
    e, _, n = oracle.xc_build(b, P, W, D, method)
    assert abs(e - EXC[method]) < TOL_EXC_PUBLISHED, (e, EXC[method])
    assert abs(n - 10.0) < 1e-5
    _check_gradient(oracle.xc_gradient(b, P, W, D, method), method)


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["lda", "pbe", "blyp"])
def test_gpu_matches_reference_isolated_xc_values(method):
    b, D = water_hf_case()
    dft = og.DFT(method, b)
    P, W = dft.grid()
    e_ref, V_ref, _ = oracle.xc_build(b, P, W, D, method)
    V = dft.compute_vxc(D, og.FP64)
    e = dft.exchange_correlation_energy()
    assert abs(e - EXC[method]) < TOL_EXC_PUBLISHED
    assert abs(e - e_ref) < 1e-8 and np.max(np.abs(V - V_ref)) < 1e-9
    dft.compute_vxc(D, og.MIXED)
    assert abs(dft.exchange_correlation_energy() - EXC[method]) < TOL_EXC_PUBLISHED
    g = dft.compute_xc_gradient(D)
    _check_gradient(g, method)
    assert np.max(np.abs(g - oracle.xc_gradient(b, P, W, D, method))) < 1e-9
