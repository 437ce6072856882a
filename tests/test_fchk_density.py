"""A converged RHF density of water (6-31G(d,p), pure; the Gaussian checkpoint
in the reference's tests/wavefunction_io_tests.cpp, converted to OCC's AO
order by tests/golden/make_fchk_density.py).  With a real SCF density the
integrated density must be the electron count: a check of the basis
normalisation, the AO order and the collocation that a random density cannot
give."""
import os

import numpy as np
import pytest

import occ_gb300 as og
import oracle
from helpers import TOL_E_FP64, TOL_E_MIXED, TOL_V_FP64, TOL_V_MIXED, host_grid

HERE = os.path.dirname(os.path.abspath(__file__))


def fchk_case():
    f = np.load(os.path.join(HERE, "golden", "water_rhf_631gdp.npz"))
    atoms = [og.Atom(int(z), *xyz) for z, xyz in zip(f["Z"], f["xyz_bohr"])]
    lib = og.library()
    shells, off = [], 0
    for l, a, n in zip(f["shell_l"], f["shell_atom"], f["shell_nprim"]):
        e = f["exponents"][off:off + n].copy()
        c = f["coefficients"][off:off + n].copy()
        from occ_gb300.xc import _ptr
        assert lib.occ_xc_normalize_shell(int(l), int(n), _ptr(e), _ptr(c)) == 0
        shells.append(og.Shell(int(l), int(a), np.array(f["xyz_bohr"][a]), e, c))
        off += n
    b = og.AOBasis(atoms, shells, "6-31g(d,p)")
    b.set_pure(True)
    return b, f["D"], int(f["nelec"])


def test_converged_density_integrates_to_electron_count():
    b, D, nelec = fchk_case()
    assert b.nbf() == D.shape[0] == 24
    P, W = host_grid(b)
    for method in ("lda", "pbe", "b3lyp"):
        e, V, n = oracle.xc_build(b, P, W, D, method)
        assert abs(n - nelec) < 2e-5, (method, n)
        assert np.allclose(V, V.T, atol=1e-12)
    # E_xc of water near its SCF density: LDA about -8.9 Ha (a sanity window)
    e_lda, _, _ = oracle.xc_build(b, P, W, D, "lda")
    assert -9.5 < e_lda < -8.5


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["lda", "svwn5", "pbe", "blyp", "b3lyp"])
def test_converged_density_gpu_parity(method):
    b, D, nelec = fchk_case()
    dft = og.DFT(method, b)
    V = dft.compute_vxc(D, og.FP64)
    P, W = dft.grid()
    e_ref, V_ref, n_ref = oracle.xc_build(b, P, W, D, method)
    assert abs(dft.exchange_correlation_energy() - e_ref) <= TOL_E_FP64
    assert np.max(np.abs(V - V_ref)) <= TOL_V_FP64
    assert abs(dft.integrated_density() - nelec) < 2e-5
    Vm = dft.compute_vxc(D, og.MIXED)
    assert abs(dft.exchange_correlation_energy() - e_ref) <= TOL_E_MIXED
    assert np.max(np.abs(Vm - V_ref)) <= TOL_V_MIXED
