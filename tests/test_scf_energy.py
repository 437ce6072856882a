"""Kohn-Sham SCF total energies with the GPU XC build inside the loop: the
tensor-core (mixed) build against the FP64 build, and the FP64 build against
the oracle's XC build.

OCC's SCF (src/qm/scf.h) is outside the XC path; this test supplies its own
closed-shell Roothaan-Hall loop with DIIS and the one- and two-electron
integrals of tests/golden/make_hf_density.py (McMurchie-Davidson over s and p
shells, the AOs exactly as the collocation evaluates them), so that the
quantity the XC build ultimately feeds, the converged total energy
E = tr(P H) + 1/2 tr(P J[P]) + E_xc[P] + E_nuc with P = 2 mo.D and the Fock
matrix F = H + J[P] + V_xc, is compared between precisions: the mixed build
within 1e-6 Ha of FP64, the FP64 build within 1e-8 Ha of the oracle."""
import os
import sys

import numpy as np
import pytest

import occ_gb300 as og
import oracle
from occ_gb300 import workloads as wl

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_hf_density as hf  # noqa: E402

TOL_E_MIXED = 1e-6   # Ha, mixed against FP64
TOL_E_ORACLE = 1e-8  # Ha, FP64 against the oracle


def _system(name):
    if name == "water_631g":
        mol, basis_name = wl.water(), "6-31g"
    else:  # water dimer, 3-21G
        mol, basis_name = wl.water_cluster(2, box=4.0, seed=3), "3-21g"
    b = wl.basis_for(mol, basis_name)
    atoms = mol.atoms()  # Bohr
    Z = np.array([a.atomic_number for a in atoms], dtype=float)
    xyz = np.array([[a.x, a.y, a.z] for a in atoms])
    enuc = sum(Z[i] * Z[j] / np.linalg.norm(xyz[i] - xyz[j])
               for i in range(len(Z)) for j in range(i))
    aos = hf.ao_list(b)
    S, T, V = hf.one_electron(aos, Z, xyz)
    G = hf.eri(aos)
    nocc = int(round(Z.sum())) // 2
    return b, S, T + V, G, nocc, enuc


_CACHE = {}


def _cached(name):
    if name not in _CACHE:
        _CACHE[name] = _system(name)
    return _CACHE[name]


def ks_scf(S, H, G, nocc, enuc, xc, tol=1e-8, etol=1e-10, maxiter=200):
    """Closed-shell KS SCF with DIIS: xc(D) -> (E_xc, V_xc) for mo.D = D.
    Converged when max |F P S - S P F| < tol and the energy moves by less
    than etol.  Returns the total energy and the iteration count."""
    s, U = np.linalg.eigh(S)
    X = U @ np.diag(s ** -0.5) @ U.T
    F = H.copy()
    errs, focks = [], []
    E_old = 0.0
    for it in range(maxiter):
        _, Cp = np.linalg.eigh(X.T @ F @ X)
        C = X @ Cp
        D = C[:, :nocc] @ C[:, :nocc].T
        P = 2 * D
        J = np.einsum("ijkl,kl->ij", G, P)
        exc, Vxc = xc(D)
        F = H + J + Vxc
        E = np.sum(P * H) + 0.5 * np.sum(P * J) + exc + enuc
        err = F @ P @ S - S @ P @ F
        if np.max(np.abs(err)) < tol and abs(E - E_old) < etol:
            return E, it
        E_old = E
        errs.append(err)
        focks.append(F.copy())
        errs, focks = errs[-8:], focks[-8:]
        if len(errs) > 1:
            m = len(errs)
            B = -np.ones((m + 1, m + 1))
            B[m, m] = 0.0
            for a in range(m):
                for c in range(m):
                    B[a, c] = np.sum(errs[a] * errs[c])
            rhs = np.zeros(m + 1)
            rhs[m] = -1.0
            w = np.linalg.solve(B, rhs)[:m]
            F = sum(wi * Fi for wi, Fi in zip(w, focks))
    raise AssertionError("SCF did not converge")


def _gpu_xc(dft, precision):
    def xc(D):
        V = dft.compute_vxc(D, precision)
        return dft.exchange_correlation_energy(), V
    return xc


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["lda", "pbe", "blyp"])
@pytest.mark.parametrize("system", ["water_631g", "water2_321g"])
def test_scf_total_energy_mixed_vs_fp64(system, method):
    b, S, H, G, nocc, enuc = _cached(system)
    dft = og.DFT(method, b)
    e64, it64 = ks_scf(S, H, G, nocc, enuc, _gpu_xc(dft, og.FP64))
    # the mixed build's V_xc carries FP32-level rounding that does not vary
    # smoothly with D (operand slices on power-of-two scales chosen from D),
    # so its SCF is converged to a commutator of 1e-6 (the energy error that
    # leaves is second order, ~1e-12 Ha)
    emx, itmx = ks_scf(S, H, G, nocc, enuc, _gpu_xc(dft, og.MIXED), tol=1e-6, etol=1e-8)
    assert abs(emx - e64) <= TOL_E_MIXED, (emx, e64, emx - e64)
    # the plain FP64 path inside the same SCF against the oracle's XC build
    P, W = dft.grid()

    def xc_oracle(D):
        e, V, _ = oracle.xc_build(b, P, W, D, method)
        return e, V
    eor, _ = ks_scf(S, H, G, nocc, enuc, xc_oracle)
    assert abs(e64 - eor) <= TOL_E_ORACLE, (e64, eor, e64 - eor)
