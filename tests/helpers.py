"""Shared fixtures for the parity tests: molecules, bases, densities and the
oracle run on the grid the library built."""
import ctypes as C

import numpy as np

import occ_gb300 as og
from occ_gb300 import workloads as wl
from occ_gb300.xc import _GridSettings, _dp, _ip, _ptr

# Parity bars for the FP64 path against the oracle.
TOL_E_FP64 = 1e-8   # Ha
TOL_V_FP64 = 1e-9   # max |dV_xc|
# Mixed precision path against the FP64 oracle.
TOL_E_MIXED = 1e-6  # Ha


def host_grid(basis, settings=None):
    """Molecular grid from the library's host-only entry point (no GPU)."""
    lib = og.library()
    lib.occ_xc_molecular_grid.argtypes = [C.c_int, _ip, _dp, C.c_int, _ip, _ip, _ip, _dp, _dp,
                                          C.c_int, C.POINTER(_GridSettings),
                                          C.POINTER(C.c_long), _dp, _dp]
    atoms = basis.atoms()
    Z = np.array([a.atomic_number for a in atoms], dtype=np.int32)
    xyz = np.array([[a.x, a.y, a.z] for a in atoms], dtype=np.float64).ravel()
    l, at, npr, ex, co = basis.arrays()
    gs = (settings or og.GridSettings())._c()
    n = C.c_long(0)
    args = (len(Z), _ptr(Z, _ip), _ptr(xyz), len(l), _ptr(l, _ip), _ptr(at, _ip), _ptr(npr, _ip),
            _ptr(ex), _ptr(co), int(basis.pure), C.byref(gs), C.byref(n))
    assert lib.occ_xc_molecular_grid(*args, None, None) == 0
    P = np.zeros((n.value, 3))
    W = np.zeros(n.value)
    assert lib.occ_xc_molecular_grid(*args, _ptr(P), _ptr(W)) == 0
    return P, W


def water_case(basis_name="6-31g", nocc=5, seed=0, pure=True):
    mol = wl.water()
    b = wl.basis_for(mol, basis_name, pure)
    D = wl.random_density(b.nbf(), nocc, seed)
    return mol, b, D
TOL_V_MIXED = 1e-5  # max |dV_xc| of the mixed path against FP64
