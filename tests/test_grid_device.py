"""The molecular grid with the Becke partition on the device
(occ_xc_molecular_grid_device, occ_gb300/csrc/xc_grid.cu) against the host
restatement of src/numint/grid_utils.cpp:149-200 (occ_xc_molecular_grid)."""
import ctypes as C
import time

import numpy as np
import pytest

import occ_gb300 as og
from occ_gb300 import workloads as wl
from occ_gb300.xc import _ip, _ptr
from helpers import host_grid


def test_grid_count_needs_no_partition():
    """The count call (NULL buffers) skips the O(N natom^2) partition."""
    mol = wl.water_cluster(16, box=8.0, seed=1)
    b = wl.basis_for(mol, "def2-svp")
    lib = og.library()
    atoms = b.atoms()
    Z = np.array([a.atomic_number for a in atoms], dtype=np.int32)
    xyz = np.array([[a.x, a.y, a.z] for a in atoms], dtype=np.float64).ravel()
    l, at, npr, ex, co = b.arrays()
    gs = og.GridSettings()._c()
    n = C.c_long(0)
    t = time.perf_counter()
    assert lib.occ_xc_molecular_grid(len(Z), _ptr(Z, _ip), _ptr(xyz), len(l), _ptr(l, _ip),
                                     _ptr(at, _ip), _ptr(npr, _ip), _ptr(ex), _ptr(co), 1,
                                     C.byref(gs), C.byref(n), None, None) == 0
    assert time.perf_counter() - t < 0.5
    assert n.value > 400000


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["water", "water8", "mixed_elements", "cartesian_6-31g"])
def test_device_partition_matches_host(case):
    if case == "water":
        b = wl.basis_for(wl.water(), "6-31g")
    elif case == "water8":
        b = wl.basis_for(wl.water_cluster(8, box=7.0, seed=5), "def2-svp")
    elif case == "mixed_elements":  # H, C, N, O: every Treutler-Ahlrichs pair
        mol = og.Molecule([6, 7, 8, 1, 1, 1, 6],
                          [[0, 0, 0], [1.4, 0.1, 0], [-0.8, 1.1, 0.2], [-0.5, -0.9, 0.3],
                           [2.0, 0.9, 0.1], [1.9, -0.8, -0.2], [0.2, 0.3, 1.5]])
        b = wl.basis_for(mol, "def2-svp")
    else:
        b = wl.basis_for(wl.water_cluster(3, box=5.0, seed=2), "6-31g(d,p)", pure=False)
    P_h, W_h = og.molecular_grid(b)
    P_d, W_d = og.molecular_grid(b, device=0)
    assert np.array_equal(P_h, P_d)
    scale = np.max(np.abs(W_h))
    assert np.max(np.abs(W_d - W_h)) <= 1e-13 * scale, np.max(np.abs(W_d - W_h)) / scale
    assert abs(W_d.sum() - W_h.sum()) <= 1e-12 * abs(W_h.sum())


@pytest.mark.gpu
def test_molecule_grid_is_the_device_grid():
    """A molecule created on a context carries the device-partitioned grid,
    and its E_xc still matches the oracle on that grid."""
    import oracle
    b = wl.basis_for(wl.water_cluster(4, box=6.0, seed=7), "def2-svp")
    D = wl.random_density(b.nbf(), 20, seed=3)
    dft = og.DFT("pbe", b)
    P, W = dft.grid()
    P_h, W_h = host_grid(b)
    assert np.max(np.abs(W - W_h)) <= 1e-13 * np.max(np.abs(W_h))
    dft.compute_vxc(D, og.FP64)
    e_ref = oracle.xc_build(b, P_h, W_h, D, "pbe")[0]
    assert abs(dft.exchange_correlation_energy() - e_ref) <= 1e-8
