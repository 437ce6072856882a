"""XC nuclear gradient, dE_xc/dR with the grid held fixed (OCC's
DFT::compute_xc_gradient, include/occ/dft/dft.h:599-749 and
src/dft/dft_gradient_kernels.cpp:472-595).

The oracle's gradient is pinned as the derivative of the oracle's E_xc (itself
pinned to the reference's golden vectors): central differences over shifts of
one atom's basis functions, grid fixed, on the converged water density.  The
screened gradient matches the dense one as the reference's
"DFT XC screening matches dense (gradient)" test requires (tests/dft_tests.cpp
:904-931)."""
import numpy as np
import pytest

import occ_gb300 as og
import oracle
from helpers import host_grid
from test_fchk_density import fchk_case


def _shifted(b, atom, axis, h):
    shells = []
    for s in b.shells:
        o = np.array(s.origin, dtype=np.float64).copy()
        if s.atom == atom:
            o[axis] += h
        shells.append(og.Shell(s.l, s.atom, o, s.exponents, s.coefficients))
    nb = og.AOBasis(b.atoms(), shells, b.name)
    nb.set_pure(b.pure)
    return nb


@pytest.mark.parametrize("method", ["lda", "pbe"])
def test_oracle_gradient_is_derivative_of_exc(method):
    b, D, _ = fchk_case()
    P, W = host_grid(b)
    g = oracle.xc_gradient(b, P, W, D, method, screen=1e-14)
    h = 1e-4
    for atom in range(3):
        for axis in range(3):
            ep = oracle.xc_build(_shifted(b, atom, axis, h), P, W, D, method, screen=1e-14)[0]
            em = oracle.xc_build(_shifted(b, atom, axis, -h), P, W, D, method, screen=1e-14)[0]
            assert abs(g[atom, axis] - (ep - em) / (2 * h)) < 1e-7, (atom, axis)


def test_oracle_gradient_screened_matches_dense():
    b, D, _ = fchk_case()
    P, W = host_grid(b)
    gs = oracle.xc_gradient(b, P, W, D, "pbe", screen=1e-10)
    gd = oracle.xc_gradient(b, P, W, D, "pbe", screen=0.0)
    assert np.max(np.abs(gs - gd)) < 1e-8


TOL_GRAD = 1e-9  # Ha/Bohr, FP64 gradient against the oracle


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["lda", "svwn5", "pbe", "blyp", "b3lyp"])
def test_gradient_converged_water_gpu_parity(method):
    b, D, _ = fchk_case()
    dft = og.DFT(method, b)
    g = dft.compute_xc_gradient(D)
    P, W = dft.grid()
    g_ref = oracle.xc_gradient(b, P, W, D, method)
    assert g.shape == (3, 3)
    assert np.max(np.abs(g - g_ref)) <= TOL_GRAD, np.max(np.abs(g - g_ref))
    e_ref = oracle.xc_build(b, P, W, D, method)[0]
    assert abs(dft.exchange_correlation_energy() - e_ref) <= 1e-8


@pytest.mark.gpu
@pytest.mark.parametrize("basis_name,pure,method", [("def2-svp", True, "pbe"),
                                                    ("6-31g(d,p)", False, "b3lyp"),
                                                    ("def2-tzvp", True, "lda")])
def test_gradient_water_cluster_gpu_parity(basis_name, pure, method):
    """Several waters: leaves with more than one 64-AO tile, d and f shells,
    Cartesian and pure."""
    from occ_gb300 import workloads as wl
    mol = wl.water_cluster(4, box=6.0, seed=3)
    b = wl.basis_for(mol, basis_name, pure)
    D = wl.random_density(b.nbf(), 20, seed=4)
    dft = og.DFT(method, b)
    g = dft.compute_xc_gradient(D)
    P, W = dft.grid()
    g_ref = oracle.xc_gradient(b, P, W, D, method)
    scale = max(1.0, np.max(np.abs(g_ref)))
    assert np.max(np.abs(g - g_ref)) <= TOL_GRAD * scale, np.max(np.abs(g - g_ref))


@pytest.mark.gpu
def test_gradient_leaf_groups_match_one_group():
    """A small workspace cap splits the leaves into many groups; the gradient
    is the same (up to the order of the atomic adds)."""
    b, D, _ = fchk_case()
    dft = og.DFT("pbe", b)
    g1 = dft.compute_xc_gradient(D)
    dft.set_gradient_workspace_cap(2 << 20)
    g2 = dft.compute_xc_gradient(D)
    assert np.max(np.abs(g1 - g2)) < 1e-12
    dft.set_gradient_workspace_cap(0)
    assert np.max(np.abs(dft.compute_xc_gradient(D) - g1)) < 1e-12


@pytest.mark.gpu
def test_gradient_device_entry_point():
    torch = pytest.importorskip("torch")
    import ctypes as C
    b, D, _ = fchk_case()
    dft = og.DFT("b3lyp", b)
    g_host = dft.compute_xc_gradient(D)
    dD = torch.from_numpy(np.ascontiguousarray(D.T)).cuda()
    dg = torch.zeros(9, dtype=torch.float64, device="cuda")
    de = torch.zeros(2, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = dft.ctx.lib.occ_xc_compute_xc_gradient_device(
        dft.ctx.h, dft.h, C.c_void_p(dD.data_ptr()), og.FP64, C.c_void_p(dg.data_ptr()),
        C.c_void_p(de.data_ptr()), None)
    assert rc == 0, dft.ctx.error()
    torch.cuda.synchronize()
    assert np.max(np.abs(dg.cpu().numpy().reshape(3, 3) - g_host)) < 1e-12
    assert abs(de[0].item() - dft.exchange_correlation_energy()) < 1e-12


TOL_GRAD_MIXED = 3e-5  # Ha/Bohr, tensor-core (3xTF32) gradient against the FP64 oracle


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["lda", "pbe", "b3lyp"])
def test_mixed_gradient_converged_water(method):
    b, D, _ = fchk_case()
    dft = og.DFT(method, b)
    g = dft.compute_xc_gradient(D, og.MIXED)
    P, W = dft.grid()
    g_ref = oracle.xc_gradient(b, P, W, D, method)
    assert np.max(np.abs(g - g_ref)) <= TOL_GRAD_MIXED, np.max(np.abs(g - g_ref))


@pytest.mark.gpu
@pytest.mark.parametrize("basis_name,pure,method", [("def2-svp", True, "pbe"),
                                                    ("6-31g(d,p)", False, "blyp"),
                                                    ("def2-tzvp", True, "lda")])
def test_mixed_gradient_water_cluster(basis_name, pure, method):
    from occ_gb300 import workloads as wl
    mol = wl.water_cluster(4, box=6.0, seed=3)
    b = wl.basis_for(mol, basis_name, pure)
    D = wl.random_density(b.nbf(), 20, seed=4)
    dft = og.DFT(method, b)
    g = dft.compute_xc_gradient(D, og.MIXED)
    g64 = dft.compute_xc_gradient(D, og.FP64)
    assert np.max(np.abs(g - g64)) <= TOL_GRAD_MIXED, np.max(np.abs(g - g64))
    # repeated calls reuse the resident AO values
    assert np.max(np.abs(dft.compute_xc_gradient(D, og.MIXED) - g)) < 1e-9
