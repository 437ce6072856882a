"""Unrestricted (UKS) XC build: compute_K_dft<deriv, Unrestricted>
(include/occ/dft/dft.h:192-388, src/dft/xc_potential_matrix.cpp:61-105) with
the polarised functionals.

The polarised functionals are parity unpinned at the Libxc boundary (Libxc is
not here); they are pinned structurally: at zeta = 0 they reduce to the
unpolarised ones (value and derivatives, every component), exchange obeys the
exact spin scaling, the oracle's complex-step derivatives match central
differences, and a closed-shell unrestricted density gives the restricted
build's E_xc and V_xc for both spins."""
import numpy as np
import pytest

import occ_gb300 as og
import oracle
from occ_gb300 import workloads as wl
from helpers import host_grid

IDS = [1, 7, 8, 30, 101, 106, 130, 131, 402, 475]
GGA = {101, 106, 130, 131, 402, 475}


def _points(n=12, seed=0):
    rng = np.random.default_rng(seed)
    ra = rng.uniform(1e-3, 2.0, n)
    rb = rng.uniform(1e-3, 2.0, n)
    ga = rng.normal(size=(n, 3)) * 0.4
    gb = rng.normal(size=(n, 3)) * 0.4
    return ra, rb, (ga * ga).sum(1), (ga * gb).sum(1), (gb * gb).sum(1)


@pytest.mark.parametrize("fid", IDS)
def test_polarized_reduces_to_unpolarized(fid):
    rho = np.linspace(0.01, 2.0, 9)
    sig = np.linspace(0.0, 0.5, 9)
    e0, v0, s0 = oracle.functional(fid, rho, sig)
    e, vr, vs = oracle.functional_polarized(fid, rho / 2, rho / 2, sig / 4, sig / 4, sig / 4)
    assert np.allclose(e, e0, rtol=1e-13, atol=1e-15)
    assert np.allclose(vr[:, 0], v0, rtol=1e-13, atol=1e-15)
    assert np.allclose(vr[:, 1], v0, rtol=1e-13, atol=1e-15)
    if fid in GGA:  # along s_aa = s_ab = s_bb = sigma / 4
        assert np.allclose(vs.sum(1), 4 * s0, rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("fid", [1, 101, 106])
def test_exchange_spin_scaling(fid):
    ra, rb, saa, sab, sbb = _points()
    e, _, _ = oracle.functional_polarized(fid, ra, rb, saa, sab, sbb)
    ea, _, _ = oracle.functional(fid, 2 * ra, 4 * saa)
    eb, _, _ = oracle.functional(fid, 2 * rb, 4 * sbb)
    lhs = e * (ra + rb)
    rhs = 0.5 * (ea * 2 * ra + eb * 2 * rb)
    assert np.allclose(lhs, rhs, rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("fid", IDS)
def test_polarized_derivatives_match_finite_differences(fid):
    x = list(_points(6, seed=fid))
    e, vr, vs = oracle.functional_polarized(fid, *x)
    E = lambda xs: oracle.functional_polarized(fid, *xs)[0] * (xs[0] + xs[1])
    nvar = 5 if fid in GGA else 2
    for k in range(nvar):
        h = 1e-6 * np.maximum(np.abs(x[k]), 1e-3)
        xp = [v.copy() for v in x]
        xm = [v.copy() for v in x]
        xp[k] += h
        xm[k] -= h
        fd = (E(xp) - E(xm)) / (2 * h)
        an = vr[:, k] if k < 2 else vs[:, k - 2]
        assert np.allclose(an, fd, rtol=2e-6, atol=1e-8), (k, an, fd)


def _closed_shell_case(method):
    mol = wl.water()
    b = wl.basis_for(mol, "6-31g")
    D = wl.random_density(b.nbf(), 5, seed=2)
    return b, D


@pytest.mark.parametrize("method", ["lda", "pbe", "b3lyp"])
def test_oracle_closed_shell_unrestricted_equals_restricted(method):
    b, D = _closed_shell_case(method)
    P, W = host_grid(b)
    e_r, V_r, n_r = oracle.xc_build(b, P, W, D, method)
    e_u, V_u, n_u = oracle.xc_build_unrestricted(b, P, W, np.vstack([D / 2, D / 2]), method)
    nbf = b.nbf()
    assert abs(e_u - e_r) < 1e-11
    assert np.max(np.abs(V_u[:nbf] - V_r)) < 1e-11
    assert np.max(np.abs(V_u[nbf:] - V_r)) < 1e-11
    assert abs(n_u[0] - n_r / 2) < 1e-11 and abs(n_u[1] - n_r / 2) < 1e-11


def radical_case(basis_name="def2-svp", seed=5):
    """The OH radical (doublet, 5 alpha and 4 beta electrons)."""
    mol = og.Molecule([8, 1], [[0.0, 0.0, 0.0], [0.97, 0.0, 0.0]])
    b = wl.basis_for(mol, basis_name)
    D = wl.random_density_unrestricted(b.nbf(), 5, 4, seed=seed)
    return b, D


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["lda", "svwn5", "pbe", "blyp", "b3lyp"])
def test_unrestricted_gpu_parity(method):
    b, D = radical_case()
    dft = og.DFT(method, b)
    V = dft.compute_vxc(D, og.FP64)
    P, W = dft.grid()
    e_ref, V_ref, n_ref = oracle.xc_build_unrestricted(b, P, W, D, method)
    assert V.shape == (2 * b.nbf(), b.nbf())
    assert abs(dft.exchange_correlation_energy() - e_ref) <= 1e-8
    assert np.max(np.abs(V - V_ref)) <= 1e-9
    na, nb = dft.integrated_spin_densities()
    assert abs(na - n_ref[0]) < 1e-9 and abs(nb - n_ref[1]) < 1e-9


@pytest.mark.gpu
def test_unrestricted_gpu_water_cluster_cartesian():
    mol = wl.water_cluster(3, box=5.0, seed=4)
    b = wl.basis_for(mol, "6-31g(d,p)", pure=False)
    D = wl.random_density_unrestricted(b.nbf(), 16, 14, seed=9)
    dft = og.DFT("pbe", b)
    V = dft.compute_vxc_unrestricted(D)
    P, W = dft.grid()
    e_ref, V_ref, _ = oracle.xc_build_unrestricted(b, P, W, D, "pbe")
    assert abs(dft.exchange_correlation_energy() - e_ref) <= 1e-8
    assert np.max(np.abs(V - V_ref)) <= 1e-9


@pytest.mark.gpu
def test_unrestricted_closed_shell_equals_restricted_gpu():
    b, D = _closed_shell_case("pbe")
    dft = og.DFT("pbe", b)
    V_r = dft.compute_vxc(D, og.FP64)
    e_r = dft.exchange_correlation_energy()
    V_u = dft.compute_vxc(np.vstack([D / 2, D / 2]), og.FP64)
    nbf = b.nbf()
    assert abs(dft.exchange_correlation_energy() - e_r) < 1e-11
    assert np.max(np.abs(V_u[:nbf] - V_r)) < 1e-11
    assert np.max(np.abs(V_u[nbf:] - V_r)) < 1e-11


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["lda", "pbe", "b3lyp"])
def test_unrestricted_mixed_against_oracle(method):
    """The tensor-core UKS build against the FP64 oracle, at the restricted
    mixed path's bars."""
    from helpers import TOL_E_MIXED, TOL_V_MIXED
    b, D = radical_case()
    dft = og.DFT(method, b)
    V = dft.compute_vxc(D, og.MIXED)
    P, W = dft.grid()
    e_ref, V_ref, n_ref = oracle.xc_build_unrestricted(b, P, W, D, method)
    assert abs(dft.exchange_correlation_energy() - e_ref) <= TOL_E_MIXED
    assert np.max(np.abs(V - V_ref)) <= TOL_V_MIXED
    na, nb = dft.integrated_spin_densities()
    assert abs(na - n_ref[0]) < 1e-6 and abs(nb - n_ref[1]) < 1e-6
    # the restricted build of the same molecule still works after it
    Dr = wl.random_density(b.nbf(), 4, seed=1)
    Vr = dft.compute_vxc(Dr, og.MIXED)
    e_r, V_r, _ = oracle.xc_build(b, P, W, Dr, method)
    assert abs(dft.exchange_correlation_energy() - e_r) <= TOL_E_MIXED
    assert np.max(np.abs(Vr - V_r)) <= TOL_V_MIXED


@pytest.mark.gpu
def test_unrestricted_device_entry_point():
    torch = pytest.importorskip("torch")
    import ctypes as C
    b, D = radical_case("6-31g")
    dft = og.DFT("blyp", b)
    V = dft.compute_vxc(D, og.FP64)
    dD = torch.from_numpy(np.asfortranarray(D).ravel(order="F").copy()).cuda()
    dV = torch.zeros_like(dD)
    d3 = torch.zeros(3, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = dft.ctx.lib.occ_xc_compute_vxc_unrestricted_device(
        dft.ctx.h, dft.h, C.c_void_p(dD.data_ptr()), og.FP64, C.c_void_p(dV.data_ptr()),
        C.c_void_p(d3.data_ptr()), None)
    assert rc == 0, dft.ctx.error()
    torch.cuda.synchronize()
    Vd = dV.cpu().numpy().reshape(b.nbf(), 2 * b.nbf()).T
    assert np.max(np.abs(Vd - V)) < 1e-13
    assert abs(d3[0].item() - dft.exchange_correlation_energy()) < 1e-13


# ---- the unrestricted XC gradient (accumulate_gradient_contribution_U) ------

@pytest.mark.parametrize("method", ["svwn5", "pbe", "tpss"])
def test_oracle_unrestricted_gradient_is_derivative_of_exc(method):
    """Central differences of the unrestricted E_xc over shifts of one atom's
    basis functions, grid fixed (the default lda's VWN3 spin interpolation
    is not smooth enough at this radical's zeta ~ 1 points for a 1e-4 step)."""
    from test_xc_gradient import _shifted
    b, D = radical_case("6-31g")
    P, W = host_grid(b)
    g = oracle.xc_gradient_unrestricted(b, P, W, D, method, screen=1e-14)
    h = 1e-4
    for atom in range(2):
        for axis in range(3):
            ep = oracle.xc_build_unrestricted(_shifted(b, atom, axis, h), P, W, D, method,
                                              screen=1e-14)[0]
            em = oracle.xc_build_unrestricted(_shifted(b, atom, axis, -h), P, W, D, method,
                                              screen=1e-14)[0]
            assert abs(g[atom, axis] - (ep - em) / (2 * h)) < 1e-8, (atom, axis)


@pytest.mark.parametrize("method", ["lda", "pbe", "tpss"])
def test_oracle_closed_shell_unrestricted_gradient_equals_restricted(method):
    b, D = _closed_shell_case(method)
    P, W = host_grid(b)
    gr = oracle.xc_gradient(b, P, W, D, method)
    gu = oracle.xc_gradient_unrestricted(b, P, W, np.vstack([D / 2, D / 2]), method)
    assert np.max(np.abs(gr - gu)) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["lda", "svwn5", "pbe", "blyp", "b3lyp", "tpss"])
def test_unrestricted_gradient_gpu_parity(method):
    b, D = radical_case()
    dft = og.DFT(method, b)
    g = dft.compute_xc_gradient(D)
    P, W = dft.grid()
    g_ref = oracle.xc_gradient_unrestricted(b, P, W, D, method)
    assert g.shape == (2, 3)
    assert np.max(np.abs(g - g_ref)) <= 1e-9, np.max(np.abs(g - g_ref))
    e_ref = oracle.xc_build_unrestricted(b, P, W, D, method)[0]
    assert abs(dft.exchange_correlation_energy() - e_ref) <= 1e-8


@pytest.mark.gpu
def test_unrestricted_gradient_water_cluster_and_groups():
    mol = wl.water_cluster(3, box=5.0, seed=4)
    b = wl.basis_for(mol, "6-31g(d,p)", pure=False)
    D = wl.random_density_unrestricted(b.nbf(), 15, 14, seed=9)
    dft = og.DFT("pbe", b)
    g = dft.compute_xc_gradient(D)
    P, W = dft.grid()
    g_ref = oracle.xc_gradient_unrestricted(b, P, W, D, "pbe")
    assert np.max(np.abs(g - g_ref)) <= 1e-9 * max(1.0, np.max(np.abs(g_ref)))
    dft.set_gradient_workspace_cap(2 << 20)
    assert np.max(np.abs(dft.compute_xc_gradient(D) - g)) < 1e-11
    # the tensor-core form (3xTF32 contractions) at the restricted one's bar
    gm = dft.compute_xc_gradient(D, og.MIXED)
    assert np.max(np.abs(gm - g)) <= 3e-5, np.max(np.abs(gm - g))


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["lda", "pbe", "b3lyp"])
def test_unrestricted_gradient_mixed_against_oracle(method):
    b, D = radical_case()
    dft = og.DFT(method, b)
    g = dft.compute_xc_gradient(D, og.MIXED)
    P, W = dft.grid()
    g_ref = oracle.xc_gradient_unrestricted(b, P, W, D, method)
    assert np.max(np.abs(g - g_ref)) <= 3e-5, np.max(np.abs(g - g_ref))
    e_ref = oracle.xc_build_unrestricted(b, P, W, D, method)[0]
    assert abs(dft.exchange_correlation_energy() - e_ref) <= 1e-6
    # the restricted tensor-core gradient of the same molecule after it
    Dr = 2.0 * D[:b.nbf()]
    gr = dft.compute_xc_gradient(Dr, og.MIXED)
    assert np.max(np.abs(gr - oracle.xc_gradient(b, P, W, Dr, method))) <= 3e-5


@pytest.mark.gpu
def test_unrestricted_gradient_closed_shell_equals_restricted_gpu():
    b, D = _closed_shell_case("b3lyp")
    dft = og.DFT("b3lyp", b)
    gr = dft.compute_xc_gradient(D)
    gu = dft.compute_xc_gradient(np.vstack([D / 2, D / 2]))
    assert np.max(np.abs(gr - gu)) < 1e-12
