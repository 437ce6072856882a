"""Meta-GGA (TPSS) XC build: compute_K_dft<2, Restricted> (include/occ/dft/
dft.h:192-388) with tau in the density (src/gto/density.cpp:73-101) and the
tau term of V_xc (src/dft/xc_potential_matrix.cpp:43-58).

Libxc, which evaluates mgga_x_tpss / mgga_c_tpss in the reference, is absent,
the oracle's TPSS is pinned against the reference's own Libxc known answers
(tests/dft_tests.cpp:138-193: exchange and correlation energies, correlation
vrho, vsigma, vtau) and by the functional's exact constraints: the uniform-gas
limit (F_x = 1, correlation = PW92), the exact hydrogen-atom exchange energy
(-0.3125 Ha, to which TPSS's constants c and e were fitted) and zero
correlation for any one-electron density.  The oracle's V_xc is pinned as the
derivative of its E_xc."""
import numpy as np
import pytest

import occ_gb300 as og
import oracle
from helpers import host_grid
from test_fchk_density import fchk_case

K2 = (3 * np.pi ** 2) ** (2 / 3)

# The reference's TPSS known answers (tests/dft_tests.cpp:138-193, Libxc's
# mgga_x_tpss / mgga_c_tpss through DensityFunctional::evaluate, asserted
# there at 1e-6): rows rho, d_x rho, d_y rho, d_z rho, laplacian, tau.
TPSS_POINTS = np.array([
    [0.06019401627252133, -0.12747174847145987, -0.0, 0.03731311973522952,
     0.09472176570942804, 0.036634279981580156],
    [0.06019401627252133, -0.0, -0.12747174847145987, 0.03731311973522952,
     0.09472176570942804, 0.036634279981580156],
    [0.30171849914696935, -0.0, -0.0, 0.26070301592021455, -2.594981941107205,
     0.02815789498408782],
    [0.3550246251878335, -0.0, -0.0, 0.15685208520532756, -6.307746108179051,
     0.008662278222335566]])
TPSS_EXC_X = np.array([-0.33175882, -0.33175882, -0.56154382, -0.59257418])
TPSS_EXC_C = np.array([-0.02276044, -0.02276044, -0.04168478, -0.04268936])
TPSS_VRHO_C = np.array([-5.57565777e-02, -5.57565777e-02, -8.00593613e-02, -8.53775165e-02])
TPSS_VSIGMA_C = np.array([3.91761083e-02, 3.91761083e-02, 1.47458233e-01, 5.51608074e-01])
TPSS_VTAU_C = np.array([1.10283011e-03, 1.10283011e-03, -3.50002323e-01, -1.56487879e+00])


def _tpss_inputs():
    """rho, sigma, tau of the known-answer points (contiguous arrays)."""
    rho = np.ascontiguousarray(TPSS_POINTS[:, 0])
    tau = np.ascontiguousarray(TPSS_POINTS[:, 5])
    return rho, (TPSS_POINTS[:, 1:4] ** 2).sum(1), tau


def test_oracle_tpss_matches_reference_known_answers():
    """The oracle's TPSS against the reference's Libxc values (1e-6 there;
    the values are printed to 8 digits, and the oracle meets them to 1e-8).
    All four points have tau = tau_W after Libxc's sigma <= 8 rho tau clamp."""
    rho, sig, tau = _tpss_inputs()
    ex = oracle.functional_mgga(202, rho, sig, tau)[0]
    ec, vr, vs, vt = oracle.functional_mgga(231, rho, sig, tau)
    for got, want in ((ex, TPSS_EXC_X), (ec, TPSS_EXC_C), (vr, TPSS_VRHO_C),
                      (vs, TPSS_VSIGMA_C), (vt, TPSS_VTAU_C)):
        assert np.max(np.abs(got - want)) < 1e-8, (got, want)


def test_tpss_uniform_gas_limit():
    rho = np.array([1e-3, 0.05, 1.0, 30.0])
    tau = 0.3 * K2 * rho ** (5 / 3)  # tau_unif, alpha = 1
    sig = np.full(4, 1e-40)
    ex = oracle.functional_mgga(202, rho, sig, tau)[0]
    assert np.allclose(ex, oracle.functional(1, rho)[0], rtol=1e-14, atol=0)
    ec = oracle.functional_mgga(231, rho, sig, tau)[0]
    assert np.allclose(ec, oracle.functional(130, rho, sig)[0], rtol=1e-14, atol=0)


def _hydrogen():
    t = np.linspace(-12.0, 4.0, 20001)
    r = np.exp(t)
    dv = 4 * np.pi * r ** 3 * (t[1] - t[0])  # 4 pi r^2 dr on a log grid
    n = np.exp(-2 * r) / np.pi
    return n, 4 * n * n, n / 2, dv  # density, |grad n|^2, tau_W, volume element


def test_tpss_hydrogen_atom_exchange_and_correlation():
    n, s, t, dv = _hydrogen()
    z = np.zeros_like(n)
    ex = oracle.functional_mgga_polarized(202, n, z, s, z, z, t, z)[0]
    ec = oracle.functional_mgga_polarized(231, n, z, s, z, z, t, z)[0]
    assert abs(np.sum(ex * n * dv) + 0.3125) < 1e-6
    assert abs(np.sum(ec * n * dv)) < 1e-12


def test_tpss_one_electron_correlation_vanishes_pointwise():
    rng = np.random.default_rng(5)
    n = 10 ** rng.uniform(-6, 1, 64)
    s = 10 ** rng.uniform(-6, 2, 64)
    t = s / (8 * n)  # a single orbital: tau = tau_W
    z = np.zeros_like(n)
    ec = oracle.functional_mgga_polarized(231, n, z, s, z, z, t, z)[0]
    assert np.max(np.abs(ec)) < 1e-14


def test_tpss_restricted_is_the_polarised_form_at_zeta_zero():
    rng = np.random.default_rng(6)
    rho = 10 ** rng.uniform(-4, 1, 32)
    sig = rho ** (8 / 3) * 10 ** rng.uniform(-3, 1, 32)
    tau = sig / (8 * rho) * (1 + 10 ** rng.uniform(-2, 1, 32))
    for fid in (202, 231):
        e, vr, vs, vt = oracle.functional_mgga(fid, rho, sig, tau)
        ep, vrp, vsp, vtp = oracle.functional_mgga_polarized(
            fid, rho / 2, rho / 2, sig / 4, sig / 4, sig / 4, tau / 2, tau / 2)
        assert np.allclose(e, ep, rtol=1e-13, atol=0)
        assert np.allclose(vr, 0.5 * vrp.sum(1), rtol=1e-10, atol=1e-14)
        assert np.allclose(vs, 0.25 * vsp.sum(1), rtol=1e-10, atol=1e-14)
        assert np.allclose(vt, 0.5 * vtp.sum(1), rtol=1e-10, atol=1e-14)


@pytest.mark.parametrize("fid", [202, 231])
def test_tpss_derivatives_match_finite_differences(fid):
    rng = np.random.default_rng(7)
    for _ in range(8):
        r = 10 ** rng.uniform(-2, 0.5)
        s = r ** (8 / 3) * 10 ** rng.uniform(-2, 0.5)
        t = s / (8 * r) * (1 + 10 ** rng.uniform(-1, 1))
        _, vr, vs, vt = oracle.functional_mgga(fid, [r], [s], [t])

        def e(R, S, T):
            return oracle.functional_mgga(fid, [R], [S], [T])[0][0] * R

        for x, v, f in ((r, vr[0], lambda h: e(r + h, s, t)),
                        (s, vs[0], lambda h: e(r, s + h, t)),
                        (t, vt[0], lambda h: e(r, s, t + h))):
            h = 1e-5 * x
            fd = (f(h) - f(-h)) / (2 * h)
            assert abs(fd - v) <= 1e-6 * max(1.0, abs(v)), (x, v, fd)


def test_oracle_tpss_potential_is_derivative_of_energy():
    """dE_xc/d eps along a symmetric dD is 2 tr(V dD) (D2 = 2 D), the same
    relation the GGA build satisfies: the tau term's 0.5 w vtau is exact."""
    b, D, _ = fchk_case()
    P, W = host_grid(b)
    rng = np.random.default_rng(1)
    E = rng.standard_normal(D.shape)
    E = E + E.T
    E *= 1e-3 / np.linalg.norm(E)
    _, V, _ = oracle.xc_build(b, P, W, D, "tpss")
    h = 1e-3
    fd = (oracle.xc_build(b, P, W, D + h * E, "tpss")[0] -
          oracle.xc_build(b, P, W, D - h * E, "tpss")[0]) / (2 * h)
    assert abs(fd - 2 * np.sum(V * E)) < 1e-9


def test_oracle_tpss_screened_matches_dense():
    b, D, _ = fchk_case()
    P, W = host_grid(b)
    es, Vs, _ = oracle.xc_build(b, P, W, D, "tpss", screen=1e-10)
    ed, Vd, _ = oracle.xc_build(b, P, W, D, "tpss", screen=0.0)
    assert abs(es - ed) < 1e-8
    assert np.max(np.abs(Vs - Vd)) < 1e-8


TOL_E = 1e-8   # Ha, FP64 E_xc against the oracle
TOL_V = 1e-9   # max |dV|, FP64


@pytest.mark.gpu
def test_tpss_converged_water_gpu_parity():
    b, D, _ = fchk_case()
    dft = og.DFT("tpss", b)
    V = dft.compute_vxc(D)
    P, W = dft.grid()
    e_ref, V_ref, n_ref = oracle.xc_build(b, P, W, D, "tpss")
    assert abs(dft.exchange_correlation_energy() - e_ref) <= TOL_E
    assert np.max(np.abs(V - V_ref)) <= TOL_V
    assert abs(dft.integrated_density() - n_ref) <= 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("basis_name,pure,method", [("def2-svp", True, "tpss"),
                                                    ("6-31g(d,p)", False, "tpss"),
                                                    ("def2-tzvp", True, "mgga_x_tpss gga_c_pbe")])
def test_tpss_water_cluster_gpu_parity(basis_name, pure, method):
    """Several 64-AO tiles, d and f shells, Cartesian and pure, and a method
    that mixes a meta-GGA with a GGA component."""
    from occ_gb300 import workloads as wl
    mol = wl.water_cluster(4, box=6.0, seed=3)
    b = wl.basis_for(mol, basis_name, pure)
    D = wl.random_density(b.nbf(), 20, seed=4)
    dft = og.DFT(method, b)
    V = dft.compute_vxc(D)
    P, W = dft.grid()
    ids = {"tpss": [202, 231], "mgga_x_tpss gga_c_pbe": [202, 130]}[method]
    e_ref, V_ref, _ = oracle.xc_build(b, P, W, D, method, func_ids=ids)
    assert abs(dft.exchange_correlation_energy() - e_ref) <= TOL_E * max(1.0, abs(e_ref))
    assert np.max(np.abs(V - V_ref)) <= TOL_V * max(1.0, np.max(np.abs(V_ref)))


TOL_E_MIXED = 1e-6  # Ha, tensor-core (3xTF32) build against FP64
TOL_V_MIXED = 1e-5


@pytest.mark.gpu
def test_tpss_mixed_converged_water():
    b, D, _ = fchk_case()
    dft = og.DFT("tpss", b)
    Vm = dft.compute_vxc(D, og.MIXED)
    em = dft.exchange_correlation_energy()
    P, W = dft.grid()
    e_ref, V_ref, _ = oracle.xc_build(b, P, W, D, "tpss")
    assert abs(em - e_ref) <= TOL_E_MIXED
    assert np.max(np.abs(Vm - V_ref)) <= TOL_V_MIXED
    # the cached AO planes serve the next build
    Vm2 = dft.compute_vxc(D, og.MIXED)
    assert np.max(np.abs(Vm2 - Vm)) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("basis_name,pure", [("def2-svp", True), ("6-31g(d,p)", False)])
def test_tpss_mixed_water_cluster(basis_name, pure):
    from occ_gb300 import workloads as wl
    mol = wl.water_cluster(4, box=6.0, seed=3)
    b = wl.basis_for(mol, basis_name, pure)
    D = wl.random_density(b.nbf(), 20, seed=4)
    dft = og.DFT("tpss", b)
    V64 = dft.compute_vxc(D, og.FP64)
    e64 = dft.exchange_correlation_energy()
    Vm = dft.compute_vxc(D, og.MIXED)
    assert abs(dft.exchange_correlation_energy() - e64) <= TOL_E_MIXED
    assert np.max(np.abs(Vm - V64)) <= TOL_V_MIXED


TOL_G_MIXED = 3e-5  # Ha/Bohr, tensor-core XC gradient (as tests/test_xc_gradient.py)


@pytest.mark.gpu
def test_tpss_unrestricted_mixed_gradient():
    """The unrestricted tensor-core meta-GGA gradient (per spin the restricted
    meta gradient's operand pairs) against the FP64 one, an open shell and a
    closed shell written as alpha = beta (equal to the restricted gradient)."""
    from occ_gb300 import workloads as wl
    mol = wl.water_cluster(3, box=5.0, seed=4)
    b = wl.basis_for(mol, "def2-svp")
    D = wl.random_density_unrestricted(b.nbf(), 15, 14, seed=9)
    dft = og.DFT("tpss", b)
    g64 = dft.compute_xc_gradient(D, og.FP64)
    gm = dft.compute_xc_gradient(D, og.MIXED)
    scale = max(1.0, np.max(np.abs(g64)))
    assert np.max(np.abs(gm - g64)) <= TOL_G_MIXED * scale, np.max(np.abs(gm - g64))
    Dr = wl.random_density(b.nbf(), 15, seed=9)
    gr = dft.compute_xc_gradient(Dr, og.MIXED)
    gu = dft.compute_xc_gradient(np.vstack([0.5 * Dr, 0.5 * Dr]), og.MIXED)
    assert np.max(np.abs(gu - gr)) <= TOL_G_MIXED * max(1.0, np.max(np.abs(gr)))


@pytest.mark.gpu
def test_tpss_mixed_gradient_converged_water():
    """The tensor-core meta-GGA gradient (tau term as three operand pairs of
    the V_xc kernel per direction) against the oracle."""
    b, D, _ = fchk_case()
    dft = og.DFT("tpss", b)
    g = dft.compute_xc_gradient(D, og.MIXED)
    P, W = dft.grid()
    g_ref = oracle.xc_gradient(b, P, W, D, "tpss")
    assert np.max(np.abs(g - g_ref)) <= TOL_G_MIXED, np.max(np.abs(g - g_ref))
    e_ref = oracle.xc_build(b, P, W, D, "tpss")[0]
    assert abs(dft.exchange_correlation_energy() - e_ref) <= TOL_E_MIXED
    # the meta build on the same molecule (its planes share the workspace)
    Vm = dft.compute_vxc(D, og.MIXED)
    _, V_ref, _ = oracle.xc_build(b, P, W, D, "tpss")
    assert np.max(np.abs(Vm - V_ref)) <= TOL_V_MIXED
    g2 = dft.compute_xc_gradient(D, og.MIXED)
    assert np.max(np.abs(g2 - g)) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("basis_name,pure", [("def2-svp", True), ("6-31g(d,p)", False)])
def test_tpss_mixed_gradient_water_cluster(basis_name, pure):
    from occ_gb300 import workloads as wl
    mol = wl.water_cluster(4, box=6.0, seed=3)
    b = wl.basis_for(mol, basis_name, pure)
    D = wl.random_density(b.nbf(), 20, seed=4)
    dft = og.DFT("tpss", b)
    g64 = dft.compute_xc_gradient(D, og.FP64)
    gm = dft.compute_xc_gradient(D, og.MIXED)
    scale = max(1.0, np.max(np.abs(g64)))
    assert np.max(np.abs(gm - g64)) <= TOL_G_MIXED * scale, np.max(np.abs(gm - g64))


@pytest.mark.gpu
def test_tpss_noalloc_entry_point():
    torch = pytest.importorskip("torch")
    import ctypes as C
    b, D, _ = fchk_case()
    dft = og.DFT("tpss", b)
    V = dft.compute_vxc(D)
    dD = torch.from_numpy(np.ascontiguousarray(D.T)).cuda()
    dV = torch.zeros_like(dD)
    de = torch.zeros(2, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = dft.ctx.lib.occ_xc_compute_vxc_noalloc(dft.ctx.h, dft.h, C.c_void_p(dD.data_ptr()),
                                               C.c_void_p(dV.data_ptr()),
                                               C.c_void_p(de.data_ptr()), None)
    assert rc == 0, dft.ctx.error()
    torch.cuda.synchronize()
    assert np.max(np.abs(dV.cpu().numpy().T - V)) < 1e-12
    assert abs(de[0].item() - dft.exchange_correlation_energy()) < 1e-12


# ---- unrestricted meta-GGA (compute_K_dft<2, Unrestricted>) -----------------

def test_oracle_tpss_closed_shell_unrestricted_equals_restricted():
    from test_uks import _closed_shell_case
    b, D = _closed_shell_case("tpss")
    P, W = host_grid(b)
    e_r, V_r, _ = oracle.xc_build(b, P, W, D, "tpss")
    e_u, V_u, _ = oracle.xc_build_unrestricted(b, P, W, np.vstack([D / 2, D / 2]), "tpss")
    nbf = b.nbf()
    assert abs(e_u - e_r) < 1e-11
    assert np.max(np.abs(V_u[:nbf] - V_r)) < 1e-11
    assert np.max(np.abs(V_u[nbf:] - V_r)) < 1e-11


def test_oracle_tpss_unrestricted_potential_is_derivative_of_energy():
    from test_uks import radical_case
    b, D = radical_case()
    P, W = host_grid(b)
    rng = np.random.default_rng(2)
    nbf = b.nbf()
    E = rng.standard_normal((2 * nbf, nbf))
    E[:nbf] += E[:nbf].T
    E[nbf:] += E[nbf:].T
    E *= 1e-3 / np.linalg.norm(E)
    _, V, _ = oracle.xc_build_unrestricted(b, P, W, D, "tpss")
    h = 1e-3
    fd = (oracle.xc_build_unrestricted(b, P, W, D + h * E, "tpss")[0] -
          oracle.xc_build_unrestricted(b, P, W, D - h * E, "tpss")[0]) / (2 * h)
    assert abs(fd - 2 * np.sum(V * E)) < 1e-9


@pytest.mark.gpu
def test_tpss_unrestricted_gpu_parity():
    from test_uks import radical_case
    b, D = radical_case()
    dft = og.DFT("tpss", b)
    V = dft.compute_vxc(D, og.FP64)
    P, W = dft.grid()
    e_ref, V_ref, n_ref = oracle.xc_build_unrestricted(b, P, W, D, "tpss")
    assert V.shape == (2 * b.nbf(), b.nbf())
    assert abs(dft.exchange_correlation_energy() - e_ref) <= TOL_E
    assert np.max(np.abs(V - V_ref)) <= TOL_V
    na, nb = dft.integrated_spin_densities()
    assert abs(na - n_ref[0]) < 1e-9 and abs(nb - n_ref[1]) < 1e-9


@pytest.mark.gpu
def test_tpss_unrestricted_gpu_water_cluster():
    from occ_gb300 import workloads as wl
    mol = wl.water_cluster(3, box=5.0, seed=4)
    b = wl.basis_for(mol, "def2-svp")
    D = wl.random_density_unrestricted(b.nbf(), 15, 14, seed=9)
    dft = og.DFT("tpss", b)
    V = dft.compute_vxc(D)
    P, W = dft.grid()
    e_ref, V_ref, _ = oracle.xc_build_unrestricted(b, P, W, D, "tpss")
    assert abs(dft.exchange_correlation_energy() - e_ref) <= TOL_E * max(1.0, abs(e_ref))
    assert np.max(np.abs(V - V_ref)) <= TOL_V * max(1.0, np.max(np.abs(V_ref)))


@pytest.mark.gpu
def test_tpss_unrestricted_closed_shell_equals_restricted_gpu():
    from test_uks import _closed_shell_case
    b, D = _closed_shell_case("tpss")
    dft = og.DFT("tpss", b)
    V_r = dft.compute_vxc(D, og.FP64)
    e_r = dft.exchange_correlation_energy()
    V_u = dft.compute_vxc(np.vstack([D / 2, D / 2]), og.FP64)
    nbf = b.nbf()
    assert abs(dft.exchange_correlation_energy() - e_r) < 1e-11
    assert np.max(np.abs(V_u[:nbf] - V_r)) < 1e-11
    assert np.max(np.abs(V_u[nbf:] - V_r)) < 1e-11


@pytest.mark.gpu
def test_tpss_unrestricted_mixed_against_oracle():
    from test_uks import radical_case
    b, D = radical_case()
    dft = og.DFT("tpss", b)
    V = dft.compute_vxc(D, og.MIXED)
    P, W = dft.grid()
    e_ref, V_ref, n_ref = oracle.xc_build_unrestricted(b, P, W, D, "tpss")
    assert abs(dft.exchange_correlation_energy() - e_ref) <= TOL_E_MIXED
    assert np.max(np.abs(V - V_ref)) <= TOL_V_MIXED
    na, nb = dft.integrated_spin_densities()
    assert abs(na - n_ref[0]) < 1e-6 and abs(nb - n_ref[1]) < 1e-6
    # the restricted tensor-core meta build of the same molecule after it
    Dr = np.vstack([D[:b.nbf()], D[b.nbf():]])[:b.nbf()] * 2.0
    Vr = dft.compute_vxc(Dr, og.MIXED)
    e_r, V_r, _ = oracle.xc_build(b, P, W, Dr, "tpss")
    assert abs(dft.exchange_correlation_energy() - e_r) <= TOL_E_MIXED
    assert np.max(np.abs(Vr - V_r)) <= TOL_V_MIXED


@pytest.mark.gpu
def test_tpss_unrestricted_mixed_water_cluster():
    from occ_gb300 import workloads as wl
    mol = wl.water_cluster(3, box=5.0, seed=4)
    b = wl.basis_for(mol, "def2-svp")
    D = wl.random_density_unrestricted(b.nbf(), 15, 14, seed=9)
    dft = og.DFT("tpss", b)
    V64 = dft.compute_vxc(D, og.FP64)
    e64 = dft.exchange_correlation_energy()
    Vm = dft.compute_vxc(D, og.MIXED)
    assert abs(dft.exchange_correlation_energy() - e64) <= TOL_E_MIXED
    assert np.max(np.abs(Vm - V64)) <= TOL_V_MIXED


# ---- meta-GGA XC gradient (accumulate_gradient_contribution_R<2>) ----------

def test_oracle_tpss_gradient_is_derivative_of_exc():
    """The reference's tau term (bra-side second derivatives, the ket side
    through the factor 2 of the distribution) is the derivative of E_xc."""
    from test_xc_gradient import _shifted
    b, D, _ = fchk_case()
    P, W = host_grid(b)
    g = oracle.xc_gradient(b, P, W, D, "tpss", screen=1e-14)
    h = 1e-4
    for atom in range(3):
        for axis in range(3):
            ep = oracle.xc_build(_shifted(b, atom, axis, h), P, W, D, "tpss", screen=1e-14)[0]
            em = oracle.xc_build(_shifted(b, atom, axis, -h), P, W, D, "tpss", screen=1e-14)[0]
            assert abs(g[atom, axis] - (ep - em) / (2 * h)) < 1e-7, (atom, axis)


@pytest.mark.gpu
def test_tpss_gradient_gpu_parity():
    b, D, _ = fchk_case()
    dft = og.DFT("tpss", b)
    g = dft.compute_xc_gradient(D)
    P, W = dft.grid()
    g_ref = oracle.xc_gradient(b, P, W, D, "tpss")
    assert np.max(np.abs(g - g_ref)) <= 1e-9, np.max(np.abs(g - g_ref))
    e_ref = oracle.xc_build(b, P, W, D, "tpss")[0]
    assert abs(dft.exchange_correlation_energy() - e_ref) <= 1e-8


@pytest.mark.gpu
def test_tpss_gradient_water_cluster_gpu_parity():
    from occ_gb300 import workloads as wl
    mol = wl.water_cluster(4, box=6.0, seed=3)
    b = wl.basis_for(mol, "def2-svp")
    D = wl.random_density(b.nbf(), 20, seed=4)
    dft = og.DFT("tpss", b)
    g = dft.compute_xc_gradient(D)
    P, W = dft.grid()
    g_ref = oracle.xc_gradient(b, P, W, D, "tpss")
    scale = max(1.0, np.max(np.abs(g_ref)))
    assert np.max(np.abs(g - g_ref)) <= 1e-9 * scale, np.max(np.abs(g - g_ref))
    # a small workspace cap: many leaf groups, the same gradient
    dft.set_gradient_workspace_cap(2 << 20)
    assert np.max(np.abs(dft.compute_xc_gradient(D) - g)) < 1e-11


@pytest.mark.gpu
def test_tpss_in_batches_and_the_server():
    """FP64 batches and an FP64 server build meta-GGA molecules with the rest;
    the tensor-core batch and server refuse them with a message."""
    from occ_gb300 import workloads as wl
    water = wl.water()
    b1 = wl.basis_for(water, "6-31g")
    b2 = wl.basis_for(wl.water_cluster(2, box=4.0, seed=3), "def2-svp")
    cases = [(og.DFT("tpss", b1), wl.random_density(b1.nbf(), 5, seed=31)),
             (og.DFT("pbe", b2), wl.random_density(b2.nbf(), 10, seed=32))]
    direct = []
    for dft, D in cases:
        direct.append((dft.compute_vxc(D), dft.exchange_correlation_energy()))
    batch = og.Batch([c[0] for c in cases])
    Vs, exc, _ = batch.compute_vxc([c[1] for c in cases], og.FP64)
    for i, (V, e) in enumerate(direct):
        assert abs(exc[i] - e) <= 1e-11
        assert np.max(np.abs(Vs[i] - V)) <= 1e-11
    with pytest.raises(og.XCError, match="meta-GGA"):
        batch.compute_vxc([c[1] for c in cases], og.MIXED)
    srv = og.Server(precision=og.FP64)
    try:
        sid = srv.open("tpss", b1)
        V, e, _ = srv.wait(srv.submit(sid, cases[0][1]))
        assert abs(e - direct[0][1]) <= 1e-11
        assert np.max(np.abs(V - direct[0][0])) <= 1e-11
        srv.close(sid)
    finally:
        srv.shutdown()
    srv = og.Server(precision=og.MIXED)
    try:
        with pytest.raises(og.XCError, match="meta-GGA"):
            srv.open("tpss", b1)
    finally:
        srv.shutdown()
