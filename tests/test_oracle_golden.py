"""CPU: the oracle and the host set-up pinned against the reference.

- collocation: oracle vs gau2grid outputs (golden fixture made from the
  reference's own gau2grid sources, tests/golden/make_golden.py)
- Lebedev rules: the library's generated rules vs the reference table
- PBE exchange: the known-answer test of tests/dft_tests.cpp:71-111
- functionals: vrho / vsigma are the derivatives of the energy density
- LYP: the closed-shell form equals the spin-resolved Miehlich form
"""
import ctypes as C
import os

import numpy as np
import pytest

import occ_gb300 as og
import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FUNCS = {"lda_x": 1, "lda_c_vwn": 7, "lda_c_vwn_rpa": 8, "lda_c_vwn_3": 30, "gga_x_pbe": 101,
         "gga_x_b88": 106, "gga_c_pbe": 130, "gga_c_lyp": 131, "b3lyp": 402, "b3lyp5": 475}
GGA = {101, 106, 130, 131, 402, 475}


@pytest.mark.parametrize("pure", [1, 0])
@pytest.mark.parametrize("l", [0, 1, 2, 3, 4])
def test_oracle_collocation_vs_gau2grid(pure, l):
    g = np.load(os.path.join(GOLDEN, "gau2grid_ref.npz"))
    key = f"{'pure' if pure else 'cart'}_l{l}"
    out = oracle.collocation(l, pure, g[key + "_exps"], g[key + "_coefs"], g[key + "_A"],
                             g[key + "_xyz"], deriv=1)
    ref = g[key + "_vals"]
    assert np.max(np.abs(out - ref)) <= 1e-13 * max(1.0, np.max(np.abs(ref)))


def test_lebedev_rules_match_reference_table():
    ref = np.load(os.path.join(GOLDEN, "lebedev_ref.npz"))
    lib = og.library()
    lib.occ_xc_lebedev.argtypes = [C.c_int, C.c_void_p]
    for key in ref.files:
        n = int(key[1:])
        R = ref[key]
        mine = np.zeros((n, 4))
        assert lib.occ_xc_lebedev(n, mine.ctypes.data) == n
        # same point set: match every reference point to its nearest point
        d = ((R[:, None, :3] - mine[None, :, :3]) ** 2).sum(-1)
        j = d.argmin(1)
        # the generated rules are numerical roots of the moment equations:
        # points agree to 1e-14, weights to 2e-14 (relative 1e-11 of the
        # smallest weight), far below the grid's integration error
        assert len(set(j)) == n, n
        assert np.sqrt(d.min(1).max()) < 1e-14, n
        assert np.abs(R[:, 3] - mine[j, 3]).max() < 2e-14, n
        assert abs(mine[:, 3].sum() - 1.0) < 1e-14


def test_lebedev_unsupported_order():
    lib = og.library()
    lib.occ_xc_lebedev.argtypes = [C.c_int, C.c_void_p]
    buf = np.zeros((400, 4))
    assert lib.occ_xc_lebedev(350, buf.ctypes.data) == 0


def test_pbe_exchange_known_answer():
    """tests/dft_tests.cpp:71-111: rho and grad rho rows, expected exc."""
    rows = np.array([
        [3.009700173159170558e-02, -6.373586084157208120e-02, -0.0, 1.865655330995227498e-02],
        [3.009700173159170558e-02, -0.0, -6.373586084157208120e-02, 1.865655330995227498e-02],
        [1.508591677559790178e-01, -0.0, -0.0, 1.303514966003518905e-01],
        [1.775122853194434636e-01, -0.0, -0.0, 7.842601108050306635e-02]])
    rho = rows[:, 0]
    sigma = (rows[:, 1:] ** 2).sum(1)
    exc, _, _ = oracle.functional(FUNCS["gga_x_pbe"], rho, sigma)
    expected = np.array([-0.27851489, -0.27851489, -0.39899553, -0.41654061])
    assert np.all(np.abs(exc - expected) <= 1e-6)


@pytest.mark.parametrize("name", list(FUNCS))
def test_functional_derivatives(name):
    fid = FUNCS[name]
    rng = np.random.default_rng(fid)
    rho = 10.0 ** rng.uniform(-4, 2, 64)
    sigma = (10.0 ** rng.uniform(-3, 1, 64)) * rho ** (8 / 3) if fid in GGA else np.zeros(64)
    e, vr, vs = oracle.functional(fid, rho, sigma)
    h = 1e-6
    ep, _, _ = oracle.functional(fid, rho * (1 + h), sigma)
    em, _, _ = oracle.functional(fid, rho * (1 - h), sigma)
    d_num = (ep * rho * (1 + h) - em * rho * (1 - h)) / (2 * h * rho)
    assert np.allclose(vr, d_num, rtol=1e-6, atol=1e-12)
    if fid in GGA:
        # a larger step in sigma: the sigma-dependent part of e can be small
        # next to the LDA part, so a tiny step drowns in cancellation
        hs = 1e-4
        sp, _, _ = oracle.functional(fid, rho, sigma * (1 + hs))
        sm, _, _ = oracle.functional(fid, rho, sigma * (1 - hs))
        ds_num = (sp - sm) * rho / (2 * hs * sigma)
        assert np.allclose(vs, ds_num, rtol=1e-6, atol=1e-12)


def test_functional_density_threshold():
    e, vr, vs = oracle.functional(FUNCS["gga_x_pbe"], np.array([1e-16, 0.0]), np.array([1e-30, 0.0]))
    assert np.all(e == 0) and np.all(vr == 0) and np.all(vs == 0)


def _lyp_spin(ra, rb, saa, sab, sbb):
    """Lee-Yang-Parr correlation, spin-resolved gradient form (Miehlich,
    Savin, Stoll, Preuss, Chem. Phys. Lett. 157, 200 (1989), eq. 2)."""
    a, b, c, d = 0.04918, 0.132, 0.2533, 0.349
    cf = 0.3 * (3 * np.pi ** 2) ** (2 / 3)
    r = ra + rb
    rm = r ** (-1 / 3)
    w = np.exp(-c * rm) / (1 + d * rm) * r ** (-11 / 3)
    de = c * rm + d * rm / (1 + d * rm)
    g = saa + 2 * sab + sbb
    t = (2 ** (11 / 3) * cf * (ra ** (8 / 3) + rb ** (8 / 3)) + (47 / 18 - 7 * de / 18) * g
         - (5 / 2 - de / 18) * (saa + sbb) - (de - 11) / 9 * (ra / r * saa + rb / r * sbb))
    return (-a * 4 / (1 + d * rm) * ra * rb / r
            - a * b * w * (ra * rb * t - 2 / 3 * r ** 2 * g + (2 / 3 * r ** 2 - ra ** 2) * sbb
                           + (2 / 3 * r ** 2 - rb ** 2) * saa))


def test_lyp_closed_shell_equals_spin_form():
    rng = np.random.default_rng(3)
    rho = 10.0 ** rng.uniform(-3, 1.5, 50)
    sigma = 10.0 ** rng.uniform(-2, 1, 50) * rho ** (8 / 3)
    e, _, _ = oracle.functional(FUNCS["gga_c_lyp"], rho, sigma)
    ref = _lyp_spin(rho / 2, rho / 2, sigma / 4, sigma / 4, sigma / 4) / rho
    assert np.allclose(e, ref, rtol=1e-12, atol=0)


def test_b3lyp_is_its_mixture():
    rng = np.random.default_rng(4)
    rho = 10.0 ** rng.uniform(-3, 1, 30)
    sigma = 10.0 ** rng.uniform(-2, 1, 30) * rho ** (8 / 3)
    parts = {k: oracle.functional(FUNCS[k], rho, sigma)[0] for k in
             ("lda_x", "gga_x_b88", "lda_c_vwn_rpa", "gga_c_lyp")}
    mix = 0.08 * parts["lda_x"] + 0.72 * parts["gga_x_b88"] + 0.19 * parts["lda_c_vwn_rpa"] + \
        0.81 * parts["gga_c_lyp"]
    assert np.allclose(oracle.functional(FUNCS["b3lyp"], rho, sigma)[0], mix, rtol=1e-13)


def test_slater_closed_form():
    rho = np.array([1e-3, 0.1, 1.0, 10.0])
    e, v, _ = oracle.functional(FUNCS["lda_x"], rho)
    cx = 0.75 * (3 / np.pi) ** (1 / 3)
    assert np.allclose(e, -cx * rho ** (1 / 3), rtol=1e-14)
    assert np.allclose(v, -4 / 3 * cx * rho ** (1 / 3), rtol=1e-14)


@pytest.mark.parametrize("pure", [1, 0])
@pytest.mark.parametrize("l", [0, 1, 2, 3, 4])
def test_oracle_second_derivatives_vs_gau2grid(pure, l):
    """AO Hessians (the XC gradient's GGA term) against the reference's gau2grid."""
    g = np.load(os.path.join(GOLDEN, "gau2grid_deriv2_ref.npz"))
    key = f"{'pure' if pure else 'cart'}_l{l}"
    out = oracle.collocation(l, pure, g[key + "_exps"], g[key + "_coefs"], g[key + "_A"],
                             g[key + "_xyz"], deriv=2)
    ref = g[key + "_vals"]
    assert np.max(np.abs(out - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref)))


@pytest.mark.parametrize("mid,parts", [(406, [(101, 0.75), (130, 1.0)]),
                                       (435, [(1, 0.5), (131, 1.0)]),
                                       (436, [(106, 0.5), (131, 1.0)])])
def test_oracle_hybrid_mixtures(mid, parts):
    """Libxc's local parts of the hybrids OCC names pbeh, bhandh and bhandhlyp
    (hyb_gga_xc_pbeh, _bhandh, _bhandhlyp) are the weighted sums of their
    components."""
    rng = np.random.default_rng(5)
    n = 64
    rho = 10.0 ** rng.uniform(-6, 2, n)
    sigma = 10.0 ** rng.uniform(-8, 1, n) * rho ** (8.0 / 3.0)
    e, vr, vs = oracle.functional(mid, rho, sigma)
    es = sum(c * oracle.functional(i, rho, sigma)[0] for i, c in parts)
    vrs = sum(c * oracle.functional(i, rho, sigma)[1] for i, c in parts)
    vss = sum(c * oracle.functional(i, rho, sigma)[2] for i, c in parts)
    assert np.allclose(e, es, rtol=1e-14, atol=0)
    assert np.allclose(vr, vrs, rtol=1e-13, atol=0)
    assert np.allclose(vs, vss, rtol=1e-13, atol=0)
