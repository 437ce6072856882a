"""The mixed path's functional evaluator (double-float energy densities, FP32
derivatives, FP64 below rho = 1e-10) against the FP64 evaluator, point by
point, for every method, over the density and reduced-gradient ranges of a
molecular grid."""
import ctypes as C

import numpy as np
import pytest

import occ_gb300 as og
from occ_gb300.xc import _context, _dp, _ptr

pytestmark = pytest.mark.gpu

METHODS = ["lda", "svwn5", "pbe", "blyp", "bpbe", "b3lyp", "b3lyp5", "pbeh", "bhandh",
           "bhandhlyp"]


def _points(n, seed):
    rng = np.random.default_rng(seed)
    rho = 10.0 ** rng.uniform(-12, 3, n)
    kf2 = (3 * np.pi ** 2 * rho) ** (2.0 / 3.0)
    s2 = 10.0 ** rng.uniform(-8, 2, n)
    sigma = s2 * 4 * kf2 * rho ** 2
    sigma[:16] = 0.0  # stationary points of the density
    return rho, sigma


@pytest.mark.parametrize("entry", ["occ_xc_selftest_functional", "occ_xc_selftest_functional_f2"])
@pytest.mark.parametrize("method", METHODS)
def test_mixed_functional_matches_fp64(method, entry):
    """eval_xc_mixed (gradient, unrestricted builds) and eval_xc_mixed_f2
    (the restricted build's stage, inputs split by integer operations)."""
    ctx = _context(0)
    lib = ctx.lib
    fn = getattr(lib, entry)
    fn.argtypes = [C.c_void_p, C.c_char_p, C.c_int, _dp, _dp, _dp, _dp]
    n = 20000
    rho, sigma = _points(n, 7)
    o64 = np.zeros(3 * n)
    om = np.zeros(3 * n)
    rc = fn(ctx.h, method.encode(), n, _ptr(rho), _ptr(sigma), _ptr(o64), _ptr(om))
    assert rc == 0, ctx.error()
    e64, vr64, vs64 = o64[0::3], o64[1::3], o64[2::3]
    em, vrm, vsm = om[0::3], om[1::3], om[2::3]
    assert np.all(np.isfinite(om))
    # energy density: double-float accuracy, no bias
    rel = (em - e64) / (np.abs(e64) + 1e-300)
    assert np.max(np.abs(rel)) <= 1e-10
    assert abs(np.mean(rel)) <= 1e-13
    # potentials: FP32 accuracy on the scale of the point's energy density
    # (a derivative's own value can vanish where terms cancel)
    scale = np.abs(e64) + np.abs(vr64 * rho) + np.abs(vs64 * sigma) + 1e-300
    assert np.max(np.abs(vrm - vr64) * rho / scale) <= 1e-5
    assert np.max(np.abs(vsm - vs64) * sigma / scale) <= 1e-5


def _mgga_points(n, seed):
    rng = np.random.default_rng(seed)
    rho = 10.0 ** rng.uniform(-12, 3, n)
    kf2 = (3 * np.pi ** 2 * rho) ** (2.0 / 3.0)
    # s^2 up to 1e6: density tails reach large reduced gradients
    sigma = 10.0 ** rng.uniform(-8, 6, n) * 4 * kf2 * rho ** 2
    sigma[:16] = 0.0
    # tau >= tau_W = sigma / (8 rho), from one orbital (z = 1) up to 1e3 tau_W
    tau = sigma / (8 * rho) * (1 + 10.0 ** rng.uniform(-6, 3, n))
    tau[:16] = 0.3 * kf2[:16] * rho[:16]  # the uniform gas
    return rho, sigma, tau


@pytest.mark.parametrize("method", ["tpss", "mgga_x_tpss gga_c_pbe"])
def test_mgga_functional_matches_oracle(method):
    """The GPU's meta-GGA evaluators against the oracle's (complex-step
    derivatives of the spin-polarised form), point by point: the FP64 one
    tightly, the tensor-core path's (FP64 values, FP32 derivatives) at FP32
    accuracy for the derivatives."""
    import oracle
    ctx = _context(0)
    lib = ctx.lib
    lib.occ_xc_selftest_functional_mgga.argtypes = [C.c_void_p, C.c_char_p, C.c_int, _dp, _dp,
                                                    _dp, _dp, _dp]
    n = 20000
    rho, sigma, tau = _mgga_points(n, 11)
    o64 = np.zeros(4 * n)
    om = np.zeros(4 * n)
    rc = lib.occ_xc_selftest_functional_mgga(ctx.h, method.encode(), n, _ptr(rho), _ptr(sigma),
                                             _ptr(tau), _ptr(o64), _ptr(om))
    assert rc == 0, ctx.error()
    e64, vr64, vs64, vt64 = (o64[k::4] for k in range(4))
    ids = {"tpss": [202, 231], "mgga_x_tpss gga_c_pbe": [202, 130]}[method]
    er = np.zeros(n)
    vrr, vsr, vtr = np.zeros(n), np.zeros(n), np.zeros(n)
    for fid in ids:
        if fid in oracle.MGGA_IDS:
            e, a, b, c = oracle.functional_mgga(fid, rho, sigma, tau)
            vtr += c
        else:
            e, a, b = oracle.functional(fid, rho, sigma)
        er += e * rho
        vrr += a
        vsr += b
    scale = np.abs(er) + np.abs(vrr * rho) + np.abs(vsr * sigma) + np.abs(vtr * tau) + 1e-300
    assert np.all(np.isfinite(o64))
    assert np.max(np.abs(e64 - er) / scale) <= 1e-12
    # derivatives where neither the tau floor (1e-20) nor the sigma <= 8 rho
    # tau clamp acts: at a clamped point both report the derivative at the
    # clamped arguments, which is not the derivative of the energy there
    free = tau >= 1e-18
    assert np.count_nonzero(free) > 0.8 * n
    for a, b, x in ((vr64, vrr, rho), (vs64, vsr, sigma), (vt64, vtr, tau)):
        err = np.where(free, np.abs(a - b) * x / scale, 0.0)
        i = int(np.argmax(err))
        assert err[i] <= 1e-10, (i, rho[i], sigma[i], tau[i], a[i], b[i])
    # the tensor-core path's evaluator against the FP64 one
    em, vrm, vsm, vtm = (om[k::4] for k in range(4))
    assert np.all(np.isfinite(om))
    # FP64 values by other roundings (a division for the reciprocal and
    # product): the GGA evaluators' bounds, 1e-10 a point and no bias
    rel = (em - e64) / scale
    assert np.max(np.abs(rel)) <= 1e-10
    assert abs(np.mean(rel)) <= 1e-13
    for a, b, x in ((vrm, vr64, rho), (vsm, vs64, sigma), (vtm, vt64, tau)):
        err = np.where(free, np.abs(a - b) * x / scale, 0.0)
        i = int(np.argmax(err))
        assert err[i] <= 1e-5, (i, rho[i], sigma[i], tau[i], a[i], b[i])


@pytest.mark.parametrize("method", ["lda", "svwn5", "pbe", "blyp", "b3lyp"])
def test_polarised_mixed_functional_matches_fp64(method):
    """The tensor-core UKS build's polarised evaluator (FP64 values, FP32
    derivatives; FP64 where a spin density is below 1e-10) against the FP64
    one, point by point, over spin polarisations from closed shell to one
    spin channel empty."""
    ctx = _context(0)
    lib = ctx.lib
    lib.occ_xc_selftest_functional_pol.argtypes = [C.c_void_p, C.c_char_p, C.c_int, _dp, _dp,
                                                   _dp]
    n = 20000
    rng = np.random.default_rng(13)
    rho = 10.0 ** rng.uniform(-12, 3, n)
    zeta = rng.uniform(-1, 1, n)
    zeta[:200] = 1.0  # beta channel empty
    ra, rb = 0.5 * rho * (1 + zeta), 0.5 * rho * (1 - zeta)
    kf2 = (3 * np.pi ** 2 * rho) ** (2.0 / 3.0)
    ga = rng.normal(size=(n, 3)) * np.sqrt(10.0 ** rng.uniform(-8, 2, n) * kf2 * ra ** 2)[:, None]
    gb = rng.normal(size=(n, 3)) * np.sqrt(10.0 ** rng.uniform(-8, 2, n) * kf2 * rb ** 2)[:, None]
    saa, sab, sbb = (ga * ga).sum(1), (ga * gb).sum(1), (gb * gb).sum(1)
    in5 = np.concatenate([ra, rb, saa, sab, sbb])
    o64 = np.zeros(6 * n)
    om = np.zeros(6 * n)
    rc = lib.occ_xc_selftest_functional_pol(ctx.h, method.encode(), n, _ptr(in5), _ptr(o64),
                                            _ptr(om))
    assert rc == 0, ctx.error()
    assert np.all(np.isfinite(om))
    e64, em = o64[0::6], om[0::6]
    scale = (np.abs(e64) + np.abs(o64[1::6] * ra) + np.abs(o64[2::6] * rb) +
             np.abs(o64[3::6] * saa) + np.abs(o64[4::6] * sab) + np.abs(o64[5::6] * sbb) + 1e-300)
    rel = (em - e64) / scale
    assert np.max(np.abs(rel)) <= 1e-10 and abs(np.mean(rel)) <= 1e-13
    # FP32 derivatives; the spin interpolations' differences (VWN's eps_F -
    # eps_P) cost a few more bits than the unpolarised forms, hence 5e-5
    # (the whole UKS builds are held to 1e-5 in V against the oracle)
    for k, x in ((1, ra), (2, rb), (3, saa), (4, np.abs(sab)), (5, sbb)):
        err = np.abs(om[k::6] - o64[k::6]) * x / scale
        i = int(np.argmax(err))
        assert err[i] <= 5e-5, (k, i, ra[i], rb[i], om[6 * i + k], o64[6 * i + k])


def test_mgga_functional_matches_reference_known_answers():
    """Both GPU meta-GGA evaluators at the reference's TPSS known answers
    (tests/dft_tests.cpp:138-193, asserted there at 1e-6)."""
    from test_mgga import (TPSS_EXC_C, TPSS_EXC_X, TPSS_VRHO_C, TPSS_VSIGMA_C, TPSS_VTAU_C,
                           _tpss_inputs)
    ctx = _context(0)
    lib = ctx.lib
    lib.occ_xc_selftest_functional_mgga.argtypes = [C.c_void_p, C.c_char_p, C.c_int, _dp, _dp,
                                                    _dp, _dp, _dp]
    rho, sig, tau = _tpss_inputs()
    n = len(rho)
    for method, checks in (("mgga_x_tpss", ((0, TPSS_EXC_X * rho),)),
                           ("mgga_c_tpss", ((0, TPSS_EXC_C * rho), (1, TPSS_VRHO_C),
                                            (2, TPSS_VSIGMA_C), (3, TPSS_VTAU_C)))):
        o64 = np.zeros(4 * n)
        om = np.zeros(4 * n)
        rc = lib.occ_xc_selftest_functional_mgga(ctx.h, method.encode(), n, _ptr(rho),
                                                 _ptr(sig), _ptr(tau), _ptr(o64), _ptr(om))
        assert rc == 0, ctx.error()
        for k, want in checks:
            assert np.max(np.abs(o64[k::4] - want)) < 1e-8, (method, k)
            assert np.max(np.abs(om[k::4] - want)) < 1e-6, (method, k)
