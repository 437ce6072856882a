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

METHODS = ["lda", "svwn5", "pbe", "blyp", "bpbe", "b3lyp", "b3lyp5"]


def _points(n, seed):
    rng = np.random.default_rng(seed)
    rho = 10.0 ** rng.uniform(-12, 3, n)
    kf2 = (3 * np.pi ** 2 * rho) ** (2.0 / 3.0)
    s2 = 10.0 ** rng.uniform(-8, 2, n)
    sigma = s2 * 4 * kf2 * rho ** 2
    sigma[:16] = 0.0  # stationary points of the density
    return rho, sigma


@pytest.mark.parametrize("method", METHODS)
def test_mixed_functional_matches_fp64(method):
    ctx = _context(0)
    lib = ctx.lib
    lib.occ_xc_selftest_functional.argtypes = [C.c_void_p, C.c_char_p, C.c_int, _dp, _dp, _dp,
                                               _dp]
    n = 20000
    rho, sigma = _points(n, 7)
    o64 = np.zeros(3 * n)
    om = np.zeros(3 * n)
    rc = lib.occ_xc_selftest_functional(ctx.h, method.encode(), n, _ptr(rho), _ptr(sigma),
                                        _ptr(o64), _ptr(om))
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
