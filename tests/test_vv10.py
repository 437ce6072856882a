"""VV10 non-local correlation (OCC's NonLocalCorrelationFunctional,
src/dft/nonlocal_correlation.cpp), the post-SCF NLC correction of the "-V"
methods.  The oracle's pair kernel is checked against a plain-Python
transcription of the reference's loop (vv10_kernel, :37-110, partners j < i
in grid order); the GPU against the oracle on OCC's NLC grid."""
import numpy as np
import pytest

import occ_gb300 as og
import oracle
from occ_gb300 import workloads as wl
from helpers import host_grid


def _python_vv10(P, W, rho, sigma, b=6.0, C=0.01):
    pi = np.pi
    kf = b * 1.5 * pi * (9 * pi) ** (-1.0 / 6)
    beta = (3.0 / (b * b)) ** 0.75 / 32.0
    rw = rho * W
    tmp = C * (sigma / rho ** 2) ** 2
    om = np.sqrt(tmp + 4 * pi / 3 * rho)
    dom_r = (0.5 * 4 * pi / 3 * rho - 2 * tmp) / om
    dom_g = tmp * rho / (sigma * om)
    kap = kf * rho ** (1 / 6)
    F, U, Wt = np.zeros(len(W)), np.zeros(len(W)), np.zeros(len(W))
    for i in range(len(W)):
        if rho[i] < 1e-8:
            continue
        k = kap[i]
        f = rw[i] / (2 * k ** 3)
        u = f * (1 / k + 1 / (2 * k))
        w = 0.0
        for j in range(i):
            if rho[j] < 1e-8:
                continue
            r2 = np.sum((P[i] - P[j]) ** 2)
            gi = r2 * om[i] + kap[i]
            gj = r2 * om[j] + kap[j]
            t = 2 * rw[j] / (gi * gj * (gi + gj))
            f += t
            t *= 1 / gi + 1 / (gi + gj)
            u += t
            w += t * r2
        F[i], U[i], Wt[i] = -1.5 * f, u, w
    exc = (beta + 0.5 * F) * W
    vr = (beta + F + 1.5 * (U * kap / 6 + Wt * dom_r)) * W
    vs = 1.5 * Wt * dom_g * W
    return exc, vr, vs


def test_oracle_vv10_kernel_matches_transcription():
    rng = np.random.default_rng(3)
    n = 60
    P = rng.normal(size=(n, 3)) * 2.0
    W = rng.uniform(0.01, 0.5, n)
    rho = np.exp(rng.uniform(-12, 0, n))
    rho[5] = 1e-9  # below the 1e-8 cut
    sigma = rho ** 2 * rng.uniform(0.0, 3.0, n)
    got = oracle.vv10_kernel(P, W, rho, sigma)
    ref = _python_vv10(P, W, rho, sigma)
    for a, r in zip(got, ref):
        assert np.allclose(a, r, rtol=1e-12, atol=1e-300)


def test_oracle_vv10_water_is_finite_and_symmetric():
    b = wl.basis_for(wl.water(), "6-31g")
    D = wl.random_density(b.nbf(), 5, seed=0)
    P, W = host_grid(b, og.GridSettings(**oracle.NLC_GRID))
    e, V = oracle.nlc_vv10(b, P, W, D)
    assert np.isfinite(e) and 0.0 < e < 1.0
    assert np.allclose(V, V.T, atol=1e-14)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["water_svp", "water4_svp", "water_631gdp_cart"])
def test_vv10_gpu_parity(case):
    if case == "water_svp":
        b = wl.basis_for(wl.water(), "def2-svp")
        D = wl.random_density(b.nbf(), 5, seed=1)
    elif case == "water4_svp":
        b = wl.basis_for(wl.water_cluster(4, box=6.0, seed=2), "def2-svp")
        D = wl.random_density(b.nbf(), 20, seed=2)
    else:
        b = wl.basis_for(wl.water(), "6-31g(d,p)", pure=False)
        D = wl.random_density(b.nbf(), 5, seed=3)
    dft = og.DFT("pbe", b)
    e, V = dft.nlc_vv10(D)
    P, W = dft.nlc_grid()
    P_h, W_h = host_grid(b, og.GridSettings(**oracle.NLC_GRID))
    assert np.array_equal(P, P_h)
    assert np.max(np.abs(W - W_h)) <= 1e-13 * np.max(np.abs(W_h))
    e_ref, V_ref = oracle.nlc_vv10(b, P_h, W_h, D)
    assert abs(e - e_ref) <= 1e-10 * max(1.0, abs(e_ref)), (e, e_ref)
    assert np.max(np.abs(V - V_ref)) <= 1e-9
    e2, none = dft.nlc_vv10(D, want_V=False)
    assert none is None and abs(e2 - e) < 1e-13
    # FP32 pair sums (compensated) against the FP64 ones
    em, Vm = dft.nlc_vv10(D, precision=og.MIXED)
    assert abs(em - e) <= 1e-8 * max(1.0, abs(e)), (em, e)
    assert np.max(np.abs(Vm - V)) <= 1e-7
