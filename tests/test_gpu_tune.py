"""Build settings and the autotuner: any leaf size the tuner may choose still
matches the oracle run with the same leaves, and the tuner's choice keeps
E_xc within its tolerance of OCC's default blocking."""
import numpy as np
import pytest

import occ_gb300 as og
import oracle
from occ_gb300 import workloads as wl
from helpers import TOL_E_FP64, TOL_V_FP64, TOL_E_MIXED

pytestmark = pytest.mark.gpu


def _dimer():
    b = wl.basis_for(wl.water_cluster(2, box=4.0, seed=3), "def2-svp")
    return b, wl.random_density(b.nbf(), 10, seed=1)


@pytest.mark.parametrize("target,lmin,lmax", [(64, 16, 128), (512, 128, 1024)])
def test_leaf_sizes_match_oracle(target, lmin, lmax):
    """Leaves above 256 points exercise the multi-pass functional stage."""
    b, D = _dimer()
    dft = og.DFT("pbe", b)
    bs = og.BuildSettings(leaf_target=target, leaf_min=lmin, leaf_max=lmax)
    dft.set_build_settings(bs)
    V = dft.compute_vxc(D, og.FP64)
    P, W = dft.grid()
    e_ref, V_ref, _ = oracle.xc_build(b, P, W, D, "pbe", leaf=(target, lmin, lmax))
    assert abs(dft.exchange_correlation_energy() - e_ref) <= TOL_E_FP64
    assert np.max(np.abs(V - V_ref)) <= TOL_V_FP64
    dft.compute_vxc(D, og.MIXED)
    assert abs(dft.exchange_correlation_energy() - e_ref) <= TOL_E_MIXED


def test_autotune_keeps_energy_and_caches(tmp_path, monkeypatch):
    b, D = _dimer()
    dft = og.DFT("pbe", b)
    dft.compute_vxc(D, og.MIXED)
    e0 = dft.exchange_correlation_energy()
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("OCC_XC_TUNE_CACHE", str(cache))
    r = dft.autotune(D, og.MIXED, tol_exc=1e-7)
    assert r["from_cache"] == 0 and r["candidates"] == 6
    assert r["leaf_target"] in (64, 128, 256, 512) and r["vxc_tile_n"] in (128, 256)
    assert r["ms_per_build"] <= r["default_ms_per_build"]
    dft.compute_vxc(D, og.MIXED)
    assert abs(dft.exchange_correlation_energy() - e0) <= 1e-7 + 1e-9
    assert cache.read_text().strip()
    dft2 = og.DFT("pbe", b)
    r2 = dft2.autotune(D, og.MIXED)
    assert r2["from_cache"] == 1 and r2["leaf_target"] == r["leaf_target"]
    dft2.compute_vxc(D, og.MIXED)
    assert abs(dft2.exchange_correlation_energy() - dft.exchange_correlation_energy()) <= 1e-11


def test_bad_build_settings_rejected():
    b, _ = _dimer()
    dft = og.DFT("lda", b)
    with pytest.raises(og.XCError):
        dft.set_build_settings(og.BuildSettings(leaf_target=4096, leaf_min=32, leaf_max=8192))
