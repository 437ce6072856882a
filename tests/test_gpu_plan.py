"""The build plan made on the GPU (xc_plan.cu: Morton keys and a stable
radix sort, leaf bounding spheres, per-leaf shell screening) against the host
restatement (host/plan.cpp, selected with OCC_XC_PLAN=host): the same leaves
with the same significant-AO counts, and the same build."""
import ctypes as C

import numpy as np
import pytest

import occ_gb300 as og
from occ_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _cases():
    return [
        ("water_631g", wl.basis_for(wl.water(), "6-31g"), "lda"),
        ("waters8_def2svp", wl.basis_for(wl.water_cluster(8, box=6.3, seed=0), "def2-svp"), "pbe"),
        ("butane_def2tzvp", wl.basis_for(wl.alkane(4), "def2-tzvp"), "b3lyp"),
    ]


def _leaves(dft):
    n = dft.info()["nleaves"]
    cnt = np.zeros(n, dtype=np.int32)
    m = np.zeros(n, dtype=np.int32)
    lib = dft.ctx.lib
    lib.occ_xc_molecule_leaves.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    assert lib.occ_xc_molecule_leaves(dft.h, cnt.ctypes.data, m.ctypes.data) == 0
    return cnt, m


@pytest.mark.parametrize("case", range(3))
def test_device_plan_equals_host_plan(case, monkeypatch):
    name, b, method = _cases()[case]
    D = wl.random_density(b.nbf(), 5, seed=case)
    monkeypatch.setenv("OCC_XC_PLAN", "host")
    host = og.DFT(method, b)
    monkeypatch.delenv("OCC_XC_PLAN")
    dev = og.DFT(method, b)
    ih, idv = host.info(), dev.info()
    assert ih["npoints"] == idv["npoints"] and ih["nleaves"] == idv["nleaves"], name
    ch, mh = _leaves(host)
    cd, md = _leaves(dev)
    assert np.array_equal(ch, cd) and np.array_equal(mh, md), name
    assert ih["flops_per_build"] == idv["flops_per_build"]
    for prec in (og.FP64, og.MIXED):
        Vh = host.compute_vxc(D, prec)
        eh = host.exchange_correlation_energy()
        Vd = dev.compute_vxc(D, prec)
        ed = dev.exchange_correlation_energy()
        assert abs(eh - ed) < 1e-12 and np.max(np.abs(Vh - Vd)) < 1e-12, (name, prec)
