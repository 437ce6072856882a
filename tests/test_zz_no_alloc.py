"""The no-allocation entry point (occ_xc_compute_vxc_noalloc) against the
ordinary device entry point (occ_xc_compute_vxc_device).

occ_xc_compute_vxc_noalloc serves callers that cannot allocate device memory:
code living inside an application that owns the GPU's memory through its own
pool, or code that must never block in the allocator.  It runs the same FP64
build with its scratch in one static 64 MiB device array.  Checked here: its
results equal the device entry point's on two calls in a row (LDA, GGA and
meta-GGA), the second call leaves the device's free memory unchanged, a
molecule on another context and an oversized molecule are refused.  This
file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

import occ_gb300 as og
from helpers import TOL_E_FP64, TOL_V_FP64, water_case

pytestmark = pytest.mark.gpu


def _bind(lib):
    lib.occ_xc_compute_vxc_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.c_void_p, C.c_void_p]
    lib.occ_xc_compute_vxc_noalloc.restype = C.c_int


def _buffers(torch, D):
    nbf = D.shape[0]
    dD = torch.tensor(np.asfortranarray(D).ravel(order="F"), device="cuda", dtype=torch.float64)
    return dD, torch.zeros(nbf * nbf, device="cuda", dtype=torch.float64), \
        torch.zeros(2, device="cuda", dtype=torch.float64)


@pytest.mark.parametrize("method", ["pbe", "lda", "tpss"])
def test_noalloc_matches_device_entry_point_twice(method):
    torch = pytest.importorskip("torch")
    mol, basis, D = water_case("6-31g")
    dft = og.DFT(method, basis)
    lib = dft.ctx.lib
    _bind(lib)
    nbf = basis.nbf()
    dD, dV_ref, dE_ref = _buffers(torch, D)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        rc = lib.occ_xc_compute_vxc_device(dft.ctx.h, dft.h, C.c_void_p(dD.data_ptr()), og.FP64,
                                           C.c_void_p(dV_ref.data_ptr()),
                                           C.c_void_p(dE_ref.data_ptr()),
                                           C.c_void_p(stream.cuda_stream))
        assert rc == 0, dft.ctx.error()
        stream.synchronize()
        V_ref = dV_ref.cpu().numpy().reshape(nbf, nbf, order="F").copy()
        E_ref = float(dE_ref[0].item())
        for call in range(2):
            dV = torch.full((nbf * nbf,), 7.0, device="cuda", dtype=torch.float64)
            dE = torch.full((2,), 7.0, device="cuda", dtype=torch.float64)
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            rc = lib.occ_xc_compute_vxc_noalloc(dft.ctx.h, dft.h, C.c_void_p(dD.data_ptr()),
                                                C.c_void_p(dV.data_ptr()),
                                                C.c_void_p(dE.data_ptr()),
                                                C.c_void_p(stream.cuda_stream))
            assert rc == 0, dft.ctx.error()
            stream.synchronize()
            if call == 1:
                # the first call may load the module that holds the static
                # array; after it, a call takes no device memory
                assert torch.cuda.mem_get_info()[0] == free0
            V = dV.cpu().numpy().reshape(nbf, nbf, order="F")
            assert abs(float(dE[0].item()) - E_ref) <= TOL_E_FP64, call
            assert np.max(np.abs(V - V_ref)) <= TOL_V_FP64, call


def test_noalloc_rejects_oversized_molecule():
    torch = pytest.importorskip("torch")
    from occ_gb300 import workloads as wl
    mol = wl.water_cluster(2, box=4.0, seed=3)
    basis = wl.basis_for(mol, "def2-svp")
    D = wl.random_density(basis.nbf(), 10, seed=1)
    dft = og.DFT("pbe", basis)
    lib = dft.ctx.lib
    _bind(lib)
    dD, dV, dE = _buffers(torch, D)
    rc = lib.occ_xc_compute_vxc_noalloc(dft.ctx.h, dft.h, C.c_void_p(dD.data_ptr()),
                                        C.c_void_p(dV.data_ptr()), C.c_void_p(dE.data_ptr()),
                                        None)
    assert rc == -1
    assert "static maximum" in dft.ctx.error()


def test_noalloc_rejects_molecule_of_another_context():
    torch = pytest.importorskip("torch")
    mol, basis, D = water_case("6-31g")
    from occ_gb300.xc import _Context
    dft = og.DFT("lda", basis)
    other = _Context(0)  # a second context on the same device
    lib = dft.ctx.lib
    _bind(lib)
    dD, dV, dE = _buffers(torch, D)
    rc = lib.occ_xc_compute_vxc_noalloc(other.h, dft.h, C.c_void_p(dD.data_ptr()),
                                        C.c_void_p(dV.data_ptr()), C.c_void_p(dE.data_ptr()),
                                        None)
    assert rc == -1
    assert "another context" in other.error()
