"""Batches and CUDA graphs: a molecule built inside a batch, or replayed from a
captured graph, gets the result of its own direct build (include/occ/dft/dft.h
compute_vxc is one molecule per call; these are the GB300 additions)."""
import numpy as np
import pytest

import occ_gb300 as og
import oracle
from occ_gb300 import workloads as wl
from helpers import TOL_E_MIXED, TOL_V_MIXED

pytestmark = pytest.mark.gpu

# Batch vs direct build: identical blocks and arithmetic; only the order of
# the FP64 atomic additions into V_xc differs.
TOL_SAME_E = 1e-11
TOL_SAME_V = 1e-11


def _cases():
    water = wl.water()
    dimer = wl.water_cluster(2, box=4.0, seed=3)
    methane = og.Molecule([6, 1, 1, 1, 1],
                          [[0, 0, 0], [0.63, 0.63, 0.63], [-0.63, -0.63, 0.63],
                           [-0.63, 0.63, -0.63], [0.63, -0.63, -0.63]])
    specs = [(water, "6-31g", "pbe", 5), (dimer, "def2-svp", "pbe", 10),
             (water, "6-31g", "lda", 5), (methane, "def2-svp", "blyp", 5)]
    out = []
    for k, (mol, bname, method, nocc) in enumerate(specs):
        b = wl.basis_for(mol, bname)
        out.append((og.DFT(method, b), wl.random_density(b.nbf(), nocc, seed=10 + k), method, b))
    return out


@pytest.fixture(scope="module")
def cases():
    return _cases()


@pytest.mark.parametrize("precision", [og.MIXED, og.FP64])
def test_batch_matches_direct_builds(cases, precision):
    direct = []
    for dft, D, _, _ in cases:
        V = dft.compute_vxc(D, precision)
        direct.append((V, dft.exchange_correlation_energy(), dft.integrated_density()))
    batch = og.Batch([c[0] for c in cases])
    Vs, exc, nel = batch.compute_vxc([c[1] for c in cases], precision)
    for i, (V, e, n) in enumerate(direct):
        assert abs(exc[i] - e) <= TOL_SAME_E, i
        assert abs(nel[i] - n) <= TOL_SAME_E, i
        assert np.max(np.abs(Vs[i] - V)) <= TOL_SAME_V, i


def test_workspace_cap_splits_into_sub_batches(cases):
    """A cap below every molecule's workspace: each molecule its own
    sub-batch, same results."""
    direct = []
    for dft, D, _, _ in cases:
        V = dft.compute_vxc(D, og.MIXED)
        direct.append((V, dft.exchange_correlation_energy()))
    batch = og.Batch([c[0] for c in cases], workspace_cap_bytes=1.0)
    Vs, exc, _ = batch.compute_vxc([c[1] for c in cases], og.MIXED)
    for i, (V, e) in enumerate(direct):
        assert abs(exc[i] - e) <= TOL_SAME_E
        assert np.max(np.abs(Vs[i] - V)) <= TOL_SAME_V


def test_mixed_batch_against_oracle(cases):
    batch = og.Batch([c[0] for c in cases])
    Vs, exc, _ = batch.compute_vxc([c[1] for c in cases], og.MIXED)
    for i, (dft, D, method, b) in enumerate(cases):
        P, W = dft.grid()
        e_ref, V_ref, _ = oracle.xc_build(b, P, W, D, method)
        assert abs(exc[i] - e_ref) <= TOL_E_MIXED, i
        assert np.max(np.abs(Vs[i] - V_ref)) <= TOL_V_MIXED, i


def test_batch_rejects_repeated_molecule(cases):
    with pytest.raises(og.XCError):
        og.Batch([cases[0][0], cases[1][0], cases[0][0]])


@pytest.mark.parametrize("precision", [og.MIXED, og.FP64])
def test_batch_graph_replays_with_new_densities(cases, precision):
    batch = og.Batch([c[0] for c in cases])
    g = batch.capture_graph(precision)
    for seed in (0, 1):
        Ds = [wl.random_density(c[0].nbf(), 5, seed=100 * seed + i) for i, c in enumerate(cases)]
        for i, D in enumerate(Ds):
            batch.set_density(i, D)
        g.launch()
        batch.check()
        for i, (dft, _, _, _) in enumerate(cases):
            V, e, _ = batch.result(i)
            Vd = dft.compute_vxc(Ds[i], precision)
            assert abs(e - dft.exchange_correlation_energy()) <= TOL_SAME_E
            assert np.max(np.abs(V - Vd)) <= TOL_SAME_V


@pytest.mark.parametrize("precision", [og.MIXED, og.FP64])
def test_scf_graph_of_iterations(cases, precision):
    """Several consecutive builds (one per SCF iteration) in one graph."""
    torch = pytest.importorskip("torch")
    dft, _, _, _ = cases[1]
    n = dft.nbf()
    niter = 4
    Ds = [wl.random_density(n, 10, seed=50 + k) for k in range(niter)]
    dD = [torch.from_numpy(np.asfortranarray(D).T.copy()).cuda() for D in Ds]
    dV = [torch.zeros((n, n), dtype=torch.float64, device="cuda") for _ in range(niter)]
    dE = [torch.zeros(2, dtype=torch.float64, device="cuda") for _ in range(niter)]
    torch.cuda.synchronize()
    g = og.capture_scf_graph(dft, precision, [t.data_ptr() for t in dD],
                             [t.data_ptr() for t in dV], [t.data_ptr() for t in dE])
    for _ in range(2):
        g.launch()
        torch.cuda.synchronize()
        for k in range(niter):
            Vd = dft.compute_vxc(Ds[k], precision)
            assert abs(dE[k][0].item() - dft.exchange_correlation_energy()) <= TOL_SAME_E
            assert np.max(np.abs(dV[k].cpu().numpy() - Vd)) <= TOL_SAME_V


def test_persistent_cta_count_does_not_change_results(cases):
    dft, D, _, _ = cases[1]
    V0 = dft.compute_vxc(D, og.MIXED)
    e0 = dft.exchange_correlation_energy()
    try:
        for ctas in (1, 7, 64):
            og.set_persistent_ctas(ctas)
            V = dft.compute_vxc(D, og.MIXED)
            assert abs(dft.exchange_correlation_energy() - e0) <= TOL_SAME_E
            assert np.max(np.abs(V - V0)) <= TOL_SAME_V
    finally:
        og.set_persistent_ctas(0)
