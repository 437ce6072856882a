"""Serving loop: continuous batching over sessions, admission against a device
memory budget, ordering, back-pressure.  Every result served in a mixed tick
must equal the same molecule's build run alone."""
import time

import numpy as np
import pytest

import occ_gb300 as og
from occ_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

TOL_SAME = 1e-11  # only the order of FP64 atomic additions differs


def _specs():
    water = wl.water()
    return [
        ("pbe", wl.basis_for(water, "6-31g"), 5),
        ("pbe", wl.basis_for(wl.water_cluster(2, box=4.0, seed=3), "def2-svp"), 10),
        ("lda", wl.basis_for(water, "6-31g"), 5),
        ("blyp", wl.basis_for(wl.water_cluster(3, box=5.0, seed=5), "def2-svp"), 15),
        ("pbe", wl.basis_for(wl.water_cluster(4, box=5.5, seed=6), "def2-svp"), 20),
    ]


@pytest.fixture(scope="module")
def specs():
    return _specs()


def _direct(method, basis, D, precision):
    dft = og.DFT(method, basis)
    V = dft.compute_vxc(D, precision)
    return V, dft.exchange_correlation_energy(), dft.integrated_density()


@pytest.mark.parametrize("precision", [og.MIXED, og.FP64])
def test_each_result_same_alone_and_in_the_mix(specs, precision):
    srv = og.Server(precision=precision)
    try:
        srv.pause(True)  # queue everything, then serve it as one tick
        sessions, tickets, Ds = [], [], []
        for k, (method, b, nocc) in enumerate(specs):
            sid = srv.open(method, b)
            D = wl.random_density(b.nbf(), nocc, seed=200 + k)
            sessions.append(sid)
            Ds.append(D)
            tickets.append(srv.submit(sid, D))
        srv.pause(False)
        got = [srv.wait(t) for t in tickets]
        st = srv.stats()
        assert st["completed"] == len(specs) and st["failed"] == 0
        assert st["ticks"] == 1 and st["mean_batch"] == len(specs)
        for (method, b, _), D, (V, e, n) in zip(specs, Ds, got):
            Vd, ed, nd = _direct(method, b, D, precision)
            assert abs(e - ed) <= TOL_SAME
            assert abs(n - nd) <= TOL_SAME
            assert np.max(np.abs(V - Vd)) <= TOL_SAME
        for sid in sessions:
            srv.close(sid)
    finally:
        srv.shutdown()


def test_iterations_of_a_session_run_in_order(specs):
    method, b, nocc = specs[1]
    srv = og.Server()
    try:
        sid = srv.open(method, b)
        Ds = [wl.random_density(b.nbf(), nocc, seed=300 + k) for k in range(4)]
        tickets = [srv.submit(sid, D) for D in Ds]
        for D, t in zip(Ds, tickets):
            V, e, _ = srv.wait(t)
            Vd, ed, _ = _direct(method, b, D, og.MIXED)
            assert abs(e - ed) <= TOL_SAME
            assert np.max(np.abs(V - Vd)) <= TOL_SAME
        assert srv.stats()["ticks"] == 4  # one build of a session per tick
    finally:
        srv.shutdown()


def _charge(method, b):
    """Admission charge of a session: resident state plus its workspace."""
    probe = og.Server()
    try:
        info = probe.session_info(probe.open(method, b))
    finally:
        probe.shutdown()
    return info["resident_bytes"]


def test_admission_waits_for_memory(specs):
    """Room for one session, not two: the second waits until the first closes."""
    method, b, nocc = specs[4]
    charge = _charge(method, b)
    budget = 1.5 * charge
    srv = og.Server(hbm_budget_bytes=budget)
    try:
        a = srv.open(method, b)
        c = srv.open(method, b)
        D = wl.random_density(b.nbf(), nocc, seed=7)
        ta = srv.submit(a, D)
        tc = srv.submit(c, D)
        Va, ea, _ = srv.wait(ta)
        with pytest.raises(og.XCError) as ex:
            srv.wait(tc, timeout=1.0)
        assert ex.value.code == og.xc.ERR_TIMEOUT
        st = srv.stats()
        assert st["sessions_admitted"] == 1 and st["sessions_waiting"] == 1
        info = srv.session_info(a)
        # resident: grid, screening and the workspace that keeps the AO values
        assert info["admitted"] and info["mixed_workspace_bytes"] <= info["device_bytes"]
        assert info["device_bytes"] <= info["resident_bytes"]
        srv.close(a)
        Vc, ec, _ = srv.wait(tc, timeout=120.0)
        assert abs(ec - ea) <= TOL_SAME and np.max(np.abs(Vc - Va)) <= TOL_SAME
        assert srv.stats()["peak_admitted_bytes"] <= budget
    finally:
        srv.shutdown()


def test_resident_sessions_share_ticks_across_iterations(specs):
    """Two admitted sessions, three iterations each, served two per tick; the
    AO values computed on the first iteration serve the later ones."""
    method, b, nocc = specs[4]
    charge = _charge(method, b)
    srv = og.Server(hbm_budget_bytes=2.2 * charge)
    try:
        a = srv.open(method, b)
        c = srv.open(method, b)
        for it in range(3):
            D = wl.random_density(b.nbf(), nocc, seed=20 + it)
            srv.pause(True)
            ta, tc = srv.submit(a, D), srv.submit(c, D)
            srv.pause(False)
            (Va, ea, _), (Vc, ec, _) = srv.wait(ta), srv.wait(tc)
            Vd, ed, _ = _direct(method, b, D, og.MIXED)
            assert abs(ea - ed) <= TOL_SAME and abs(ec - ed) <= TOL_SAME
            assert np.max(np.abs(Va - Vd)) <= TOL_SAME and np.max(np.abs(Vc - Vd)) <= TOL_SAME
        st = srv.stats()
        assert st["ticks"] == 3 and st["mean_batch"] == 2 and st["sessions_admitted"] == 2
        assert st["peak_admitted_bytes"] <= 2.2 * charge
    finally:
        srv.shutdown()


def test_molecule_larger_than_budget_is_refused(specs):
    method, b, _ = specs[1]
    srv = og.Server(hbm_budget_bytes=1e6)
    try:
        with pytest.raises(og.XCError) as ex:
            srv.open(method, b)
        assert ex.value.code == og.xc.ERR_NOMEM
    finally:
        srv.shutdown()


def test_full_queue_returns_busy(specs):
    method, b, nocc = specs[0]
    srv = og.Server(queue_capacity=2)
    try:
        srv.pause(True)
        sid = srv.open(method, b)
        D = wl.random_density(b.nbf(), nocc, seed=1)
        t1 = srv.submit(sid, D)
        t2 = srv.submit(sid, D)
        with pytest.raises(og.XCError) as ex:
            srv.submit(sid, D)
        assert ex.value.code == og.xc.ERR_BUSY
        srv.pause(False)
        r1, r2 = srv.wait(t1), srv.wait(t2)
        assert r1[1] == pytest.approx(r2[1], abs=TOL_SAME)
    finally:
        srv.shutdown()


def test_poll_then_collect_once(specs):
    method, b, nocc = specs[0]
    srv = og.Server()
    try:
        sid = srv.open(method, b)
        t = srv.submit(sid, wl.random_density(b.nbf(), nocc, seed=2))
        deadline = time.time() + 120
        res = None
        while res is None and time.time() < deadline:
            res = srv.poll(t)
            time.sleep(0.001)
        assert res is not None
        with pytest.raises(og.XCError):
            srv.poll(t)  # a ticket is collected once
    finally:
        srv.shutdown()
