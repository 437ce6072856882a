"""Benchmark harness for the workloads beside the 32-water headline build.

alkane_graph    n-C30H62, def2-TZVP, B3LYP (local part), 15 SCF-iteration
                densities captured as one CUDA graph per precision; graph
                replays timed with CUDA events; E_xc of every iteration,
                mixed against FP64.
clusters        512 water clusters, n uniform in {1..24}, box 3.1 n^(1/3)
                Angstrom, def2-SVP, PBE, built as one batch (one launch
                sequence per sub-batch); leaf size and tile from the
                autotuner, tuned on one molecule of each of seven sizes and
                applied to the molecules nearest in size; builds/s and grid
                points/s, mixed against FP64 (at most 2 timed batches).
stream          Poisson arrivals (seeded rate) of requests of 8-20 SCF
                iterations for water clusters with n uniform in {2..48},
                def2-SVP, PBE, each iteration's density the previous one plus
                seeded symmetric noise of norm 1e-3, served through the
                serving loop (continuous batching, 150 GB budget); p50 / p99
                latency (submit to result ready) and throughput, mixed and
                FP64.
gradient        XC nuclear gradient of 32 waters, def2-SVP, PBE (the headline
                molecule), FP64 and tensor-core (mixed): gradients/s through
                the device entry point (CUDA events) and through the host one
                (D in, gradient out), parity with the oracle, the oracle's own
                time on the host cores, and the FP64 rate of the contractions.
grid            molecular grid of 32 waters (def2-SVP, 965,504 points): the
                Becke partition on the GPU against the host restatement on all
                host cores, and the whole molecule set-up (grid, leaves,
                screening, upload) that a DFT object or a served session pays.
uks             unrestricted (UKS) build of a 32-water cation radical (def2-SVP,
                PBE, 160 alpha / 159 beta orbitals), FP64 and tensor-core:
                builds/s through the device entry point (CUDA events) and the
                host one, and the mixed result against FP64.
vv10            VV10 non-local correlation of 32 waters (def2-SVP, 254,976
                NLC points): FP64 and FP32-pair-sum calls, their difference.
cosx            seminumerical (COSX) exchange matrix of an 8-water cluster
                (def2-SVP) on the for_sgx(50) grid, FP64 and with the ESP
                integrals in FP32, device and host entry points, set-up apart.

Every input is seeded synthetic data with the shapes of these workloads.
Each function returns a dict for one JSON line.
"""
import ctypes as C
import time

import numpy as np

from . import workloads as wl
from .xc import FP64, MIXED, Batch, DFT, Server, capture_scf_graph


def _pct(v, q):
    return float(np.percentile(np.asarray(v), q)) if len(v) else None


def alkane_graph(torch, steps=3, warmup=3, iterations=15, seed=0, ncarbon=30):
    mol = wl.alkane(ncarbon)
    basis = wl.basis_for(mol, "def2-tzvp")
    nbf = basis.nbf()
    nocc = (6 * ncarbon + 2 * ncarbon + 2) // 2  # electrons / 2
    D0 = wl.random_density(nbf, nocc, seed=seed)
    Ds = [wl.perturbed(D0, 1e-3, seed + 1 + k) if k else D0 for k in range(iterations)]
    t0 = time.perf_counter()
    dft = DFT("b3lyp", basis)
    setup_s = time.perf_counter() - t0
    info = dft.info()
    dD = [torch.from_numpy(np.ascontiguousarray(D.T)).cuda() for D in Ds]
    out = {"workload": f"alkane_c{ncarbon}_def2tzvp_b3lyp_graph{iterations}",
           "natoms": len(mol), "nbf": nbf, "npoints": info["npoints"],
           "flops_per_build": info["flops_per_build"], "host_setup_s": setup_s}
    stream = torch.cuda.Stream()
    excs = {}
    for prec, name in ((FP64, "fp64"), (MIXED, "mixed")):
        dV = [torch.zeros((nbf, nbf), dtype=torch.float64, device="cuda") for _ in Ds]
        dE = [torch.zeros(2, dtype=torch.float64, device="cuda") for _ in Ds]
        torch.cuda.synchronize()
        g = capture_scf_graph(dft, prec, [t.data_ptr() for t in dD], [t.data_ptr() for t in dV],
                              [t.data_ptr() for t in dE])
        for _ in range(warmup):
            g.launch(stream.cuda_stream)
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        ev[0].record(stream)
        for i in range(steps):
            g.launch(stream.cuda_stream)
            ev[i + 1].record(stream)
        torch.cuda.synchronize()
        per = [ev[i].elapsed_time(ev[i + 1]) for i in range(steps)]
        excs[name] = np.array([float(e[0].item()) for e in dE])
        out[name] = {"builds_per_s": iterations * steps / (sum(per) / 1e3),
                     "ms_per_graph": float(np.median(per)),
                     "ms_per_build": float(np.median(per)) / iterations}
        del g
    de = excs["mixed"] - excs["fp64"]
    out["max_abs_dE_xc_per_iteration"] = float(np.max(np.abs(de)))
    out["dE_xc_sum_over_iterations"] = float(np.sum(de))
    out["exc_fp64_first_last"] = [float(excs["fp64"][0]), float(excs["fp64"][-1])]
    return out


def _progress(msg):
    import sys
    sys.stderr.write(f"[{time.strftime('%H:%M:%S')}] {msg}\n")
    sys.stderr.flush()


def clusters_batch(torch, steps=2, warmup=1, nclusters=512, seed=0, autotune=True):
    rng = np.random.default_rng(seed)
    sizes = rng.integers(1, 25, nclusters)
    t0 = time.perf_counter()
    dfts, Ds, bases = [], [], []
    for i, n in enumerate(sizes):
        mol = wl.water_cluster(int(n), box=3.1 * float(n) ** (1.0 / 3.0), seed=seed + 1000 + i)
        b = wl.basis_for(mol, "def2-svp")
        bases.append(b)
        dfts.append(DFT("pbe", b))
        Ds.append(wl.random_density(b.nbf(), 5 * int(n), seed=seed + 5000 + i))
    setup_s = time.perf_counter() - t0
    _progress(f"clusters: {nclusters} molecules set up in {setup_s:.1f} s")
    # the tuner runs on one molecule of each of seven sizes; every molecule
    # takes the choice of the nearest tuned size
    tuned = {}
    t0 = time.perf_counter()
    if autotune:
        reps = (1, 4, 8, 12, 16, 20, 24)
        for i, n in enumerate(sizes):
            n = int(n)
            if n in reps and n not in tuned:
                tuned[n] = dfts[i].autotune(Ds[i], MIXED, tol_exc=1e-7)
        for i, n in enumerate(sizes):
            near = min(tuned, key=lambda r: abs(r - int(n)))
            dfts[i].apply_tuning(tuned[near])
    tune_s = time.perf_counter() - t0
    _progress(f"clusters: tuned in {tune_s:.1f} s")
    npts = sum(d.info()["npoints"] for d in dfts)
    out = {"workload": f"clusters{nclusters}_n1to24_def2svp_pbe_batch", "nclusters": nclusters,
           "total_points": int(npts), "total_atoms": int(3 * sizes.sum()),
           "host_setup_s": setup_s, "autotune_s": tune_s,
           "tuned_leaf_targets": sorted({int(t["leaf_target"]) for t in tuned.values()})}
    batch = Batch(dfts)
    for i, D in enumerate(Ds):
        batch.set_density(i, D)
    lib = batch.ctx.lib
    stream = torch.cuda.Stream()
    res = {}
    for prec, name in ((FP64, "fp64"), (MIXED, "mixed")):
        def one():
            rc = lib.occ_xc_batch_compute(batch.ctx.h, batch.h, prec,
                                          C.c_void_p(stream.cuda_stream))
            if rc != 0:
                raise RuntimeError(batch.ctx.error())
        for _ in range(warmup):
            one()
        torch.cuda.synchronize()
        _progress(f"clusters: {name} warm-up done")
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        ev[0].record(stream)
        for i in range(steps):
            one()
            ev[i + 1].record(stream)
        torch.cuda.synchronize()
        batch.check(C.c_void_p(stream.cuda_stream))
        _progress(f"clusters: {name} timed")
        per = [ev[i].elapsed_time(ev[i + 1]) for i in range(steps)]
        ms = float(np.median(per))
        res[name] = np.array([batch.result(i)[1] for i in range(nclusters)])
        out[name] = {"builds_per_s": nclusters / (ms / 1e3), "points_per_s": npts / (ms / 1e3),
                     "ms_per_batch": ms}
    de = np.abs(res["mixed"] - res["fp64"])
    out["max_abs_dE_xc"] = float(de.max())
    out["max_abs_dE_xc_per_atom"] = float(np.max(de / (3 * sizes)))
    return out


def serve_stream(precision, nreq=32, rate=10.0, seed=0, budget=150e9, sessions=None):
    """One pass of the seeded request stream through a server.  Each request
    opens its session when it arrives (grid, screening and admission inside
    the timed stream, on a pool of opener threads so that the polling loop
    keeps running), then submits its SCF iterations one after another.
    Latencies: per build (submit -> result, the server's own statistics),
    per session open, and per request to its first result (arrival -> first
    V_xc, open included).  `sessions` (basis, D0, iterations) may be passed in
    to reuse the host inputs."""
    from concurrent.futures import ThreadPoolExecutor
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, nreq)
    arrivals = np.cumsum(gaps) - gaps[0]
    if sessions is None:
        # inputs made before the clock starts: each request's basis and its
        # sequence of densities (the first a seeded guess, then perturbed by
        # seeded symmetric noise per iteration), so that the client submits
        # as fast as results come back
        sessions = []
        for i in range(nreq):
            n = int(rng.integers(2, 49))
            mol = wl.water_cluster(n, box=10.0 * (n / 32.0) ** (1.0 / 3.0), seed=seed + 100 + i)
            b = wl.basis_for(mol, "def2-svp")
            iters = int(rng.integers(8, 21))
            Ds = [wl.random_density(b.nbf(), 5 * n, seed=seed + 300 + i)]
            for it in range(1, iters):
                Ds.append(wl.perturbed(Ds[-1], 1e-3, seed + 10000 * i + it))
            sessions.append((b, Ds, iters))
    srv = Server(precision=precision, hbm_budget_bytes=budget)
    pool = ThreadPoolExecutor(max_workers=8)
    try:
        def opener(r):
            t = time.perf_counter()
            sid = srv.open("pbe", sessions[r][0])
            return sid, time.perf_counter() - t
        opening = {}  # request -> future of (session id, open seconds)
        state = {}    # request -> [iteration, ticket, D, session id]
        open_s, first_ms = [], []
        done_req, nxt, builds = 0, 0, 0
        h2d = d2h = 0
        t0 = time.perf_counter()
        while done_req < nreq:
            now = time.perf_counter() - t0
            while nxt < nreq and arrivals[nxt] <= now:
                opening[nxt] = pool.submit(opener, nxt)
                nxt += 1
            progressed = False
            for r in list(opening):
                f = opening[r]
                if not f.done():
                    continue
                sid, dt = f.result()
                open_s.append(dt)
                D0 = sessions[r][1][0]
                state[r] = [0, srv.submit(sid, D0), D0, sid]
                h2d += D0.size * 8
                del opening[r]
                progressed = True
            for r in list(state):
                it, ticket, D, sid = state[r]
                res = srv.poll(ticket)
                if res is None:
                    continue
                progressed = True
                builds += 1
                d2h += res[0].size * 8 + 16
                if it == 0:
                    first_ms.append((time.perf_counter() - t0 - arrivals[r]) * 1e3)
                if it + 1 < sessions[r][2]:
                    Dn = sessions[r][1][it + 1]
                    state[r] = [it + 1, srv.submit(sid, Dn), Dn, sid]
                    h2d += Dn.size * 8
                else:
                    srv.close(sid)
                    del state[r]
                    done_req += 1
            if not progressed:
                time.sleep(0.0002)
        wall = time.perf_counter() - t0
        st = srv.stats()
    finally:
        pool.shutdown()
        srv.shutdown()
    return {"builds": builds, "wall_s": wall, "builds_per_s": builds / wall,
            "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "max_ms": st["max_ms"],
            "open_p50_ms": float(np.percentile(open_s, 50) * 1e3),
            "open_p99_ms": float(np.percentile(open_s, 99) * 1e3),
            "first_result_p50_ms": float(np.percentile(first_ms, 50)),
            "first_result_p99_ms": float(np.percentile(first_ms, 99)),
            "mean_batch": st["mean_batch"], "ticks": st["ticks"], "failed": st["failed"],
            "peak_admitted_gb": st["peak_admitted_bytes"] / 1e9,
            "h2d_bytes_per_build": h2d / max(builds, 1),
            "d2h_bytes_per_build": d2h / max(builds, 1)}, sessions


def stream(nreq=32, rate=10.0, seed=0):
    out = {"workload": f"stream{nreq}_poisson{rate:g}_n2to48_def2svp_pbe", "requests": nreq,
           "rate_per_s": rate, "budget_gb": 150,
           "note": "sessions open at arrival inside the timed stream (open and first-result "
                   "latencies reported beside the per-build ones)"}
    m, sessions = serve_stream(MIXED, nreq, rate, seed)
    out["mixed"] = m
    f, _ = serve_stream(FP64, nreq, rate, seed, sessions=sessions)
    out["fp64"] = f
    return out


def water_latency(torch, steps=200, warmup=20, method="lda", seed=0):
    """The smallest configuration: water (O at the origin, H at (+-0.757,
    0.586, 0) Angstrom), 6-31G (13 AOs), OCC's "lda" (Slater + VWN3) on the
    default grid, D from 5 occupied columns of a seeded orthonormal matrix.
    Launch- and latency-bound: per-build latency p50 / p99 with D, V on the
    device, through the host entry point, and the oracle's time beside it."""
    import os
    import sys
    mol = wl.water()
    b = wl.basis_for(mol, "6-31g")
    D = wl.random_density(b.nbf(), 5, seed=seed)
    dft = DFT(method, b)
    info = dft.info()
    lib = dft.ctx.lib
    nbf = b.nbf()
    dD = torch.tensor(np.asfortranarray(D).ravel(order="F"), device="cuda", dtype=torch.float64)
    dV = torch.zeros(nbf * nbf, device="cuda", dtype=torch.float64)
    dE = torch.zeros(2, device="cuda", dtype=torch.float64)
    stream = torch.cuda.Stream()
    out = {"workload": f"water_631g_{method}", "nbf": nbf, "npoints": info["npoints"]}
    excs = {}
    for prec, name in ((FP64, "fp64"), (MIXED, "mixed")):
        def one():
            rc = lib.occ_xc_compute_vxc_device(dft.ctx.h, dft.h, C.c_void_p(dD.data_ptr()), prec,
                                               C.c_void_p(dV.data_ptr()),
                                               C.c_void_p(dE.data_ptr()),
                                               C.c_void_p(stream.cuda_stream))
            if rc != 0:
                raise RuntimeError(dft.ctx.error())
        for _ in range(warmup):
            one()
        torch.cuda.synchronize()
        per = []
        for _ in range(steps):
            a = torch.cuda.Event(enable_timing=True)
            z = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            one()
            z.record(stream)
            z.synchronize()
            per.append(a.elapsed_time(z))
        excs[name] = float(dE[0].item())
        # through the host entry point: D in, V and E_xc out, synchronous
        for _ in range(warmup):
            dft.compute_vxc(D, prec)
        lat = []
        for _ in range(steps):
            t = time.perf_counter()
            dft.compute_vxc(D, prec)
            lat.append((time.perf_counter() - t) * 1e3)
        out[name] = {"builds_per_s": 1e3 / float(np.mean(per)),
                     "p50_ms": float(np.percentile(per, 50)),
                     "p99_ms": float(np.percentile(per, 99)),
                     "e2e": {"value": 1e3 / float(np.mean(lat)), "unit": "builds/s",
                             "p50_ms": float(np.percentile(lat, 50)),
                             "p99_ms": float(np.percentile(lat, 99)),
                             "h2d_bytes_per_step": nbf * nbf * 8,
                             "d2h_bytes_per_step": nbf * nbf * 8 + 16}}
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "oracle"))
    import oracle
    P, W = dft.grid()
    t = time.perf_counter()
    reps = 20
    for _ in range(reps):
        e_ref, _, _ = oracle.xc_build(b, P, W, D, method)
    cpu_s = (time.perf_counter() - t) / reps
    out["dE_xc_fp64_vs_oracle"] = excs["fp64"] - e_ref
    out["dE_xc_mixed_vs_oracle"] = excs["mixed"] - e_ref
    out["cpu_baseline"] = {"value": 1.0 / cpu_s, "unit": "builds/s", "cores": os.cpu_count(),
                           "kind": "port", "sample": f"{reps} whole builds"}
    out["e2e"] = out["fp64"]["e2e"]
    return out


FP64_PEAK_TFLOPS = 1.25  # GB300 nominal dense FP64 (no measured figure)


def xc_gradient(torch, steps=5, warmup=3, waters=32, method="pbe", seed=0):
    import os
    import sys
    box = 10.0 * (waters / 32.0) ** (1.0 / 3.0)
    mol = wl.water_cluster(waters, box=box, seed=seed)
    b = wl.basis_for(mol, "def2-svp")
    D = wl.random_density(b.nbf(), 5 * waters, seed=seed)
    dft = DFT(method, b)
    info = dft.info()
    natoms = len(b.atoms())
    lib = dft.ctx.lib
    dD = torch.from_numpy(np.ascontiguousarray(D.T)).cuda()
    dg = torch.zeros(3 * natoms, dtype=torch.float64, device="cuda")
    de = torch.zeros(2, dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    flops = info["flops_per_build"] * (1.5 if info["deriv"] else 1.0)
    out = {"workload": f"water{waters}_def2svp_{method}_xc_gradient", "natoms": natoms,
           "nbf": b.nbf(), "npoints": info["npoints"], "useful_flops_per_gradient": flops}
    grads = {}
    for prec, name in ((FP64, "fp64"), (MIXED, "mixed")):
        def one():
            rc = lib.occ_xc_compute_xc_gradient_device(
                dft.ctx.h, dft.h, C.c_void_p(dD.data_ptr()), prec, C.c_void_p(dg.data_ptr()),
                C.c_void_p(de.data_ptr()), C.c_void_p(stream.cuda_stream))
            if rc != 0:
                raise RuntimeError(dft.ctx.error())
        for _ in range(warmup):
            one()
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        ev[0].record(stream)
        for i in range(steps):
            one()
            ev[i + 1].record(stream)
        torch.cuda.synchronize()
        ms = float(np.median([ev[i].elapsed_time(ev[i + 1]) for i in range(steps)]))
        g_dev = dg.cpu().numpy().reshape(natoms, 3)
        # end to end through the host entry point: D from host memory, gradient back
        t0 = time.perf_counter()
        for _ in range(steps):
            g = dft.compute_xc_gradient(D, prec)
        e2e_ms = (time.perf_counter() - t0) / steps * 1e3
        grads[name] = g
        out[name] = {"gradients_per_s": 1e3 / ms, "ms_per_gradient": ms,
                     "e2e": {"value": 1e3 / e2e_ms, "unit": "gradients/s",
                             "h2d_bytes_per_step": int(D.size * 8),
                             "d2h_bytes_per_step": int(3 * natoms * 8 + 16)},
                     "max_abs_dgrad_device_vs_host": float(np.max(np.abs(g_dev - g)))}
    out["fp64"]["roofline"] = {
        "bound": "fp64", "achieved": flops / (out["fp64"]["ms_per_gradient"] * 1e-3) / 1e12,
        "peak": FP64_PEAK_TFLOPS, "unit": "TFLOP/s",
        "frac": flops / (out["fp64"]["ms_per_gradient"] * 1e-3) / 1e12 / FP64_PEAK_TFLOPS,
        "peak_source": "nominal GB300 FP64"}
    # the oracle on the host cores, and parity
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "oracle"))
    import oracle
    P, W = dft.grid()
    t0 = time.perf_counter()
    g_ref = oracle.xc_gradient(b, P, W, D, method)
    cpu_s = time.perf_counter() - t0
    out["max_abs_dgrad_fp64_vs_oracle"] = float(np.max(np.abs(grads["fp64"] - g_ref)))
    out["max_abs_dgrad_mixed_vs_oracle"] = float(np.max(np.abs(grads["mixed"] - g_ref)))
    out["cpu_baseline"] = {"value": 1.0 / cpu_s, "unit": "gradients/s", "cores": os.cpu_count(),
                           "kind": "port", "sample": "one full gradient of the same molecule"}
    out["e2e"] = out["mixed"]["e2e"]
    return out


def grid_setup(steps=3, warmup=1, waters=32, seed=0):
    import os
    from .xc import molecular_grid
    box = 10.0 * (waters / 32.0) ** (1.0 / 3.0)
    mol = wl.water_cluster(waters, box=box, seed=seed)
    b = wl.basis_for(mol, "def2-svp")
    for _ in range(warmup):
        molecular_grid(b, device=0)
    t0 = time.perf_counter()
    for _ in range(steps):
        P_d, W_d = molecular_grid(b, device=0)
    t_dev = (time.perf_counter() - t0) / steps
    t0 = time.perf_counter()
    P_h, W_h = molecular_grid(b)
    t_host = time.perf_counter() - t0
    t0 = time.perf_counter()
    dft = DFT("pbe", b)
    t_create = time.perf_counter() - t0
    n = len(W_d)
    return {"workload": f"water{waters}_def2svp_grid_becke", "natoms": len(b.atoms()),
            "npoints": n, "points_per_s": n / t_dev, "s_per_grid": t_dev,
            "max_rel_dw_vs_host": float(np.max(np.abs(W_d - W_h)) / np.max(np.abs(W_h))),
            "positions_equal": bool(np.array_equal(P_d, P_h)),
            "molecule_create_s": t_create, "device_bytes": dft.info()["device_bytes"],
            "cpu_baseline": {"value": n / t_host, "unit": "points/s", "cores": os.cpu_count(),
                             "kind": "port", "sample": "the whole grid of the same molecule",
                             "s_per_grid": t_host}}


def uks_build(torch, steps=5, warmup=2, waters=32, seed=0):
    box = 10.0 * (waters / 32.0) ** (1.0 / 3.0)
    mol = wl.water_cluster(waters, box=box, seed=seed)
    b = wl.basis_for(mol, "def2-svp")
    nbf = b.nbf()
    D = wl.random_density_unrestricted(nbf, 5 * waters, 5 * waters - 1, seed=seed)
    dft = DFT("pbe", b)
    lib = dft.ctx.lib
    dD = torch.from_numpy(np.asfortranarray(D).ravel(order="F").copy()).cuda()
    dV = torch.zeros_like(dD)
    d3 = torch.zeros(3, dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    out = {"workload": f"water{waters}_cation_def2svp_pbe_uks", "nbf": nbf}
    res = {}
    for prec, name in ((FP64, "fp64"), (MIXED, "mixed")):
        def one():
            rc = lib.occ_xc_compute_vxc_unrestricted_device(
                dft.ctx.h, dft.h, C.c_void_p(dD.data_ptr()), prec, C.c_void_p(dV.data_ptr()),
                C.c_void_p(d3.data_ptr()), C.c_void_p(stream.cuda_stream))
            if rc != 0:
                raise RuntimeError(dft.ctx.error())
        for _ in range(warmup):
            one()
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        ev[0].record(stream)
        for i in range(steps):
            one()
            ev[i + 1].record(stream)
        torch.cuda.synchronize()
        ms = float(np.median([ev[i].elapsed_time(ev[i + 1]) for i in range(steps)]))
        t0 = time.perf_counter()
        for _ in range(steps):
            V = dft.compute_vxc(D, prec)
        e2e_ms = (time.perf_counter() - t0) / steps * 1e3
        res[name] = (dft.exchange_correlation_energy(), V)
        out[name] = {"builds_per_s": 1e3 / ms, "ms_per_build": ms,
                     "e2e": {"value": 1e3 / e2e_ms, "unit": "builds/s",
                             "h2d_bytes_per_step": int(D.size * 8),
                             "d2h_bytes_per_step": int(D.size * 8 + 8)},
                     "exc": res[name][0]}
    out["abs_dE_mixed_vs_fp64"] = abs(res["mixed"][0] - res["fp64"][0])
    out["max_abs_dV_mixed_vs_fp64"] = float(np.max(np.abs(res["mixed"][1] - res["fp64"][1])))
    out["e2e"] = out["mixed"]["e2e"]
    # the unrestricted XC gradient (host entry point), both precisions
    grads = {}
    for prec, name in ((FP64, "fp64"), (MIXED, "mixed")):
        dft.compute_xc_gradient(D, prec)
        t0 = time.perf_counter()
        for _ in range(2):
            grads[name] = dft.compute_xc_gradient(D, prec)
        out.setdefault("gradient", {})[name] = {
            "gradients_per_s": 2.0 / (time.perf_counter() - t0)}
    out["gradient"]["max_abs_dg_mixed_vs_fp64"] = float(
        np.max(np.abs(grads["mixed"] - grads["fp64"])))
    return out


def mgga_build(torch, steps=5, warmup=2, waters=32, seed=0, oracle_check=True):
    """The restricted meta-GGA (TPSS) build of the water cluster, FP64 and
    tensor-core (3xTF32) precisions, D and V resident; the full-size oracle
    build beside them (parity and the CPU baseline)."""
    import os
    import sys
    box = 10.0 * (waters / 32.0) ** (1.0 / 3.0)
    mol = wl.water_cluster(waters, box=box, seed=seed)
    b = wl.basis_for(mol, "def2-svp")
    nbf = b.nbf()
    D = wl.random_density(nbf, 5 * waters, seed=seed)
    dft = DFT("tpss", b)
    lib = dft.ctx.lib
    dD = torch.from_numpy(np.asfortranarray(D).ravel(order="F").copy()).cuda()
    dV = torch.zeros_like(dD)
    d2 = torch.zeros(2, dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    out = {"workload": f"water{waters}_def2svp_tpss", "nbf": nbf,
           "npoints": int(dft.info()["npoints"])}
    res = {}
    for prec, name in ((FP64, "fp64"), (MIXED, "mixed")):
        def one():
            rc = lib.occ_xc_compute_vxc_device(dft.ctx.h, dft.h, C.c_void_p(dD.data_ptr()),
                                               prec, C.c_void_p(dV.data_ptr()),
                                               C.c_void_p(d2.data_ptr()),
                                               C.c_void_p(stream.cuda_stream))
            if rc != 0:
                raise RuntimeError(dft.ctx.error())
        for _ in range(warmup):
            one()
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        ev[0].record(stream)
        for i in range(steps):
            one()
            ev[i + 1].record(stream)
        torch.cuda.synchronize()
        ms = float(np.median([ev[i].elapsed_time(ev[i + 1]) for i in range(steps)]))
        t0 = time.perf_counter()
        for _ in range(steps):
            V = dft.compute_vxc(D, prec)
        e2e_ms = (time.perf_counter() - t0) / steps * 1e3
        res[name] = (dft.exchange_correlation_energy(), V)
        # per-kernel device time (the library's CUDA-event profiler), two builds
        prof = _kernel_profile(dft.ctx, lambda: dft.compute_vxc(D, prec))
        out[name] = {"builds_per_s": 1e3 / ms, "ms_per_build": ms, "exc": res[name][0],
                     "kernels_ms_per_build": prof,
                     "e2e": {"value": 1e3 / e2e_ms, "unit": "builds/s",
                             "h2d_bytes_per_step": int(D.size * 8),
                             "d2h_bytes_per_step": int(D.size * 8 + 16)}}
    out["abs_dE_mixed_vs_fp64"] = abs(res["mixed"][0] - res["fp64"][0])
    out["max_abs_dV_mixed_vs_fp64"] = float(np.max(np.abs(res["mixed"][1] - res["fp64"][1])))
    out["e2e"] = out["mixed"]["e2e"]
    # the unrestricted build of the cation radical (5n alpha, 5n - 1 beta electrons)
    Du = wl.random_density_unrestricted(nbf, 5 * waters, 5 * waters - 1, seed=seed)
    dDu = torch.from_numpy(np.asfortranarray(Du).ravel(order="F").copy()).cuda()
    dVu = torch.zeros_like(dDu)
    d3 = torch.zeros(3, dtype=torch.float64, device="cuda")
    ures = {}
    for prec, name in ((FP64, "fp64"), (MIXED, "mixed")):
        def one_u():
            rc = lib.occ_xc_compute_vxc_unrestricted_device(
                dft.ctx.h, dft.h, C.c_void_p(dDu.data_ptr()), prec, C.c_void_p(dVu.data_ptr()),
                C.c_void_p(d3.data_ptr()), C.c_void_p(stream.cuda_stream))
            if rc != 0:
                raise RuntimeError(dft.ctx.error())
        nrep = steps if name == "mixed" else 2
        one_u()
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(nrep + 1)]
        ev[0].record(stream)
        for i in range(nrep):
            one_u()
            ev[i + 1].record(stream)
        torch.cuda.synchronize()
        ms = float(np.median([ev[i].elapsed_time(ev[i + 1]) for i in range(nrep)]))
        ures[name] = float(d3[0].item())
        out.setdefault("uks", {})[name] = {"builds_per_s": 1e3 / ms, "ms_per_build": ms,
                                           "exc": ures[name]}
    out["uks"]["abs_dE_mixed_vs_fp64"] = abs(ures["mixed"] - ures["fp64"])
    # the meta-GGA XC gradient (FP64), host entry point
    dft.compute_xc_gradient(D)
    t0 = time.perf_counter()
    for _ in range(2):
        g = dft.compute_xc_gradient(D)
    out["gradient_fp64"] = {"gradients_per_s": 2.0 / (time.perf_counter() - t0),
                            "max_abs_g": float(np.max(np.abs(g)))}
    # the tensor-core meta-GGA gradient, device entry point (CUDA events)
    dG = torch.zeros(3 * len(mol), dtype=torch.float64, device="cuda")
    lib.occ_xc_compute_xc_gradient_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p,
                                                      C.c_int, C.c_void_p, C.c_void_p,
                                                      C.c_void_p]

    def one_g():
        rc = lib.occ_xc_compute_xc_gradient_device(dft.ctx.h, dft.h, C.c_void_p(dD.data_ptr()),
                                                   MIXED, C.c_void_p(dG.data_ptr()),
                                                   C.c_void_p(d2.data_ptr()),
                                                   C.c_void_p(stream.cuda_stream))
        if rc != 0:
            raise RuntimeError(dft.ctx.error())
    one_g()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    ev[0].record(stream)
    for i in range(steps):
        one_g()
        ev[i + 1].record(stream)
    torch.cuda.synchronize()
    ms = float(np.median([ev[i].elapsed_time(ev[i + 1]) for i in range(steps)]))
    gm = dG.cpu().numpy().reshape(-1, 3)
    out["gradient_mixed"] = {"gradients_per_s": 1e3 / ms, "ms_per_gradient": ms,
                             "max_abs_dg_vs_fp64": float(np.max(np.abs(gm - g)))}
    if oracle_check:
        root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
        sys.path.insert(0, os.path.join(root, "oracle"))
        import oracle
        P, W = dft.grid()
        t0 = time.perf_counter()
        e_ref, V_ref, _ = oracle.xc_build(b, P, W, D, "tpss")
        t_cpu = time.perf_counter() - t0
        for name in ("fp64", "mixed"):
            out[name]["abs_dE_vs_oracle"] = abs(res[name][0] - e_ref)
            out[name]["max_abs_dV_vs_oracle"] = float(np.max(np.abs(res[name][1] - V_ref)))
        out["cpu_baseline"] = {"value": 1.0 / t_cpu, "unit": "builds/s",
                               "cores": os.cpu_count(), "kind": "port",
                               "sample": "one whole build of the same molecule"}
    return out


def vv10(steps=3, warmup=1, waters=32, seed=0):
    box = 10.0 * (waters / 32.0) ** (1.0 / 3.0)
    mol = wl.water_cluster(waters, box=box, seed=seed)
    b = wl.basis_for(mol, "def2-svp")
    D = wl.random_density(b.nbf(), 5 * waters, seed=seed)
    dft = DFT("pbe", b)
    out = {"workload": f"water{waters}_def2svp_vv10"}
    res = {}
    for prec, name in ((FP64, "fp64"), (MIXED, "mixed")):
        for _ in range(warmup):
            dft.nlc_vv10(D, precision=prec)
        t0 = time.perf_counter()
        for _ in range(steps if name == "mixed" else 1):
            e, V = dft.nlc_vv10(D, precision=prec)
        s = (time.perf_counter() - t0) / (steps if name == "mixed" else 1)
        res[name] = (e, V)
        out[name] = {"calls_per_s": 1.0 / s, "s_per_call": s, "energy": e}
    P, W = dft.nlc_grid()
    n = len(W)
    out["nlc_points"] = n
    out["pairs"] = n * (n - 1) / 2
    out["abs_dE_mixed_vs_fp64"] = abs(res["mixed"][0] - res["fp64"][0])
    out["max_abs_dV_mixed_vs_fp64"] = float(np.max(np.abs(res["mixed"][1] - res["fp64"][1])))
    return out


def _kernel_profile(ctx, call, n=2):
    """Per-kernel device time (ms per call) of n calls, from the library's
    CUDA-event profiler."""
    lib = ctx.lib
    lib.occ_xc_profile_enable.argtypes = [C.c_void_p, C.c_int]
    lib.occ_xc_profile_reset.argtypes = [C.c_void_p]
    lib.occ_xc_profile_count.argtypes = [C.c_void_p]
    lib.occ_xc_profile_entry.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_char_p),
                                         C.POINTER(C.c_double), C.POINTER(C.c_long)]
    lib.occ_xc_profile_reset(ctx.h)
    lib.occ_xc_profile_enable(ctx.h, 1)
    for _ in range(n):
        call()
    prof = {}
    for i in range(lib.occ_xc_profile_count(ctx.h)):
        kname, kms, cnt = C.c_char_p(), C.c_double(), C.c_long()
        lib.occ_xc_profile_entry(ctx.h, i, C.byref(kname), C.byref(kms), C.byref(cnt))
        prof[kname.value.decode()] = kms.value / n
    lib.occ_xc_profile_enable(ctx.h, 0)
    lib.occ_xc_profile_reset(ctx.h)
    return prof


def cosx(torch, steps=3, warmup=1, waters=8, seed=0, angular=50):
    """Seminumerical (COSX) exchange of a water cluster (def2-SVP, pure d
    shells) on the grid of GridSettings.for_sgx(angular), FP64: calls/s
    through the device entry point (CUDA events, D and K resident) and
    through the host one (D in, K out), with the set-up (grid, AO values,
    overlap projector) timed apart."""
    from .xc import GridSettings, SemiNumericalExchange
    box = 10.0 * (waters / 32.0) ** (1.0 / 3.0)
    mol = wl.water_cluster(waters, box=box, seed=seed)
    b = wl.basis_for(mol, "def2-svp")
    nbf = b.nbf()
    D = wl.random_density(nbf, 5 * waters, seed=seed)
    dft = DFT("lda", b)
    t0 = time.perf_counter()
    sgx = SemiNumericalExchange(dft, GridSettings.for_sgx(angular))
    setup_s = time.perf_counter() - t0
    dD = torch.from_numpy(np.asfortranarray(D).ravel(order="F").copy()).cuda()
    dK = torch.zeros_like(dD)
    stream = torch.cuda.Stream()
    out = {"workload": f"water{waters}_def2svp_cosx{angular}", "nbf": nbf,
           "npoints": int(sgx.grid_points()), "setup_s": setup_s}
    Ks = {}
    for prec, name in ((FP64, "fp64"), (MIXED, "mixed")):
        sgx.set_precision(prec)
        for _ in range(warmup):
            sgx.compute_K_device(dD.data_ptr(), dK.data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        ev[0].record(stream)
        for i in range(steps):
            sgx.compute_K_device(dD.data_ptr(), dK.data_ptr(), stream.cuda_stream)
            ev[i + 1].record(stream)
        torch.cuda.synchronize()
        ms = float(np.median([ev[i].elapsed_time(ev[i + 1]) for i in range(steps)]))
        t0 = time.perf_counter()
        for _ in range(steps):
            K = sgx.compute_K(D)
        e2e_s = (time.perf_counter() - t0) / steps
        Kd = dK.cpu().numpy().reshape(nbf, nbf, order="F")
        Ks[name] = K
        prof = _kernel_profile(dft.ctx, lambda: sgx.compute_K(D))
        out[name] = {"calls_per_s": 1e3 / ms, "ms_per_call": ms, "kernels_ms_per_call": prof,
                     "e2e": {"value": 1.0 / e2e_s, "unit": "calls/s",
                             "h2d_bytes_per_step": int(D.nbytes),
                             "d2h_bytes_per_step": int(K.nbytes)},
                     "host_vs_device_max_dK": float(np.abs(K - Kd).max())}
    out["max_abs_K"] = float(np.abs(Ks["fp64"]).max())
    out["max_abs_dK_mixed_vs_fp64"] = float(np.abs(Ks["mixed"] - Ks["fp64"]).max())
    out["calls_per_s"] = out["mixed"]["calls_per_s"]
    out["e2e"] = out["mixed"]["e2e"]
    return out
