#!/usr/bin/env python
"""Benchmark of the GB300 XC build.

Workload (one "step" = one XC build: D in -> V_xc, E_xc out, grid, weights
and screening already resident): a 32-water cluster (centres uniform in a
seeded 10 Angstrom cube, O-O >= 2.6 Angstrom, random orientations),
def2-SVP (768 pure AOs), PBE, OCC's default grid, mo.D = C C^T with 160
occupied columns of a seeded random orthonormal matrix.  Synthetic inputs
with the benchmark configuration's shapes (no dataset is involved).

value    builds/s of the headline precision with D, V on the device
e2e      builds/s through the public C ABI call (occ_xc_compute_vxc) with
         pinned host buffers, H2D of D and D2H of V and E_xc inside the timed
         region
Both precisions (plain FP64 and mixed) are timed back to back on the same
GPU and their E_xc difference is reported.

--impl reference times the CPU restatement of the reference algorithm
(oracle/) on the host cores instead; the reference itself (OCC) cannot be
built here (its dependencies are fetched over the network at configure time).
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "water32_def2svp_pbe"
METRIC = "XC builds/s & p50/p99 ms, mixed vs FP64 on same GPU at |dE_xc|<=1e-6 Ha"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--waters", type=int, default=32,
                    help="cluster size (32 is the benchmark; smaller only for profiling)")
    ap.add_argument("--ctas", type=int, default=0,
                    help="CTAs of the persistent tensor-core kernels (0: one per SM)")
    ap.add_argument("--workload", default="water32",
                    choices=["water32", "water", "alkane", "clusters", "stream", "gradient", "grid",
                             "uks", "vv10", "mgga", "cosx"],
                    help="water32: the headline build (default); water: one water molecule, "
                         "6-31G, LDA (latency-bound); alkane: C30H62 def2-TZVP "
                         "B3LYP, 15 iterations as one CUDA graph; clusters: 512 clusters "
                         "as one batch; stream: served Poisson request stream; gradient: "
                         "the XC nuclear gradient of the water32 molecule; grid: its molecular "
                         "grid with the Becke partition on the GPU; uks: an unrestricted FP64 "
                         "build of its cation radical; vv10: its VV10 non-local correlation; "
                         "mgga: its meta-GGA (TPSS) build; cosx: seminumerical exchange of "
                         "an 8-water cluster (--waters) on the for_sgx(50) grid, FP64")
    ap.add_argument("--clusters", type=int, default=512)
    ap.add_argument("--requests", type=int, default=32)
    ap.add_argument("--rate", type=float, default=10.0, help="stream arrivals per second")
    return ap.parse_args()


def run_workload(args):
    """The non-headline workloads (occ_gb300/bench_workloads.py), one JSON line."""
    import torch
    from occ_gb300 import bench_workloads as bw
    torch.cuda.set_device(0)
    with ClockSampler(0) as cs:
        if args.workload == "alkane":
            args.steps = min(args.steps, 3)  # graphs of 15 builds; FP64 takes seconds
            r = bw.alkane_graph(torch, steps=args.steps, warmup=args.warmup)
        elif args.workload == "clusters":
            args.steps, args.warmup = min(args.steps, 2), min(args.warmup, 1)  # FP64: ~20 s a batch
            r = bw.clusters_batch(torch, steps=args.steps, warmup=args.warmup,
                                  nclusters=args.clusters)
        elif args.workload == "gradient":
            r = bw.xc_gradient(torch, steps=args.steps, warmup=args.warmup, waters=args.waters)
        elif args.workload == "grid":
            r = bw.grid_setup(steps=args.steps, warmup=args.warmup, waters=args.waters)
        elif args.workload == "uks":
            r = bw.uks_build(torch, steps=args.steps, warmup=args.warmup, waters=args.waters)
        elif args.workload == "vv10":
            r = bw.vv10(steps=args.steps, warmup=args.warmup, waters=args.waters)
        elif args.workload == "mgga":
            r = bw.mgga_build(torch, steps=args.steps, warmup=args.warmup, waters=args.waters)
        elif args.workload == "cosx":
            r = bw.cosx(torch, steps=max(1, min(args.steps, 5)), warmup=1,
                        waters=8 if args.waters == 32 else args.waters)
        elif args.workload == "water":
            r = bw.water_latency(torch, steps=max(args.steps, 100), warmup=max(args.warmup, 10))
        else:
            r = bw.stream(nreq=args.requests, rate=args.rate)
    if args.workload in ("uks", "vv10"):
        unit = "builds/s" if args.workload == "uks" else "calls/s"
        value = r["mixed"]["builds_per_s"] if args.workload == "uks" else r["mixed"]["calls_per_s"]
        line = {"metric": ("UKS XC builds/s (tensor-core 3xTF32, FP64 beside it)"
                           if args.workload == "uks"
                           else "VV10 non-local correlation calls/s (FP32 pair sums)"),
                "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
                "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "tf32x3+f64" if args.workload == "uks" else "f32+f64",
                "data": "synthetic", "config": {"workload": r.pop("workload")},
                "clocks": cs.summary()}
        line.update(r)
        print(json.dumps(line))
        return
    if args.workload == "mgga":
        line = {"metric": "meta-GGA (TPSS) XC builds/s (tensor-core 3xTF32, FP64 beside it)",
                "value": r["mixed"]["builds_per_s"], "unit": "builds/s", "n_gpus": 1,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "tf32x3+f64",
                "data": "synthetic", "config": {"workload": r.pop("workload")},
                "clocks": cs.summary()}
        line.update(r)
        print(json.dumps(line))
        return
    if args.workload == "cosx":
        line = {"metric": "seminumerical (COSX) exchange matrices/s (ESP integrals in FP32, "
                          "FP64 beside it)",
                "value": r.pop("calls_per_s"), "unit": "calls/s", "n_gpus": 1,
                "steps": max(1, min(args.steps, 5)), "warmup": 1, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
                "data": "synthetic", "config": {"workload": r.pop("workload")},
                "clocks": cs.summary()}
        line.update(r)
        print(json.dumps(line))
        return
    if args.workload == "grid":
        line = {"metric": "molecular grid points/s (Becke partition)",
                "value": r.pop("points_per_s"), "unit": "points/s", "n_gpus": 1,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
                "data": "synthetic", "config": {"workload": r.pop("workload")},
                "clocks": cs.summary()}
        line.update(r)
        print(json.dumps(line))
        return
    if args.workload == "gradient":
        line = {"metric": "XC nuclear gradients/s (tensor-core 3xTF32, FP64 beside it)",
                "value": r["mixed"]["gradients_per_s"],
                "unit": "gradients/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "tf32x3+f64",
                "data": "synthetic", "config": {"workload": r.pop("workload")},
                "clocks": cs.summary()}
        line.update(r)
        print(json.dumps(line))
        return
    m = r["mixed"]
    line = {"metric": METRIC, "value": m["builds_per_s"], "unit": "builds/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "tf32x3+f64", "data": "synthetic",
            "config": {"workload": r.pop("workload")}, "clocks": cs.summary()}
    line.update(r)
    print(json.dumps(line))


def make_workload(seed=0, waters=32):
    """n rigid waters in a cube of side 10 (32/n)^(-1/3) Angstrom (the same
    density as the 32-water benchmark), def2-SVP, 5 occupied orbitals per
    water."""
    from occ_gb300 import workloads as wl
    box = 10.0 * (waters / 32.0) ** (1.0 / 3.0)
    mol = wl.water_cluster(waters, box=box, seed=seed)
    basis = wl.basis_for(mol, "def2-svp")
    D = wl.random_density(basis.nbf(), 5 * waters, seed=seed)
    return mol, basis, D


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def device_timing(dft, D, precision, steps, warmup, torch):
    """Builds with D, V, E_xc resident on the device; CUDA events on the
    launching stream.  Returns (total_ms, per_step_ms, exc)."""
    lib = dft.ctx.lib
    nbf = D.shape[0]
    dD = torch.tensor(np.asfortranarray(D).ravel(order="F"), device="cuda", dtype=torch.float64)
    dV = torch.zeros(nbf * nbf, device="cuda", dtype=torch.float64)
    dE = torch.zeros(2, device="cuda", dtype=torch.float64)
    torch.cuda.synchronize()
    # a dedicated stream: the library's kernels and the timing events share it
    stream = torch.cuda.Stream()
    assert stream.cuda_stream != 0

    def one():
        rc = lib.occ_xc_compute_vxc_device(dft.ctx.h, dft.h, C.c_void_p(dD.data_ptr()), precision,
                                           C.c_void_p(dV.data_ptr()), C.c_void_p(dE.data_ptr()),
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
    per = [ev[i].elapsed_time(ev[i + 1]) for i in range(steps)]
    return ev[0].elapsed_time(ev[-1]), per, float(dE[0].item()), dV


def pinned_fortran(torch, n, values=None):
    """An n x n Fortran-ordered float64 numpy view of pinned host memory."""
    a = torch.empty(n * n, dtype=torch.float64, pin_memory=True).numpy().reshape(
        (n, n), order="F")
    if values is not None:
        a[...] = values
    return a


def e2e_timing(dft, D, precision, steps, warmup, torch=None):
    """Host entry point: D from pinned host memory, V into pinned host memory
    (both copies and E_xc's inside the timed region)."""
    if torch is not None:
        Dp = pinned_fortran(torch, D.shape[0], D)
        Vp = pinned_fortran(torch, D.shape[0])
    else:
        Dp, Vp = np.asfortranarray(D), None
    for _ in range(warmup):
        dft.compute_vxc(Dp, precision, out=Vp)
    t0 = time.perf_counter()
    for _ in range(steps):
        dft.compute_vxc(Dp, precision, out=Vp)
    return (time.perf_counter() - t0) * 1e3


def kernel_profile(dft, D, precision, nbuilds, torch):
    lib = dft.ctx.lib
    lib.occ_xc_profile_enable.argtypes = [C.c_void_p, C.c_int]
    lib.occ_xc_profile_reset.argtypes = [C.c_void_p]
    lib.occ_xc_profile_count.argtypes = [C.c_void_p]
    lib.occ_xc_profile_entry.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_char_p),
                                         C.POINTER(C.c_double), C.POINTER(C.c_long)]
    lib.occ_xc_profile_reset(dft.ctx.h)
    lib.occ_xc_profile_enable(dft.ctx.h, 1)
    for _ in range(nbuilds):
        dft.compute_vxc(D, precision)
    n = lib.occ_xc_profile_count(dft.ctx.h)
    out = {}
    for i in range(n):
        name, ms, cnt = C.c_char_p(), C.c_double(), C.c_long()
        lib.occ_xc_profile_entry(dft.ctx.h, i, C.byref(name), C.byref(ms), C.byref(cnt))
        out[name.value.decode()] = (ms.value, cnt.value)
    lib.occ_xc_profile_enable(dft.ctx.h, 0)
    lib.occ_xc_profile_reset(dft.ctx.h)
    return out


def leaf_stats(dft):
    info = dft.info()
    lib = dft.ctx.lib
    n = info["nleaves"]
    cnt = np.zeros(n, dtype=np.int32)
    m = np.zeros(n, dtype=np.int32)
    lib.occ_xc_molecule_leaves.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    lib.occ_xc_molecule_leaves(dft.h, cnt.ctypes.data, m.ctypes.data)
    return cnt, m


def algorithmic_bytes(kernel, cnt, m, npts, nbf, deriv):
    """Bytes a mixed-path kernel must move once per build in this layout
    (each AO plane is FP32 [block][mp][128]):
      rho_mixed  phi (+ gradient) planes read once, the BF16 exact-grid
                 A-slice images read once (three 128 x 64 BF16 tiles per K
                 chunk of 64 AOs, the last chunk zero-padded), rho (+
                 gradient) written, D2 read once
      func       rho and the grid read, Y written (one FP32 plane) from the
                 phi (+ gradient) planes
      vxc_mixed  phi and Y (FP32 planes, split into TF32 hi / lo in shared
                 memory) read once, V written once"""
    blocks = np.ceil(cnt / 128.0)
    mp = np.ceil(m / 32.0) * 32
    pairs = float(np.sum(blocks * 128 * mp))  # point-AO entries of one plane
    ncomp = 4 if deriv else 1
    if kernel == "rho_mixed":
        a_images = float(np.sum(blocks * np.ceil(mp / 64.0))) * 3 * 128 * 64 * 2
        return ncomp * 4 * pairs + a_images + 8 * ncomp * npts + 8.0 * nbf * nbf
    if kernel == "func":
        return (ncomp + 1) * 4 * pairs + (32 + 8 * ncomp) * npts
    if kernel == "vxc_mixed":
        return 2 * 4 * pairs + 8.0 * nbf * nbf
    return float("nan")


def measured_traffic(kernel):
    """dram__bytes_read.sum + dram__bytes_write.sum per launch of `kernel` on
    this workload, from the ncu summary committed in profiles/ (None if
    absent)."""
    path = os.path.join(ROOT, "profiles", "mixed_traffic_water32_def2svp_pbe.md")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch") and f" {kernel} " in line:
                    return float(line.split("=")[1].split()[0])
    except (OSError, ValueError, IndexError):
        pass
    return None


def cpu_baseline(basis, P, W, D, target_s=15.0, method="pbe"):
    """Oracle (CPU restatement of the reference algorithm) on every host core,
    on a strided sample of leaves scaled by the sampled share of the
    contraction FLOPs, or on whole builds when one build is shorter than
    the target.  Returns (baseline dict, (E_xc, V_xc) of a whole oracle
    build of this input, for the parity check)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    cores = os.cpu_count() or 1
    L = oracle.lib()
    L.oracle_last_flops.restype = C.c_double
    L.oracle_total_flops.restype = C.c_double
    stride = 64
    t0 = time.perf_counter()
    oracle.xc_build(basis, P, W, D, method, nthreads=cores, leaf_stride=stride)
    dt = time.perf_counter() - t0
    f_sample = L.oracle_last_flops()
    f_all = L.oracle_total_flops()
    whole = None
    # grow the sample to about target_s of work
    stride2 = max(1, int(stride * dt / target_s)) if dt > 0 else stride
    if stride2 < stride:
        t0 = time.perf_counter()
        r = oracle.xc_build(basis, P, W, D, method, nthreads=cores, leaf_stride=stride2)
        dt = time.perf_counter() - t0
        f_sample = L.oracle_last_flops()
        stride = stride2
        if stride == 1:
            whole = r
    reps = 1
    if stride == 1 and dt < target_s:
        # the whole build is shorter than the target: repeat it
        reps = max(1, int(np.ceil(target_s / max(dt, 1e-3))))
        t0 = time.perf_counter()
        for _ in range(reps):
            whole = oracle.xc_build(basis, P, W, D, method, nthreads=cores)
        dt = (time.perf_counter() - t0) / reps
        f_sample = f_all
    builds_per_s = (f_sample / f_all) / dt
    what = (f"{reps} whole builds, {dt:.2f} s each" if stride == 1 else
            f"every {stride}th Morton leaf ({100 * f_sample / f_all:.1f}% of the contraction "
            f"FLOPs) of the same build, {dt:.1f} s, scaled by the FLOP share")
    if whole is None:
        whole = oracle.xc_build(basis, P, W, D, method, nthreads=cores)
    return ({"value": builds_per_s, "unit": "builds/s", "cores": cores, "kind": "port",
             "sample": f"{what}; {cores} OpenMP threads",
             "contraction_gflops": f_sample / dt / 1e9},
            (whole[0], whole[1]))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    _, basis, D = make_workload(waters=args.waters)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import host_grid
    P, W = host_grid(basis)
    vals = []
    for _ in range(max(1, args.warmup // 3)):
        cpu_baseline(basis, P, W, D, target_s=5.0)
    cb = None
    for _ in range(args.steps if args.steps <= 3 else 3):
        cb, _ = cpu_baseline(basis, P, W, D, target_s=10.0)
        vals.append(cb["value"])
    v = statistics.median(vals)
    cb["value"] = v
    line = {"metric": METRIC, "value": v, "unit": "builds/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": len(vals), "warmup": args.warmup,
            "ms_per_step": 1e3 / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "note": "CPU restatement of the reference algorithm "
                       "(oracle/); OCC itself cannot be built offline"},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "builds/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload != "water32":
        run_workload(args)
        return
    import torch
    import torch.distributed as dist

    import occ_gb300 as og
    from occ_gb300.replicas import aggregate_rate

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    mol, basis, D = make_workload(seed=0, waters=args.waters)
    dft = og.DFT("pbe", basis, device=local)
    og.set_persistent_ctas(args.ctas, device=local)
    info = dft.info()
    lib = dft.ctx.lib
    lib.occ_xc_launch_count.restype = C.c_long
    lib.occ_xc_launch_count.argtypes = [C.c_void_p]

    nbf_ = basis.nbf()
    V_fp64 = V_mixed = None
    have_mixed = True
    try:
        dft.compute_vxc(D, og.MIXED)
    except og.XCError:
        have_mixed = False
    head = og.MIXED if (have_mixed and args.precision != "fp64") else og.FP64

    results = {}
    precisions = [og.FP64] + ([og.MIXED] if have_mixed else [])
    clocks = None
    for prec in precisions:
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        l0 = lib.occ_xc_launch_count(dft.ctx.h)
        with ClockSampler(local) as cs:
            total_ms, per, exc, dV = device_timing(dft, D, prec, args.steps, args.warmup, torch)
        Vres = dV.cpu().numpy().reshape(nbf_, nbf_, order="F").copy()
        if prec == og.FP64:
            V_fp64 = Vres
        else:
            V_mixed = Vres
        launches = lib.occ_xc_launch_count(dft.ctx.h) - l0
        rate, secs, _ = aggregate_rate(args.steps, total_ms / 1e3, dist if world > 1 else None)
        results[prec] = dict(total_ms=secs * 1e3, rate=rate, per=per, exc=exc,
                             launches=launches * args.steps // (args.steps + args.warmup))
        if prec == head:
            clocks = cs.summary()
    e2e_ms = e2e_timing(dft, D, head, args.steps, max(1, args.warmup), torch)
    prof = kernel_profile(dft, D, head, 3, torch)

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    r = results[head]
    ms_per = r["total_ms"] / args.steps
    value = r["rate"]
    nbf = info["nbf"]
    # dominant kernel and its roofline
    tot = sum(v[0] for v in prof.values())
    dom = max(prof.items(), key=lambda kv: kv[1][0])
    dom_name, (dom_ms, dom_n) = dom
    dom_avg_ms = dom_ms / dom_n
    flops_half = info["flops_per_build"] / 2  # one of the two contractions
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    if "f64" in dom_name or head == og.FP64:
        achieved = flops_half / (dom_avg_ms / 1e3) / 1e12
        roof = {"bound": "fp64", "achieved": achieved, "peak": None, "unit": "TFLOP/s",
                "frac": None, "traffic": None, "kernel": dom_name,
                "note": "FP64 DFMA pipe; MEASURED_PEAKS.json has no FP64 figure"}
    else:
        cnt, m = leaf_stats(dft)
        nbytes = algorithmic_bytes(dom_name, cnt, m, info["npoints"], nbf, info["deriv"])
        peak = peaks.get("hbm_gbs", 6800.0)
        achieved = nbytes / (dom_avg_ms / 1e3) / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": measured_traffic(dom_name),
                "kernel": dom_name, "algorithmic_bytes": nbytes,
                "peak_source": ("MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks
                                else "6.8 TB/s copy bandwidth measured earlier on a GB300 "
                                     "(of fallback)"),
                # the contraction it carries, for reference (not the bound)
                "useful_tflops": (flops_half / (dom_avg_ms / 1e3) / 1e12
                                  if dom_name in ("rho_mixed", "vxc_mixed") else None)}
        if dom_name in ("rho_mixed", "vxc_mixed"):
            # the same kernel against the tensor roof: the split products
            # executed per useful product (3xTF32: 3 on the TF32 rate, half
            # the measured BF16 one; the exact-grid density: 8 BF16 MMAs per
            # K step), padding of the tiles not counted
            tf32 = dom_name == "vxc_mixed"
            bf16 = peaks.get("bf16_tflops", 1900.0)
            tpeak = bf16 / 2 if tf32 else bf16
            executed = roof["useful_tflops"] * (3 if tf32 else 8)
            roof["tensor"] = {"executed_tflops": executed, "peak": tpeak, "unit": "TFLOP/s",
                              "frac": executed / tpeak,
                              "peak_source": ("half of MEASURED_PEAKS.json bf16_tflops (TF32 rate)"
                                              if tf32 else "MEASURED_PEAKS.json bf16_tflops")
                                             + (" (of measured)" if "bf16_tflops" in peaks
                                                else " (of fallback)")}
    roof["kernel_share"] = dom_ms / tot if tot else None
    roof["kernels_ms_per_build"] = {k: v[0] / v[1] for k, v in prof.items()}

    out = {
        "metric": METRIC,
        "value": value, "unit": "builds/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if head == og.FP64 else "tf32x3+f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "natoms": len(mol), "nbf": nbf,
                   "npoints": info["npoints"], "nleaves": info["nleaves"],
                   "flops_per_build": info["flops_per_build"], "precision": "fp64" if head == og.FP64 else "mixed",
                   "parallelism": f"replicas{world}",
                   "l2": "inputs larger than L2: per-build workspace "
                         f"{(info['mixed_workspace_bytes'] if head == og.MIXED else info['workspace_bytes']) / 1e9:.1f}"
                         " GB > 129 MB"},
        "p50_ms": float(np.percentile(r["per"], 50)), "p99_ms": float(np.percentile(r["per"], 99)),
        "fp64": {"builds_per_s": args.steps / (results[og.FP64]["total_ms"] / 1e3),
                 "p50_ms": float(np.percentile(results[og.FP64]["per"], 50)),
                 "p99_ms": float(np.percentile(results[og.FP64]["per"], 99)),
                 "exc": results[og.FP64]["exc"]},
        "e2e": {"value": world * args.steps / (e2e_ms / 1e3), "unit": "builds/s",
                "h2d_bytes_per_step": nbf * nbf * 8, "d2h_bytes_per_step": nbf * nbf * 8 + 16},
        "gpu_launches": int(r["launches"]),
        "roofline": roof,
        "clocks": clocks,
    }
    if og.MIXED in results:
        m = results[og.MIXED]
        out["mixed"] = {"builds_per_s": args.steps / (m["total_ms"] / 1e3),
                        "p50_ms": float(np.percentile(m["per"], 50)),
                        "p99_ms": float(np.percentile(m["per"], 99)), "exc": m["exc"],
                        "dE_xc_vs_fp64": m["exc"] - results[og.FP64]["exc"]}
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        P, W = dft.grid()
        out["cpu_baseline"], (e_or, V_or) = cpu_baseline(basis, P, W, D)
        # parity at this size: the GPU builds against a whole oracle build of
        # the same input (bars: FP64 1e-8 Ha and 1e-9, mixed 1e-6 Ha and 1e-5)
        par = {"exc_oracle": e_or,
               "fp64": {"dE_xc": results[og.FP64]["exc"] - e_or,
                        "max_dV": float(np.max(np.abs(V_fp64 - V_or))),
                        "bars": [1e-8, 1e-9]}}
        if og.MIXED in results:
            par["mixed"] = {"dE_xc": results[og.MIXED]["exc"] - e_or,
                            "max_dV": float(np.max(np.abs(V_mixed - V_or))),
                            "bars": [1e-6, 1e-5]}
        par["within_bars"] = all(abs(v["dE_xc"]) <= v["bars"][0] and v["max_dV"] <= v["bars"][1]
                                 for k, v in par.items() if k in ("fp64", "mixed"))
        out["parity_vs_oracle"] = par
    print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
