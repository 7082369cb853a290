#!/usr/bin/env python3
"""Benchmark of the GB300 GMlib mesh-kernel path.

Workload (one "step"): the smoothing configuration on a 128^3-hex unit cube
split into 6 tets per hex with the reflected split (12,582,912 tets,
2,146,689 vertices, ragged vertex->tet degrees 4..48), interior vertices
jittered by +-0.3h, Hilbert renumbered, boundary vertices fixed: 10 Jacobi
sweeps of Laplacian smoothing over the ball of points, each followed by the
mean-ratio quality of every tet with a 64-bin histogram, min/argmin and
FP64-decided inverted-element flags.  One step is one replay of the CUDA
graph built by GmlxSmoothQualityLoop.

value      algorithmic (unique) bytes of a step / device time of a step, GB/s,
           inputs resident in HBM; timed with CUDA events on the library's
           stream over K steps after W warm-up steps.
e2e        the same bytes / wall time of a step through the C ABI with host
           buffers: upload of the coordinates (pinned host mirror), the step,
           download of the statistics and of the coordinates.
roofline   the dominant kernel, its algorithmic bytes per launch / its mean
           launch time measured here with CUDA events, against the measured
           HBM copy bandwidth.
cpu_baseline  the oracle's multithreaded port of the same workload on the
           host cores (a bounded sample: one sweep + one quality pass).

--impl reference times that CPU port as the reference arm (the reference
itself is OpenCL and has no runnable CPU path here).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_HEX = 128
SPLIT = 1
JITTER = 0.3
SEED = 2024
SWEEPS = 10
OMEGA = 1.0
FALLBACK_HBM = 6800.0
METRIC = "HBM GB/s/kernel"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=600)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--n", type=int, default=N_HEX, help="hexes per cube side")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-other-configs", action="store_true",
                   help="smooth: leave out the compact results of the quality, solver and "
                        "batch configurations (for profiler runs of the step alone)")
    p.add_argument("--refhost", action="store_true",
                   help="reference arm: also time the reference's own host library and "
                        "NodeSmoothing kernels on the CPU (needs the reference tree)")
    p.add_argument("--e2e-steps", type=int, default=20)
    p.add_argument("--workload", default="smooth",
                   choices=["smooth", "quality", "nodesmooth", "solve", "batch", "serve", "p2"],
                   help="smooth: the smoothing + quality step (default); quality: the plain "
                        "quality pass on the 32^3-hex Kuhn cube; nodesmooth: the reference's "
                        "NodeSmoothing flow through generated kernels; solve: block SpMV and CG; "
                        "batch: 512 meshes through the tile queue vs the per-mesh launch loop; "
                        "serve: the request loop on a Poisson stream; p2: the P2Quality flow "
                        "through a generated kernel")
    p.add_argument("--degree-sort", action="store_true",
                   help="nodesmooth: after the Hilbert numbering, put the vertices in at most "
                        "32 tets first (GmlxDegreeSort)")
    p.add_argument("--meshes", type=int, default=512, help="batch: number of meshes")
    p.add_argument("--duration", type=float, default=60.0, help="serve: seconds of arrivals")
    p.add_argument("--rate", type=float, default=200.0, help="serve: requests per second")
    p.add_argument("--saturate", type=int, default=600,
                   help="serve: requests of the trace replayed all at t = 0 on both paths "
                        "(capacity)")
    p.add_argument("--serial-requests", type=int, default=200,
                   help="serve: requests of the trace replayed on the serial plain path")
    p.add_argument("--sweep-seconds", type=float, default=5.0,
                   help="serve: seconds of arrivals per rate of the p99 capacity sweep (0: none)")
    return p.parse_args()


# --------------------------------------------------------------- distributed

class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x):
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# -------------------------------------------------------------------- clocks

class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev = dev
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100", "-i", str(self.dev)],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, val in zip(names, parts[5:9]):
                    if val.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "samples": len(sm), "reasons": sorted(reasons)}


# ----------------------------------------------------------------- helpers

def peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, burst copy)"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM, "fallback 6.8 TB/s"


def traffic_for(kernel):
    """Per-launch DRAM bytes of a kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d.get(kernel)
    except (OSError, ValueError):
        return None


def l1_wavefronts_for(kernel):
    """L1 data-pipe wavefronts of one launch of a kernel (ncu
    l1tex__data_pipe_lsu_wavefronts.sum) from the committed summary."""
    path = os.path.join(ROOT, "profiles", "l1_wavefronts.json")
    try:
        with open(path) as f:
            return json.load(f).get(kernel)
    except (OSError, ValueError):
        return None


def sm_count(dev):
    """Multiprocessor count of device `dev` from the CUDA driver."""
    try:
        cu = ctypes.CDLL("libcuda.so.1")
        d, n = ctypes.c_int(), ctypes.c_int()
        if cu.cuInit(0) or cu.cuDeviceGet(ctypes.byref(d), dev) \
           or cu.cuDeviceGetAttribute(ctypes.byref(n), 16, d):      # MULTIPROCESSOR_COUNT
            return None
        return n.value
    except OSError:
        return None


def l1_bound(kernel, launch_s, dev, clk):
    """The kernel's L1 data-pipe load against its bound of one wavefront per
    SM per cycle, at the SM clock sampled during the timed region."""
    w, nsm = l1_wavefronts_for(kernel), sm_count(dev)
    mhz = (clk or {}).get("sm_mhz") or 2070.0
    if not w or not nsm:
        return None
    return {"wavefronts_per_launch": w, "sms": nsm, "sm_mhz": mhz,
            "bound_us": round(w / nsm / mhz, 2),
            "frac": round(w / nsm / (mhz * 1e6) / launch_s, 4),
            "source": "ncu l1tex__data_pipe_lsu_wavefronts.sum, profiles/l1_wavefronts.json"}


def mesh(n):
    import gmlib_gb300 as G
    crd, tet, ref = G.cube_mesh(n, split=SPLIT, jitter=JITTER, seed=SEED)
    return crd, tet, ref


def degree_summary(tets):
    """Vertex -> tet degrees over one or more meshes: min, mean, max and the
    histogram {degree: vertices}."""
    hist = np.zeros(1, np.int64)
    for t in tets:
        d = np.bincount(np.bincount(np.asarray(t).ravel()))
        if len(d) > len(hist):
            hist = np.pad(hist, (0, len(d) - len(hist)))
        hist[:len(d)] += d
    hist[0] = 0
    degs = np.nonzero(hist)[0]
    return {"min": int(degs[0]), "max": int(degs[-1]),
            "mean": round(float((degs * hist[degs]).sum() / hist[degs].sum()), 3),
            "hist": {str(int(k)): int(hist[k]) for k in degs}}


def workload_config(n, nv, nt, wset_mb, degrees=None):
    return {"workload": "ball-of-points Laplacian smoothing + mean-ratio quality, "
                        "%d^3-hex cube, reflected 6-tet split" % n,
            "vertex_tet_degrees": degrees,
            "hex_per_side": n, "tets": nt, "vertices": nv, "sweeps_per_step": SWEEPS,
            "per_sweep": "Jacobi sweep (boundary fixed) + quality, 64-bin histogram, "
                         "min/argmin, FP64 inverted flags",
            "jitter": JITTER, "seed": SEED, "omega": OMEGA,
            "l2": ("inputs larger than L2: %.0f MB working set > 129 MB L2" % wset_mb
                   if wset_mb > 129 else
                   "inputs fit in L2 (%.0f MB working set): a small case, not the "
                   "benchmark configuration" % wset_mb)}


# ---------------------------------------------------------------- CPU port

def cpu_port(crd, tet, ref, nsweeps, reps):
    """Time the oracle's OpenMP port: reps steps of nsweeps sweep+quality
    passes, each from the mesh's initial coordinates; returns (seconds per
    step list, threads, ball entries, the first step's result: coordinates,
    last-sweep histogram, minimum, argmin, inverted count)."""
    import oracle as O
    lib = O.lib()
    fixed = (ref != 0).astype(np.int32)
    ptr, col = O.point_ball(len(crd), tet, fixed)
    tmp = np.zeros((len(crd), 4), np.float32)
    hist = np.zeros(64 * nsweeps, np.uint32)
    qmin = np.zeros(nsweeps, np.float32)
    imin = np.zeros(nsweeps, np.int32)
    ninv = np.zeros(nsweeps, np.uint32)
    ts, first = [], None
    for r in range(reps):
        c = np.array(crd, np.float32, copy=True)
        t0 = time.perf_counter()
        lib.orc_bench_step(len(c), len(tet), O._ptr(c), O._ptr(tmp), O._ptr(tet), O._ptr(ptr),
                           O._ptr(col), ctypes.c_float(OMEGA), nsweeps, O._ptr(hist),
                           O._ptr(qmin), O._ptr(imin), O._ptr(ninv))
        ts.append(time.perf_counter() - t0)
        if r == 0:
            first = {"crd": c, "hist": hist[-64:].copy(), "min": float(qmin[-1]),
                     "argmin": int(imin[-1]), "inverted": int(ninv[-1])}
    return ts, lib.orc_threads(), len(col), first


def step_bytes_host(nv, nt, used):
    sweep = 4.0 * nv + 4.0 * used + 32.0 * nv
    qual = 16.0 * nt + 16.0 * nv + 4.0 * ((nt + 31) // 32)
    return sweep, qual


# ------------------------------------------------------------- reference arm

def run_reference(args, dist):
    """The reference arm: the same step as the GPU arm (SWEEPS Jacobi sweeps,
    each followed by the quality pass with histogram, minimum and inverted
    count) on the same mesh, by the oracle's OpenMP port on every host core,
    --warmup untimed and --steps timed whole steps."""
    if dist.rank != 0:
        return
    n = args.n
    crd, tet, ref = mesh(n)
    ts, threads, used, _ = cpu_port(crd, tet, ref, SWEEPS, args.warmup + args.steps)
    ts = ts[args.warmup:]
    sweep, qual = step_bytes_host(len(crd), len(tet), used)
    per = statistics.median(ts)
    value = SWEEPS * (sweep + qual) / per / 1e9
    sample = "the whole step (%d sweeps + %d quality passes) on the full mesh, median of %d " \
             "timed steps" % (SWEEPS, SWEEPS, args.steps)
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "GB/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(per * 1e3, 3), "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(n, len(crd), len(tet), working_set(len(crd), len(tet), used),
                                      degree_summary([tet])),
            "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": threads,
                             "kind": "port", "sample": sample},
            "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "note": "the reference is OpenCL host code plus OpenCL kernels; no OpenCL "
                    "runtime exists on this box, so its CPU path is the oracle's "
                    "OpenMP port of the same workload"}
    if args.refhost:
        line["reference_host_nodesmoothing"] = refhost_nodesmoothing(crd, tet, ref)
    print(json.dumps(line), flush=True)


def refhost_nodesmoothing(crd, tet, ref, sweeps=8):
    """The reference's own NodeSmoothing sweep (examples/NodeSmoothing:
    scatter, gather with voyeurs, residual sum) through its unmodified host
    library on the host CPU (oracle/refhost: its generated kernels built by
    g++, one OpenMP loop over work-items), on the same mesh; seconds per
    sweep after the reference's work-group calibration (its first 13
    launches of each kernel).  Only where the reference tree is present."""
    from oracle import refhost as R
    from oracle import build as OB
    if not R.available():
        return {"unavailable": "the reference tree is not on this machine"}
    ex = os.path.join(OB.REF_ROOT, "examples", "NodeSmoothing")

    def body(name):
        with open(os.path.join(ex, name), "rb") as f:
            return f.read()
    I = R.Instance()
    I.parameters(64, body("parameters.cl"))
    t0 = time.perf_counter()
    v = I.mesh(R.GmlVertices, crd, ref)
    I.mesh(R.GmlTetrahedra, tet)
    o = I.solution(R.GmlTetrahedra, 4, R.GmlFlt4, b"OptCrd")
    r = I.solution(R.GmlVertices, 1, R.GmlFlt, b"res")
    ks = I.compile(body("scatter.cl"), b"scatter", R.GmlTetrahedra,
                   [(v, R.GmlReadMode), (o, R.GmlWriteMode)])
    kg = I.compile(body("gather.cl"), b"gather", R.GmlVertices,
                   [(r, R.GmlWriteMode), (o, R.GmlReadMode | R.GmlVoyeurs),
                    (v, R.GmlReadMode | R.GmlWriteMode)])
    setup = time.perf_counter() - t0
    ts = []
    for i in range(14 + sweeps):
        t = time.perf_counter()
        I.launch(ks)
        I.launch(kg)
        I.reduce(r, R.GmlSum)
        if i >= 14:
            ts.append(time.perf_counter() - t)
    I.stop()
    return {"seconds_per_sweep": round(statistics.median(ts), 4), "setup_seconds": round(setup, 2),
            "threads": R.lib() and __import__("oracle").lib().orc_threads(),
            "what": "reference host library (ball tables, generated kernels) + its scatter/gather "
                    "bodies, OpenMP over work-items, g++ -O2"}


def working_set(nv, nt, used):
    """MB read per step-pass of the workload, the same for both arms: tets,
    coordinates read and written, ball entries."""
    return (16.0 * nt + 32.0 * nv + 4.0 * used) / 1e6


# ------------------------------------------------------------------ GPU arm

def run_gpu(args, dist):
    import gmlib_gb300 as G
    n = args.n
    h = 1.0 / n
    dev = dist.local
    # the serving sub-result runs first, in a process of its own, while this
    # process holds nothing on the device or in page-locked host memory
    serve_first = serve_in_fresh_process(dev) \
        if dist.world == 1 and not args.no_other_configs else None
    crd, tet, ref = mesh(n)
    nv, nt = len(crd), len(tet)
    degrees = degree_summary([tet])

    g = G.lib.GmlInit(dev)
    if not g:
        raise SystemExit("GmlInit(%d) failed" % dev)
    G.lib.GmlxSetTiming(g, 0)
    vidx, tidx = G.upload_mesh(g, crd, tet, ref)
    if G.lib.GmlxMeshSetup(g, 1) != 1:
        raise SystemExit("GmlxMeshSetup failed")
    sweep_b, qual_b = ctypes.c_double(), ctypes.c_double()
    G.lib.GmlxMeshBytes(g, ctypes.byref(sweep_b), ctypes.byref(qual_b))
    step_bytes = SWEEPS * (sweep_b.value + qual_b.value)
    stored, used, mx = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_int()
    G.lib.GmlxMeshBallInfo(g, ctypes.byref(stored), ctypes.byref(used), ctypes.byref(mx))
    wset = working_set(nv, nt, used.value)
    res = (G.GmlxQuality * SWEEPS)()
    om = ctypes.c_float(OMEGA)

    for _ in range(args.warmup):
        G.lib.GmlxSmoothQualityLoop(g, SWEEPS, om, h, None)
    G.lib.GmlxSynchronize(g)

    e0, e1 = G.lib.GmlxEventCreate(), G.lib.GmlxEventCreate()
    clocks = Clocks(dev)
    dist.barrier()
    G.lib.GmlxSynchronize(g)
    clocks.start()
    time.sleep(0.3)
    G.lib.GmlxEventRecord(g, e0)
    for _ in range(args.steps):
        if G.lib.GmlxSmoothQualityLoop(g, SWEEPS, om, h, None) != 1:
            raise SystemExit("step failed")
    G.lib.GmlxEventRecord(g, e1)
    dev_s = G.lib.GmlxEventElapsed(e0, e1)
    G.lib.GmlxSynchronize(g)
    clk = clocks.stop()
    dist.barrier()
    dev_s = dist.max(dev_s)
    per_step = dev_s / args.steps
    value = dist.world * step_bytes / per_step / 1e9

    # statistics of the last step (checks that the step did its work)
    G.lib.GmlxSmoothQualityLoop(g, SWEEPS, om, h, res)
    last = res[SWEEPS - 1]

    # per-kernel launch times, same stream, CUDA events
    reps = 50
    G.lib.GmlxEventRecord(g, e0)
    for _ in range(reps):
        G.lib.GmlxSmooth(g, 2, om)
    G.lib.GmlxEventRecord(g, e1)
    t_sweep = G.lib.GmlxEventElapsed(e0, e1) / (2 * reps)
    G.lib.GmlxEventRecord(g, e0)
    for _ in range(reps):
        G.lib.GmlxQualityStats(g, h, 0, None)
    G.lib.GmlxEventRecord(g, e1)
    t_qual = G.lib.GmlxEventElapsed(e0, e1) / reps
    peak, peak_src = peak_hbm()
    kern = [("laplace_pf_kernel", sweep_b.value, t_sweep),
            ("tet_quality_tma_kernel", qual_b.value, t_qual)]
    kern.sort(key=lambda k: -k[2])
    name, kb, kt = kern[0]
    achieved = kb / kt / 1e9
    roof = {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": peak,
            "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic_for(name),
            "l1_data_pipe": l1_bound(name, kt, dev, clk),
            "algorithmic_bytes_per_launch": kb, "mean_launch_us": round(kt * 1e6, 2),
            "peak_source": peak_src,
            "other_kernels": [{"kernel": k[0], "achieved": round(k[1] / k[2] / 1e9, 1),
                               "frac": round(k[1] / k[2] / 1e9 / peak, 4),
                               "mean_launch_us": round(k[2] * 1e6, 2),
                               "l1_data_pipe": l1_bound(k[0], k[2], dev, clk)} for k in kern[1:]]}

    # end to end through the C ABI with host buffers
    host_crd = np.ascontiguousarray(crd)
    out_crd = np.empty_like(host_crd)
    e2e_t = []
    for i in range(args.e2e_steps + 2):
        t0 = time.perf_counter()
        G.lib.GmlxSetData(g, vidx, G.as_ptr(host_crd), host_crd.nbytes)
        G.lib.GmlxSmoothQualityLoop(g, SWEEPS, om, h, res)
        G.lib.GmlxGetData(g, vidx, G.as_ptr(out_crd), out_crd.nbytes)
        if i >= 2:
            e2e_t.append(time.perf_counter() - t0)
    e2e_s = dist.max(statistics.median(e2e_t))
    e2e = {"value": round(dist.world * step_bytes / e2e_s / 1e9, 3), "unit": "GB/s",
           "h2d_bytes_per_step": host_crd.nbytes,
           "d2h_bytes_per_step": out_crd.nbytes + SWEEPS * ctypes.sizeof(G.GmlxQuality),
           "ms_per_step": round(e2e_s * 1e3, 3)}

    # one step from the initial coordinates, kept for the check below
    G.lib.GmlxSetData(g, vidx, G.as_ptr(host_crd), host_crd.nbytes)
    G.lib.GmlxSmoothQualityLoop(g, SWEEPS, om, h, res)
    first_crd = np.empty_like(host_crd)
    G.lib.GmlxGetData(g, vidx, G.as_ptr(first_crd), first_crd.nbytes)
    first = res[SWEEPS - 1]

    cpu, check = None, None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        # the CPU baseline: whole steps of the port; its first step, from the
        # same initial coordinates, is also the checker of the GPU's first step
        ts, threads, cused, port = cpu_port(crd, tet, ref, SWEEPS, 3)
        sw, qu = step_bytes_host(nv, nt, cused)
        cpu = {"value": round(SWEEPS * (sw + qu) / statistics.median(ts) / 1e9, 3), "unit": "GB/s",
               "cores": threads, "kind": "port",
               "sample": "the whole step (%d sweeps + %d quality passes) on the full mesh, "
                         "median of 3" % (SWEEPS, SWEEPS)}
        dx = float(np.max(np.abs(first_crd[:, :3] - port["crd"][:, :3])))
        hd = int(np.abs(np.array(first.Hist[:], np.int64) - port["hist"].astype(np.int64)).sum())
        check = {"against": "the CPU port's step from the same coordinates (FP32)",
                 "max_coordinate_diff": dx, "histogram_abs_diff": hd,
                 "min": [first.MinQal, port["min"]], "argmin": [first.MinIdx, port["argmin"]],
                 "inverted": [first.NmbInv, port["inverted"]],
                 "pass": bool(dx <= 2e-6 and hd <= 8 and first.MinIdx == port["argmin"]
                              and abs(first.MinQal - port["min"]) <= 2e-5
                              and first.NmbInv == port["inverted"])}

    others = other_configs(G, dev, dist, serve_first) \
        if dist.world == 1 and not args.no_other_configs else None

    G.lib.GmlStop(g)

    if dist.rank == 0:
        line = {"metric": METRIC, "value": round(value, 3), "unit": "GB/s",
                "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": round(per_step * 1e3, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": workload_config(n, nv, nt, wset, degrees),
                "gpu_launches": args.steps * (2 * SWEEPS + 1),
                "roofline": roof, "e2e": e2e, "cpu_baseline": cpu, "clocks": clk,
                "result_check": {"last_sweep_min_quality": last.MinQal,
                                 "last_sweep_argmin": last.MinIdx,
                                 "inverted": last.NmbInv, "fp64_determinants": last.NmbF64,
                                 "ball_entries_used": used.value,
                                 "ball_entries_stored": stored.value,
                                 "max_ball_of_points": mx.value,
                                 "first_step_check": check},
                "other_configs": others}
        print(json.dumps(line), flush=True)


def other_configs(G, dev, dist, sv=None):
    """Compact results of the plain-quality configuration (32^3-hex Kuhn
    cube, 196,608 tets: one quality pass with statistics, L2 flushed before
    each of 20 launches), of the solver configuration (96^3-hex SPD
    block system: FP64 CG and FP32 CG inside FP64 refinement to 1e-10,
    median of 3 solves after one) and of the batch configuration (512
    meshes, 5 runs of each path after 2), for the default run."""
    out = {}
    n = Q_N
    crd, tet, ref = G.cube_mesh(n, split=0, jitter=Q_JITTER, seed=Q_SEED)
    g = G.lib.GmlInit(dev)
    if not g:
        raise SystemExit("GmlInit failed")
    G.lib.GmlxSetTiming(g, 0)
    G.upload_mesh(g, crd, tet, ref)
    if G.lib.GmlxMeshSetup(g, 1) != 1:
        raise SystemExit("GmlxMeshSetup failed")
    flush = G.lib.GmlNewVector(g, 16 << 20, 4, None, G.GmlFlt)
    one = ctypes.c_double(1.0)
    e0, e1 = G.lib.GmlxEventCreate(), G.lib.GmlxEventCreate()
    res = G.GmlxQuality()
    for _ in range(3):
        G.lib.GmlxQualityStats(g, 1.0 / n, 0, None)
    tot = 0.0
    for _ in range(20):
        G.lib.GmlScaleVec(g, flush, ctypes.byref(one))
        G.lib.GmlxEventRecord(g, e0)
        G.lib.GmlxQualityStats(g, 1.0 / n, 0, None)
        G.lib.GmlxEventRecord(g, e1)
        tot += G.lib.GmlxEventElapsed(e0, e1)
    G.lib.GmlxQualityStats(g, 1.0 / n, 0, ctypes.byref(res))
    G.lib.GmlStop(g)
    out["quality_32cube"] = {"metric": "tet qualities per second", "unit": "M tets/s",
                             "value": round(len(tet) / (tot / 20) / 1e6, 2),
                             "mean_launch_us": round(tot / 20 * 1e6, 2),
                             "min": res.MinQal, "argmin": res.MinIdx, "inverted": res.NmbInv}
    lin, col, val, rhs = G.cube_spd(SOLVE_N, 0, seed=SEED)
    nrow, nnzb = len(lin) - 1, len(col)
    g = G.lib.GmlInit(dev)
    G.lib.GmlxSetTiming(g, 0)
    IP = ctypes.POINTER(ctypes.c_int)
    v64 = np.ascontiguousarray(val)
    m64 = G.lib.GmlNewMatrix(g, nrow, nnzb, 3, G.as_ptr(v64), col.ctypes.data_as(IP),
                             lin.ctypes.data_as(IP), G.GmlDbl)
    vb = G.lib.GmlNewVector(g, nrow, 3, G.as_ptr(rhs), G.GmlDbl)
    vx = G.lib.GmlNewVector(g, nrow, 3, None, G.GmlDbl)
    solves = {}
    for mode, name in ((G.GmlxCgFp64, "cg_fp64"), (G.GmlxCgMixed, "cg_fp32_in_fp64_ir")):
        info = G.GmlxSolveInfo()
        times = []
        for i in range(4):
            if G.lib.GmlxSolveCG(g, m64, vb, vx, mode, SOLVE_TOL, 20000, ctypes.byref(info)) != 1:
                raise SystemExit("%s did not converge" % name)
            if i:
                times.append(info.Seconds)
        solves[name] = {"ms": round(statistics.median(times) * 1e3, 3), "iterations": info.NmbIte,
                        "rel_residual": info.RelRes}
    G.lib.GmlStop(g)
    out["cg_96cube"] = {"metric": "FP64 CG time / FP32-CG-in-FP64-IR time", "unit": "x",
                        "value": round(solves["cg_fp64"]["ms"] / solves["cg_fp32_in_fp64_ir"]["ms"], 3),
                        "rows": nrow, "blocks": nnzb, "solves": solves}
    bo, bi = batch_measure(G, dev, 512, 5, 2)
    out["batch_512meshes"] = {"metric": "batched meshes/s (5 sweeps + quality + min per mesh)",
                              "unit": "meshes/s", "value": bo["queue"]["meshes_per_s"],
                              "queue": bo["queue"], "loop": bo["loop"],
                              "speedup_vs_loop": bi["speedup_vs_loop"], "tets": bi["tets"],
                              "frac": bi["roofline"]["frac"], "min_quality": bi["min_quality"]}
    ns = nodesmooth_measure(G, dev, N_HEX, 5, 3, 0, dist)
    out["nodesmooth_128cube"] = {
        "metric": "NodeSmoothing flow through the reference API (generated kernels), GB/s",
        "unit": "GB/s", "value": round(ns["flow_bytes"] / ns["wall"] / 1e9, 1),
        "ms_per_flow": round(ns["wall"] * 1e3, 3),
        "kernels": {k: {"mean_launch_us": v["mean_launch_us"], "frac": v["frac"]}
                    for k, v in ns["kernels"].items()},
        "mean_quality_after": ns["q1"] / ns["nt"]}
    if sv is None:
        out["serve_200rps"] = {"unavailable": "the serve run in its own process failed or "
                                              "exceeded 900 s (its output is on stderr)"}
        ctypes.CDLL(None).fflush(None)
        return out
    out["serve_200rps"] = {
        "metric": "served requests/s (continuous batching), p50/p99 latency", "unit": "req/s",
        "value": sv["batching"]["throughput_rps"],
        "arrivals": "Poisson 200 req/s for 10 s, 50/30/20 quality / smoothing / CG, "
                    "1e4..1e7 tets, reuse 0.5, 150 GB budget",
        "batching": {k: sv["batching"][k] for k in ("throughput_rps", "p50_ms", "p99_ms")},
        "serial_prefix": {k: sv["serial_prefix"][k] for k in ("throughput_rps", "p50_ms", "p99_ms")},
        "capacity_saturated": {k: sv["capacity_saturated"][k]["throughput_rps"]
                               for k in ("batching", "serial")},
        "capacity_saturated_ratio": sv["capacity_saturated"].get("batching_over_serial"),
        "capacity_at_p99": {"p99_target_ms": sv["capacity_at_p99"]["p99_target_ms"],
                            "seconds_per_run": sv["capacity_at_p99"]["seconds_per_run"],
                            "warm_seconds": sv["capacity_at_p99"].get("warm_seconds"),
                            "batching_max_rate": sv["capacity_at_p99"]["batching"]["max_rate_at_p99"],
                            "serial_max_rate": sv["capacity_at_p99"]["serial"]["max_rate_at_p99"],
                            "ratio": sv["capacity_at_p99"].get("batching_over_serial"),
                            "ratio_at_least": sv["capacity_at_p99"].get("batching_over_serial_at_least")}
        if sv.get("capacity_at_p99") else None,
        "same_result_alone_and_in_mix": "%d of %d" % (sv["same"], sv["nser"])}
    ctypes.CDLL(None).fflush(None)
    return out


# ------------------------------------------------------------- solver workload

SOLVE_N = 96
SOLVE_TOL = 1e-10


VOP_LINES = 12 << 20       # vector lines of the vector-op timings (larger than L2)


def vector_ops(G, dev, peak):
    """The reference API's vector operations on 3-blocks (GmlAddVec3,
    GmlScaleVec, GmlMultDiagMatVec with 3x3 diagonal blocks) in FP32 and
    FP64 over VOP_LINES lines, each precision in an instance of its own:
    device time per launch, CUDA events over 20 back-to-back launches.
    Algorithmic bytes count the 3 (or 9) used values per line, reads and
    writes; the stored lines are padded to 4 (or 16) values, as the
    reference's vectors are."""
    out = {}
    nl = VOP_LINES
    for fname, ft, fs in (("f32", G.GmlFlt, 4), ("f64", G.GmlDbl, 8)):
        g = G.lib.GmlInit(dev)
        if not g:
            raise SystemExit("GmlInit failed")
        G.lib.GmlxSetTiming(g, 0)
        a, b, c, d = (G.lib.GmlNewVector(g, nl, 3, None, ft) for _ in range(4))
        dg = G.lib.GmlNewVector(g, nl, 9, None, ft)
        if min(a, b, c, d, dg) <= 0:
            raise SystemExit("vector allocation failed")
        e0, e1 = G.lib.GmlxEventCreate(), G.lib.GmlxEventCreate()
        mul = ctypes.c_double(0.5)
        ops = (("add3", lambda: G.lib.GmlAddVec3(g, a, b, c, d), 4 * 3 * fs),
               ("scale", lambda: G.lib.GmlScaleVec(g, a, ctypes.byref(mul)), 2 * 3 * fs),
               ("diag", lambda: G.lib.GmlMultDiagMatVec(g, dg, b, c), (9 + 3 + 3) * fs))
        res = {}
        for name, fn, per_line in ops:
            for _ in range(3):
                fn()
            G.lib.GmlxSynchronize(g)
            G.lib.GmlxEventRecord(g, e0)
            for _ in range(20):
                if fn() != 1:
                    raise SystemExit("%s failed" % name)
            G.lib.GmlxEventRecord(g, e1)
            t = G.lib.GmlxEventElapsed(e0, e1) / 20
            byt = per_line * float(nl)
            res[name] = {"mean_launch_us": round(t * 1e6, 2), "algorithmic_bytes": byt,
                         "achieved_gbs": round(byt / t / 1e9, 1),
                         "frac": round(byt / t / 1e9 / peak, 4)}
        G.lib.GmlStop(g)
        out[fname] = res
    return out


def run_solve(args, dist):
    """Block SpMV and CG on the 3x3-block SPD system of the vertex graph of a
    96^3-hex cube (912,673 rows, 13,465,441 blocks): SpMV launch times in FP32
    and FP64 (CUDA events, 50 launches each), then FP64 CG and FP32 CG inside
    FP64 refinement to 1e-10 relative residual (device time of each solve,
    median of --steps solves after --warmup)."""
    import gmlib_gb300 as G
    n = SOLVE_N if args.n == N_HEX else args.n
    lin, col, val, rhs = G.cube_spd(n, 0, seed=SEED)
    nrow, nnzb = len(lin) - 1, len(col)
    g = G.lib.GmlInit(dist.local)
    if not g:
        raise SystemExit("GmlInit failed")
    G.lib.GmlxSetTiming(g, 0)
    IP = ctypes.POINTER(ctypes.c_int)
    lin_c, col_c = lin.ctypes.data_as(IP), col.ctypes.data_as(IP)
    v64 = np.ascontiguousarray(val)
    v32 = v64.astype(np.float32)
    m64 = G.lib.GmlNewMatrix(g, nrow, nnzb, 3, G.as_ptr(v64), col_c, lin_c, G.GmlDbl)
    m32 = G.lib.GmlNewMatrix(g, nrow, nnzb, 3, G.as_ptr(v32), col_c, lin_c, G.GmlFlt)
    x32 = rhs.astype(np.float32)
    vx32 = G.lib.GmlNewVector(g, nrow, 3, G.as_ptr(x32), G.GmlFlt)
    vy32 = G.lib.GmlNewVector(g, nrow, 3, None, G.GmlFlt)
    vb = G.lib.GmlNewVector(g, nrow, 3, G.as_ptr(rhs), G.GmlDbl)
    vx = G.lib.GmlNewVector(g, nrow, 3, None, G.GmlDbl)
    vy = G.lib.GmlNewVector(g, nrow, 3, None, G.GmlDbl)
    if min(m64, m32, vx32, vy32, vb, vx, vy) <= 0:
        raise SystemExit("allocation failed")

    e0, e1 = G.lib.GmlxEventCreate(), G.lib.GmlxEventCreate()
    peak, peak_src = peak_hbm()
    spmv = {}
    for name, m, y, x, byt in (("f32", m32, vy32, vx32, 40.0 * nnzb + 4.0 * (nrow + 1) + 24.0 * nrow),
                               ("f64", m64, vy, vb, 76.0 * nnzb + 4.0 * (nrow + 1) + 48.0 * nrow)):
        for _ in range(3):
            G.lib.GmlMultMatVec(g, m, y, x)
        G.lib.GmlxSynchronize(g)
        G.lib.GmlxEventRecord(g, e0)
        for _ in range(50):
            G.lib.GmlMultMatVec(g, m, y, x)
        G.lib.GmlxEventRecord(g, e1)
        t = G.lib.GmlxEventElapsed(e0, e1) / 50
        spmv[name] = {"mean_launch_us": round(t * 1e6, 2), "algorithmic_bytes": byt,
                      "achieved_gbs": round(byt / t / 1e9, 1), "frac": round(byt / t / 1e9 / peak, 4),
                      "gflops": round(18.0 * nnzb / t / 1e9, 1)}

    vops = vector_ops(G, dist.local, peak)

    solves = {}
    clocks = Clocks(dist.local)
    clocks.start()
    for mode, name in ((G.GmlxCgFp64, "cg_fp64"), (G.GmlxCgMixed, "cg_fp32_in_fp64_ir")):
        info = G.GmlxSolveInfo()
        times = []
        for i in range(args.warmup + args.steps):
            rc = G.lib.GmlxSolveCG(g, m64, vb, vx, mode, SOLVE_TOL, 20000, ctypes.byref(info))
            if rc != 1:
                raise SystemExit("%s did not converge (rc %d, |r|/|b| %g)" % (name, rc, info.RelRes))
            if i >= args.warmup:
                times.append(info.Seconds)
        solves[name] = {"seconds": round(statistics.median(times), 6), "iterations": info.NmbIte,
                        "refinement_steps": info.NmbOut, "rel_residual": info.RelRes,
                        "solves_per_s": round(1.0 / statistics.median(times), 2)}
    clk = clocks.stop()
    G.lib.GmlStop(g)
    speedup = solves["cg_fp64"]["seconds"] / solves["cg_fp32_in_fp64_ir"]["seconds"]
    ctypes.CDLL(None).fflush(None)          # the library's own messages go first
    if dist.rank == 0:
        line = {"metric": "CG to 1e-10: FP64 CG time / FP32-CG-in-FP64-IR time",
                "value": round(speedup, 3), "unit": "x", "n_gpus": dist.world,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                "dtype": "f64 / f32+f64", "data": "synthetic",
                "config": {"workload": "3x3-block SPD system on the vertex graph of a %d^3-hex "
                                       "tet cube" % n, "rows": nrow, "blocks": nnzb,
                           "tol": SOLVE_TOL, "inputs": "larger than L2 (FP64 matrix %.0f MB)"
                           % (76.0 * nnzb / 1e6)},
                "spmv": spmv, "vector_ops": vops, "solves": solves, "peak_gbs": peak,
                "peak_source": peak_src,
                "clocks": clk}
        print(json.dumps(line), flush=True)


# ------------------------------------------------------------ batched meshes

def gen_meshes(specs):
    """specs: (n, split, jitter, seed) -> [(crd, tet, ref)], generated in
    parallel (the library calls release the GIL)."""
    import gmlib_gb300 as G
    from concurrent.futures import ThreadPoolExecutor

    def one(sp):
        n, split, jit, seed = sp
        return G.cube_mesh(n, split=split, jitter=jit, seed=seed)
    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        return list(ex.map(one, specs))


# ---------------------------------------------------- plain tet quality (C1)

Q_N, Q_JITTER, Q_SEED = 32, 0.25, 12345


def run_quality(args, dist):
    """The plain tet-quality configuration: 32^3-hex cube, Kuhn split
    (196,608 tets, 35,937 vertices), interior vertices jittered by +-0.25h
    (seed 12345), Hilbert order.  One pass computes the mean-ratio quality of
    every tet with min/argmin, max/argmax, the sum, the 64-bin histogram and
    the FP64-decided inverted flags (GmlxQualityStats).
    value: tets/s of the pass, CUDA events around each launch, with the L2
    flushed between launches by scaling a 256 MB vector (the mesh alone,
    4.5 MB, would stay in the 129 MB L2).  The same measure written as a
    user body, compiled by GmlCompileKernel and reduced by GmlxReduceArg, is
    reported beside it.  e2e: coordinates up, the pass, the statistics down,
    through the C ABI with host buffers.  CPU: the FP64 serial oracle on one
    core."""
    import gmlib_gb300 as G
    n = args.n if args.n != N_HEX else Q_N
    crd, tet, ref = G.cube_mesh(n, split=0, jitter=Q_JITTER, seed=Q_SEED)
    nv, nt = len(crd), len(tet)
    h = 1.0 / n
    g = G.lib.GmlInit(dist.local)
    if not g:
        raise SystemExit("GmlInit failed")
    G.lib.GmlxSetTiming(g, 0)
    G.lib.GmlNewParameters(g, len(P2_PARAMS), P2_PARAMS)
    v, t = G.upload_mesh(g, crd, tet, ref)
    if G.lib.GmlxMeshSetup(g, 1) != 1:
        raise SystemExit("GmlxMeshSetup failed")
    flush = G.lib.GmlNewVector(g, 16 << 20, 4, None, G.GmlFlt)     # 256 MB
    if flush <= 0:
        raise SystemExit("cannot allocate the L2 flush vector")
    one = ctypes.c_double(1.0)
    res = G.GmlxQuality()

    def timed(launch, k):
        e0, e1 = G.lib.GmlxEventCreate(), G.lib.GmlxEventCreate()
        tot = 0.0
        for _ in range(k):
            G.lib.GmlScaleVec(g, flush, ctypes.byref(one))
            G.lib.GmlxEventRecord(g, e0)
            launch()
            G.lib.GmlxEventRecord(g, e1)
            tot += G.lib.GmlxEventElapsed(e0, e1)
        return tot / k

    def native():
        G.lib.GmlxQualityStats(g, h, 0, None)

    for _ in range(max(args.warmup, 3)):
        native()
    clocks = Clocks(dist.local)
    dist.barrier()
    clocks.start()
    per = dist.max(timed(native, args.steps))
    clk = clocks.stop()
    if G.lib.GmlxQualityStats(g, h, 0, ctypes.byref(res)) != 1:
        raise SystemExit("GmlxQualityStats failed")

    # the same measure as a user body through the reference API
    qidx = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
    k = G.compile_kernel(g, G.mean_ratio_body(), "mean_ratio", G.GmlTetrahedra,
                         [(v, G.GmlReadMode, 0), (qidx, G.GmlWriteMode, 0)])
    if not k:
        raise SystemExit("mean-ratio body did not compile")
    for _ in range(max(args.warmup, 3) + 8):            # block-size calibration included
        G.lib.GmlLaunchKernel(g, k)
    per_gen = dist.max(timed(lambda: G.lib.GmlLaunchKernel(g, k), args.steps))
    mn, mx = ctypes.c_float(), ctypes.c_float()
    imn, imx = ctypes.c_int(), ctypes.c_int()
    G.lib.GmlxReduceArg(g, qidx, ctypes.byref(mn), ctypes.byref(imn), ctypes.byref(mx),
                        ctypes.byref(imx))
    tr = []
    for i in range(args.steps + 3):
        ts = time.perf_counter()
        G.lib.GmlLaunchKernel(g, k)
        G.lib.GmlxReduceArg(g, qidx, ctypes.byref(mn), ctypes.byref(imn), ctypes.byref(mx),
                            ctypes.byref(imx))
        if i >= 3:
            tr.append(time.perf_counter() - ts)

    # end to end: coordinates up, the pass, the statistics down
    host_crd = np.ascontiguousarray(crd)
    e2e_t = []
    for i in range(args.e2e_steps + 2):
        ts = time.perf_counter()
        G.lib.GmlxSetData(g, v, G.as_ptr(host_crd), host_crd.nbytes)
        G.lib.GmlxQualityStats(g, h, 0, ctypes.byref(res))
        if i >= 2:
            e2e_t.append(time.perf_counter() - ts)
    e2e_s = dist.max(statistics.median(e2e_t))
    G.lib.GmlStop(g)

    byts = 16.0 * nt + 16.0 * nv + 4.0 * ((nt + 31) // 32)
    peak, peak_src = peak_hbm()
    cpu = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        import oracle as O
        ts_ = []
        for _ in range(4):
            ts = time.perf_counter()
            q, _, _, _ = O.quality_stats(crd, tet)
            int(np.argmin(q)), int(np.argmax(q))
            ts_.append(time.perf_counter() - ts)
        tc = statistics.median(ts_[1:])
        cpu = {"value": round(nt / tc / 1e6, 3), "unit": "M tets/s", "cores": 1, "kind": "port",
               "sample": "FP64 serial oracle (quality, histogram, flags, argmin/argmax) on the "
                         "whole mesh, median of 3 after 1 warm-up"}
    if dist.rank == 0:
        line = {"metric": "tet qualities per second (quality + min/max/argmin pass)",
                "value": round(dist.world * nt / per / 1e6, 2), "unit": "M tets/s",
                "n_gpus": dist.world, "steps": args.steps, "warmup": max(args.warmup, 3),
                "ms_per_step": round(per * 1e3, 5), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": "mean-ratio quality + min/max/argmin, %d^3-hex cube, "
                                       "Kuhn split" % n,
                           "tets": nt, "vertices": nv, "jitter": Q_JITTER, "seed": Q_SEED,
                           "l2": "flushed between launches (256 MB vector scale); the mesh "
                                 "(%.1f MB) is smaller than L2" % (byts / 1e6)},
                "gpu_launches": 2 * args.steps,
                "roofline": {"bound": "hbm", "kernel": "tet_quality_tma_kernel",
                             "achieved": round(byts / per / 1e9, 1), "peak": peak, "unit": "GB/s",
                             "frac": round(byts / per / 1e9 / peak, 4), "traffic": None,
                             "algorithmic_bytes_per_launch": byts,
                             "mean_launch_us": round(per * 1e6, 2), "peak_source": peak_src,
                             "note": "a 4.5 MB pass is latency-bound; the fraction is context"},
                "generated": {"kernel": "gmlib_gb300/kernels/mean_ratio.cl via GmlCompileKernel",
                              "mean_launch_us": round(per_gen * 1e6, 2),
                              "launch_plus_reduce_arg_us": round(statistics.median(tr) * 1e6, 1),
                              "min": mn.value, "argmin": imn.value},
                "e2e": {"value": round(dist.world * nt / e2e_s / 1e6, 2), "unit": "M tets/s",
                        "h2d_bytes_per_step": host_crd.nbytes,
                        "d2h_bytes_per_step": ctypes.sizeof(G.GmlxQuality),
                        "ms_per_step": round(e2e_s * 1e3, 4)},
                "cpu_baseline": cpu, "clocks": clk,
                "result_check": {"min": res.MinQal, "argmin": res.MinIdx, "max": res.MaxQal,
                                 "argmax": res.MaxIdx, "inverted": res.NmbInv,
                                 "generated_argmin_agrees": imn.value == res.MinIdx}}
        print(json.dumps(line), flush=True)


# ------------------------------------------- NodeSmoothing flow (reference API)

def kernel_body(name):
    with open(os.path.join(ROOT, "tests", "kernels", name), "rb") as f:
        return f.read()


def nodesmooth_measure(G, dev, n, steps, warmup, dsort, dist):
    """The NodeSmoothing flow on the n^3-hex cube (see run_nodesmooth);
    returns the wall time of a flow (median of `steps`), the per-kernel
    device times and the flow's results."""
    crd, tet, ref = G.cube_mesh(n, split=SPLIT, jitter=JITTER, seed=SEED, degree_sort=dsort)
    nv, nt = len(crd), len(tet)
    g = G.lib.GmlInit(dev)
    if not g:
        raise SystemExit("GmlInit failed")
    G.lib.GmlxSetTiming(g, 0)
    G.lib.GmlNewParameters(g, len(P2_PARAMS), P2_PARAMS)
    v, t = G.upload_mesh(g, crd, tet, ref)
    qal = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
    opt = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 4, G.GmlFlt4, b"OptCrd")
    res = G.lib.GmlNewSolutionData(g, G.GmlVertices, 1, G.GmlFlt, b"res")
    kq = G.compile_kernel(g, kernel_body("tet_quality.cl"), "quality", G.GmlTetrahedra,
                          [(v, G.GmlReadMode, 0), (qal, G.GmlWriteMode, 0)])
    ks = G.compile_kernel(g, kernel_body("optimal_points.cl"), "scatter", G.GmlTetrahedra,
                          [(v, G.GmlReadMode, 0), (opt, G.GmlWriteMode, 0)])
    kg = G.compile_kernel(g, kernel_body("relax_to_points.cl"), "gather", G.GmlVertices,
                          [(res, G.GmlWriteMode, 0), (opt, G.GmlReadMode | G.GmlVoyeurs, 0),
                           (v, G.GmlReadMode | G.GmlWriteMode, 0)])
    if not (kq and ks and kg):
        raise SystemExit("NodeSmoothing bodies did not compile")
    host_crd = np.ascontiguousarray(crd)

    def flow():
        G.lib.GmlLaunchKernel(g, kq)
        q0 = G.reduce(g, qal, G.GmlSum)
        r = 0.0
        for _ in range(10):
            G.lib.GmlLaunchKernel(g, ks)
            G.lib.GmlLaunchKernel(g, kg)
            r = G.reduce(g, res, G.GmlSum)
        G.lib.GmlLaunchKernel(g, kq)
        return q0, r, G.reduce(g, qal, G.GmlSum)

    for _ in range(max(warmup, 3)):               # includes the block-size calibration
        G.lib.GmlxSetData(g, v, G.as_ptr(host_crd), host_crd.nbytes)
        flow()
    clocks = Clocks(dev)
    dist.barrier()
    clocks.start()
    walls = []
    for _ in range(steps):
        G.lib.GmlxSetData(g, v, G.as_ptr(host_crd), host_crd.nbytes)
        G.lib.GmlxSynchronize(g)
        ts = time.perf_counter()
        q0, r, q1 = flow()
        walls.append(time.perf_counter() - ts)
    clk = clocks.stop()
    wall = dist.max(statistics.median(walls))

    # per-kernel device times, back-to-back launches on the instance's stream
    e0, e1 = G.lib.GmlxEventCreate(), G.lib.GmlxEventCreate()
    per = {}
    for name, k in (("scatter", ks), ("gather", kg), ("quality", kq)):
        G.lib.GmlxEventRecord(g, e0)
        for _ in range(20):
            G.lib.GmlLaunchKernel(g, k)
        G.lib.GmlxEventRecord(g, e1)
        per[name] = dist.max(G.lib.GmlxEventElapsed(e0, e1) / 20)
    blk = {name: G.lib.GmlxKernelBlockSize(g, k) for name, k in
           (("scatter", ks), ("gather", kg), ("quality", kq))}
    regs = {name: G.lib.GmlxKernelRegisters(g, k) for name, k in
            (("scatter", ks), ("gather", kg), ("quality", kq))}
    G.lib.GmlStop(g)

    # algorithmic bytes: scatter 16T (tets) + 16V (coordinates) + 64T (points
    # out); gather 16T (ball entries) + 4V (degrees) + 64T (points in) + 32V
    # (coordinates in and out) + 4V (res); quality 16T + 16V + 4T; sums 4 per line
    kb = {"scatter": 80.0 * nt + 16.0 * nv, "gather": 80.0 * nt + 40.0 * nv,
          "quality": 20.0 * nt + 16.0 * nv}
    flow_bytes = 10 * (kb["scatter"] + kb["gather"] + 4.0 * nv) + 2 * (kb["quality"] + 4.0 * nt)
    peak, peak_src = peak_hbm()
    kern = {k: {"mean_launch_us": round(per[k] * 1e6, 2), "block": blk[k], "registers": regs[k],
                "algorithmic_bytes": kb[k], "achieved": round(kb[k] / per[k] / 1e9, 1),
                "frac": round(kb[k] / per[k] / 1e9 / peak, 4)} for k in per}
    return {"nv": nv, "nt": nt, "tet": tet, "wall": wall, "flow_bytes": flow_bytes,
            "kernels": kern, "peak": peak, "peak_src": peak_src, "clocks": clk,
            "q0": q0, "q1": q1, "r": r, "kb": kb}


def run_nodesmooth(args, dist):
    """The reference's NodeSmoothing example flow through the reference API on
    the smoothing mesh (128^3-hex cube, reflected split): the tet quality
    body and a sum reduction, then 10 x (scatter: 4 optimal apex points per
    tet; gather: mean of the ball's points facing each vertex through the
    vertex -> tet ball with voyeurs, 0.2 relaxation; sum of the squared
    moves), then the quality and its sum again.  Each GmlReduceVector
    returns its value to the host, as in the example.  The bodies are this
    repository's restatements of the example's scatter, gather and quality
    kernels (tests/kernels).
    value: algorithmic bytes of the flow / wall time of the flow (GB/s);
    per-kernel device times with CUDA events over back-to-back launches."""
    import gmlib_gb300 as G
    n = args.n
    dsort = 32 if args.degree_sort else 0
    m = nodesmooth_measure(G, dist.local, n, args.steps, args.warmup, dsort, dist)
    nv, nt, kern = m["nv"], m["nt"], m["kernels"]
    if dist.rank == 0:
        line = {"metric": "NodeSmoothing flow through the reference API, GB/s",
                "value": round(dist.world * m["flow_bytes"] / m["wall"] / 1e9, 1), "unit": "GB/s",
                "n_gpus": dist.world, "steps": args.steps, "warmup": max(args.warmup, 3),
                "ms_per_step": round(m["wall"] * 1e3, 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": "NodeSmoothing example flow (quality + sum, 10 x "
                                       "(scatter, gather, residual sum), quality + sum), "
                                       "%d^3-hex cube, reflected split" % n,
                           "numbering": "Hilbert, then vertices in at most 32 tets first "
                                        "(GmlxDegreeSort)" if dsort else "Hilbert",
                           "tets": nt, "vertices": nv,
                           "vertex_tet_degrees": degree_summary([m["tet"]]),
                           "l2": "inputs larger than L2 (OptCrd alone is %.0f MB)" % (64e-6 * nt),
                           "step": "wall clock of the flow, host reductions included; the "
                                   "coordinates are re-uploaded before each step, outside it"},
                "gpu_launches": args.steps * (22 + 12),
                "roofline": {"bound": "hbm", "kernel": "gather (generated)",
                             "achieved": kern["gather"]["achieved"], "peak": m["peak"],
                             "unit": "GB/s", "frac": kern["gather"]["frac"], "traffic": None,
                             "algorithmic_bytes_per_launch": m["kb"]["gather"],
                             "mean_launch_us": kern["gather"]["mean_launch_us"],
                             "peak_source": m["peak_src"]},
                "kernels": kern, "clocks": m["clocks"],
                "result_check": {"mean_quality_before": m["q0"] / nt,
                                 "mean_quality_after": m["q1"] / nt,
                                 "last_residual": m["r"]}}
        print(json.dumps(line), flush=True)


# ------------------------------------------------------------- P2 quality

P2_FLOPS = 1612.0         # flops per P2 tet, as counted by examples/P2Quality
P2_PARAMS = b"typedef struct {\n   int   foo;\n   float res;\n}GmlParSct;\n"


def run_p2(args, dist):
    """The reference's P2Quality flow on the n^3-hex cube with quadratic tets
    (Kuhn split, jitter 0.15h, mid-edge nodes moved by up to 0.05h): the
    P2 quality body (gmlib_gb300/kernels/p2_quality.cl) compiled by
    GmlCompileKernel, reading VerCrd through TetVer and MidCrd through the
    tet -> edge downlink, one quality per tet.
    value: P2 tet qualities per second, device time with CUDA events over K
    launches, inputs resident (larger than L2); e2e: the same through the C
    ABI with the vertex coordinates and mid-edge nodes uploaded and the
    qualities downloaded every step."""
    import gmlib_gb300 as G
    n = args.n
    t0 = time.perf_counter()
    crd, tet, edges, mid, tedg = G.p2_mesh(n, split=0, jitter=0.15, curve=0.05, seed=SEED)
    tgen = time.perf_counter() - t0
    nv, nt, ne = len(crd), len(tet), len(edges)
    g = G.lib.GmlInit(dist.local)
    if not g:
        raise SystemExit("GmlInit failed")
    G.lib.GmlxSetTiming(g, 0)
    G.lib.GmlNewParameters(g, len(P2_PARAMS), P2_PARAMS)
    v, t, e, m = G.upload_p2(g, crd, tet, edges, mid)
    q = G.lib.GmlNewSolutionData(g, G.GmlTetrahedra, 1, G.GmlFlt, b"qal")
    k = G.compile_kernel(g, G.p2_body(), "p2quality", G.GmlTetrahedra,
                         [(v, G.GmlReadMode, 0), (m, G.GmlReadMode, 0), (q, G.GmlWriteMode, 0)])
    if not k:
        raise SystemExit("P2 kernel did not compile")
    for _ in range(max(args.warmup, 3)):
        if G.lib.GmlLaunchKernel(g, k) != 1:
            raise SystemExit("launch failed")
    G.lib.GmlxSynchronize(g)
    e0, e1 = G.lib.GmlxEventCreate(), G.lib.GmlxEventCreate()
    clocks = Clocks(dist.local)
    dist.barrier()
    clocks.start()
    time.sleep(0.3)
    G.lib.GmlxEventRecord(g, e0)
    for _ in range(args.steps):
        G.lib.GmlLaunchKernel(g, k)
    G.lib.GmlxEventRecord(g, e1)
    dev_s = dist.max(G.lib.GmlxEventElapsed(e0, e1))
    clk = clocks.stop()
    per = dev_s / args.steps
    qg = G.get_data(g, q, np.float32, nt)
    sumq = G.reduce(g, q, G.GmlSum)
    minq = G.reduce(g, q, G.GmlMin)
    # algorithmic bytes of one launch: TetVer and the 6 used edge indices per
    # tet, each vertex and mid-edge node once, the quality out
    byts = 16.0 * nt + 24.0 * nt + 16.0 * nv + 16.0 * ne + 4.0 * nt
    achieved = byts / per / 1e9
    peak, peak_src = peak_hbm()

    # end to end: coordinates and mid-edge nodes up, qualities down
    host_crd, host_mid = np.ascontiguousarray(crd), np.ascontiguousarray(mid)
    out = np.empty(nt, np.float32)
    e2e_t = []
    for i in range(args.e2e_steps + 2):
        ts = time.perf_counter()
        G.lib.GmlxSetData(g, v, G.as_ptr(host_crd), host_crd.nbytes)
        G.lib.GmlxSetData(g, m, G.as_ptr(host_mid), host_mid.nbytes)
        G.lib.GmlLaunchKernel(g, k)
        G.lib.GmlxGetData(g, q, G.as_ptr(out), out.nbytes)
        if i >= 2:
            e2e_t.append(time.perf_counter() - ts)
    e2e_s = dist.max(statistics.median(e2e_t))
    G.lib.GmlStop(g)

    cpu = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        import oracle as O
        ns = min(nt, 2_000_000)
        O.p2_quality(crd, mid, tet[:1000], tedg[:1000])        # warm the pool
        ts = time.perf_counter()
        O.p2_quality(crd, mid, tet[:ns], tedg[:ns])
        tc = time.perf_counter() - ts
        cpu = {"value": round(ns / tc / 1e6, 3), "unit": "M P2 tets/s",
               "cores": os.cpu_count(), "kind": "port",
               "sample": "FP64 oracle (OpenMP) on the first %d tets of the same mesh" % ns}
    if dist.rank == 0:
        line = {"metric": "P2 tet qualities per second", "value": round(dist.world * nt / per / 1e6, 2),
                "unit": "M P2 tets/s", "n_gpus": dist.world, "steps": args.steps,
                "warmup": max(args.warmup, 3), "ms_per_step": round(per * 1e3, 4),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic",
                "config": {"workload": "P2 tet quality (examples/P2Quality flow), %d^3-hex cube, "
                                       "Kuhn split, curved mid-edge nodes" % n,
                           "tets": nt, "vertices": nv, "edges": ne,
                           "l2": "inputs larger than L2 (%.0f MB per launch)" % (byts / 1e6),
                           "mesh_generation_s": round(tgen, 1)},
                "gpu_launches": args.steps,
                "roofline": {"bound": "hbm", "kernel": "p2quality (generated)",
                             "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                             "frac": round(achieved / peak, 4), "traffic": None,
                             "algorithmic_bytes_per_launch": byts,
                             "gflops": round(P2_FLOPS * nt / per / 1e9, 1),
                             "mean_launch_us": round(per * 1e6, 2), "peak_source": peak_src},
                "e2e": {"value": round(dist.world * nt / e2e_s / 1e6, 2), "unit": "M P2 tets/s",
                        "h2d_bytes_per_step": host_crd.nbytes + host_mid.nbytes,
                        "d2h_bytes_per_step": out.nbytes, "ms_per_step": round(e2e_s * 1e3, 3)},
                "cpu_baseline": cpu, "clocks": clk,
                "result_check": {"mean_quality": sumq / nt, "min_quality": minq,
                                 "min_matches_download": bool(minq == float(qg.min()))}}
        print(json.dumps(line), flush=True)


def batch_measure(G, dev, nmesh, steps, warmup):
    """Config-4 batch: nmesh jittered tet cubes, hexes per side log-uniform in
    [10, 80], reflected split, Hilbert order; 5 sweeps + quality statistics
    (min/argmin) per mesh, through one persistent tile-queue launch (CUDA
    graph, tuned tiles) and through the per-mesh launch loop, `steps` runs of
    each after `warmup`."""
    rng = np.random.default_rng(SEED)
    ns = np.exp(rng.uniform(np.log(10), np.log(80), nmesh)).astype(int)
    t0 = time.time()
    ms = gen_meshes([(int(n), 1, 0.3, SEED + i) for i, n in enumerate(ns)])
    tgen = time.time() - t0
    nv = np.array([len(m[0]) for m in ms], np.int32)
    nt = np.array([len(m[1]) for m in ms], np.int32)
    degrees = degree_summary([m[1] for m in ms])
    h = 1.0 / ns.astype(np.float64)
    g = G.lib.GmlInit(dev)
    G.lib.GmlxSetTiming(g, 0)
    if G.lib.GmlxBatchCreate(g, len(ms), G.as_ptr(nv), G.as_ptr(nt), G.as_ptr(h)) != 1:
        raise SystemExit("GmlxBatchCreate failed")
    for i, (crd, tet, ref) in enumerate(ms):
        G.lib.GmlxBatchSetMesh(g, i, G.as_ptr(crd), G.as_ptr(ref), G.as_ptr(tet))
    del ms
    if G.lib.GmlxBatchSetup(g, 1) != 1:
        raise SystemExit("GmlxBatchSetup failed")
    sweeps, om = 5, ctypes.c_float(OMEGA)
    G.lib.GmlxBatchTune(g, sweeps, om)
    ts_, tt_, gr_, ntile, wt_ = (ctypes.c_int() for _ in range(5))
    res = (G.GmlxQuality * nmesh)()
    e0, e1 = G.lib.GmlxEventCreate(), G.lib.GmlxEventCreate()
    out = {}
    clocks = Clocks(dev)
    clocks.start()
    for name, mode in (("queue", G.GmlxBatchQueue), ("loop", G.GmlxBatchLoop)):
        for _ in range(warmup):
            G.lib.GmlxBatchRun(g, sweeps, om, mode, None)
        G.lib.GmlxSynchronize(g)
        G.lib.GmlxEventRecord(g, e0)
        for _ in range(steps):
            if G.lib.GmlxBatchRun(g, sweeps, om, mode, None) != 1:
                raise SystemExit("GmlxBatchRun failed")
        G.lib.GmlxEventRecord(g, e1)
        t = G.lib.GmlxEventElapsed(e0, e1) / steps
        out[name] = {"ms_per_run": round(t * 1e3, 3), "meshes_per_s": round(nmesh / t, 1)}
    clk = clocks.stop()
    G.lib.GmlxBatchRun(g, sweeps, om, G.GmlxBatchQueue, res)
    G.lib.GmlxBatchInfo(g, ctypes.byref(ts_), ctypes.byref(tt_), ctypes.byref(gr_),
                        ctypes.byref(ntile), ctypes.byref(wt_))
    stored, used, mx = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_int()
    G.lib.GmlxMeshBallInfo(g, ctypes.byref(stored), ctypes.byref(used), ctypes.byref(mx))
    G.lib.GmlxEventDestroy(e0)
    G.lib.GmlxEventDestroy(e1)
    G.lib.GmlStop(g)
    vpad = float(sum((int(v) + 255) // 256 * 256 for v in nv))
    byts = sweeps * (36.0 * vpad + 4.0 * used.value) + 16.0 * nt.sum() + 16.0 * vpad \
        + 4.0 * sum((int(t) + 31) // 32 for t in nt)
    peak, _ = peak_hbm()
    tq = out["queue"]["ms_per_run"] / 1e3
    info = {"tets": int(nt.sum()), "vertices": int(nv.sum()), "sweeps": sweeps,
            "degrees": degrees, "generation_s": round(tgen, 1),
            "speedup_vs_loop": round(out["loop"]["ms_per_run"] / out["queue"]["ms_per_run"], 2),
            "tiles": {"claimed_per": "warp" if wt_.value else "block",
                      "slices_per_sweep_tile": ts_.value, "tets_per_quality_tile": tt_.value,
                      "grid": gr_.value, "tiles": ntile.value},
            "roofline": {"bound": "hbm", "algorithmic_bytes_per_run": byts,
                         "achieved": round(byts / tq / 1e9, 1), "peak": peak,
                         "frac": round(byts / tq / 1e9 / peak, 4), "unit": "GB/s"},
            "min_quality": float(min(r.MinQal for r in res)), "clocks": clk}
    return out, info


def run_batch(args, dist):
    """The batch configuration (batch_measure) as the bench line, meshes/s
    over --steps runs of each path."""
    import gmlib_gb300 as G
    out, info = batch_measure(G, dist.local, args.meshes, args.steps, args.warmup)
    if dist.rank == 0:
        line = {"metric": "batched meshes/s (5 sweeps + quality + min per mesh)",
                "value": out["queue"]["meshes_per_s"], "unit": "meshes/s", "n_gpus": dist.world,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                "dtype": "f32", "data": "synthetic",
                "config": {"workload": "%d jittered tet cubes, hexes per side log-uniform in "
                                       "[10, 80], reflected split" % args.meshes,
                           "tets": info["tets"], "vertices": info["vertices"],
                           "sweeps": info["sweeps"], "vertex_tet_degrees": info["degrees"],
                           "generation_s": info["generation_s"]},
                "queue": out["queue"], "loop": out["loop"],
                "speedup_vs_loop": info["speedup_vs_loop"], "tiles": info["tiles"],
                "roofline": info["roofline"], "min_quality": info["min_quality"],
                "clocks": info["clocks"]}
        print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ serving

SERVE_BUCKETS = 12


SERVE_P99_MS = 100.0                       # the stated p99 of the capacity sweep
SERVE_SWEEP_RATES = (25, 50, 100, 150, 200, 300, 400, 600)


def serve_in_fresh_process(dev):
    """Config 5 for the default line (10 s at 200 req/s, with the p99 sweep
    in 4-s runs), measured by `bench.py --workload serve` in a process of its own: serve
    runs that follow other heavy workloads in one process measure slower
    (host-side state), so the default line does not inherit the others'."""
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--workload", "serve",
           "--duration", "10", "--sweep-seconds", "4"]
    env = dict(os.environ, LOCAL_RANK=str(dev), RANK="0", WORLD_SIZE="1")
    try:
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                           env=env, timeout=900)
    except subprocess.TimeoutExpired:
        return None
    for line in r.stdout.splitlines():
        if line.startswith("{"):
            d = json.loads(line)
            c = d["capacity_at_p99"]
            return {"batching": d["batching"], "serial_prefix": d["serial_prefix"],
                    "capacity_saturated": d["capacity_saturated"], "capacity_at_p99": c,
                    "same": int(d["same_result_alone_and_in_mix"].split()[0]),
                    "nser": int(d["same_result_alone_and_in_mix"].split()[-1])}
    sys.stderr.write("the serve run failed:\n" + r.stdout[-2000:] + r.stderr[-2000:] + "\n")
    return None


class ServePool:
    """Config-5 targets: meshes of 1e4..1e7 tets (log-uniform buckets, config-2
    construction) and the SPD block systems of their vertex graphs (config-3
    construction), generated in parallel (the library calls release the GIL)."""

    def __init__(self, G):
        from concurrent.futures import ThreadPoolExecutor
        self.G = G
        self.ns = np.unique(np.round(np.exp(np.linspace(np.log((1e4 / 6) ** (1 / 3)),
                                                        np.log((1e7 / 6) ** (1 / 3)),
                                                        SERVE_BUCKETS))).astype(int))
        t0 = time.time()
        self.meshes = gen_meshes([(int(n), 1, 0.3, SEED + i) for i, n in enumerate(self.ns)])
        with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
            self.systems = list(ex.map(lambda a: G.cube_spd(int(a[1]), 0, seed=SEED + a[0]),
                                       enumerate(self.ns)))
        self.tgen = time.time() - t0
        self.logt = np.log(6.0 * self.ns.astype(np.float64) ** 3)

    def bucket(self, x):
        return int(np.argmin(np.abs(self.logt - x)))

    def register(self, server, cls, b):
        G = self.G
        if cls == 0:
            crd, tet, ref = self.meshes[b]
            return G.lib.GmlxServeAddMesh(server, len(crd), G.as_ptr(crd), G.as_ptr(ref),
                                          len(tet), G.as_ptr(tet), 1.0 / self.ns[b])
        lin, col, val, rhs = self.systems[b]
        return G.lib.GmlxServeAddSystem(server, len(lin) - 1, len(col), G.as_ptr(lin),
                                        G.as_ptr(col), G.as_ptr(val), G.as_ptr(rhs))


def serve_trace(G, pool, srv, nreq, rate, rng):
    """Poisson arrivals at `rate`; 50/30/20 quality / smoothing / CG; a request
    targets a known target with probability 0.5, else registers a new one.
    Returns (requests, [(class, bucket)] registered in order)."""
    added = []
    req = (G.GmlxRequest * max(nreq, 1))()
    seen = {0: [], 1: []}
    t = 0.0
    for i in range(nreq):
        t += rng.exponential(1.0 / rate)
        u = rng.random()
        kind = G.GmlxReqQuality if u < 0.5 else (G.GmlxReqSmooth if u < 0.8 else G.GmlxReqSolve)
        cls = 1 if kind == G.GmlxReqSolve else 0
        if seen[cls] and rng.random() < 0.5:
            target = int(rng.choice(seen[cls]))
        else:
            b = pool.bucket(rng.uniform(np.log(1e4), np.log(1e7)))
            target = pool.register(srv, cls, b)
            added.append((cls, b))
            seen[cls].append(target)
        req[i].kind, req[i].target, req[i].arrival = kind, target, t
    return req, added


def serve_stats(st):
    return {"completed": st.completed, "failed": st.failed, "seconds": round(st.seconds, 2),
            "throughput_rps": round(st.throughput, 2), "p50_ms": round(st.p50 * 1e3, 2),
            "p99_ms": round(st.p99 * 1e3, 2), "max_ms": round(st.max * 1e3, 2),
            "loads": st.loads, "evictions": st.evictions,
            "peak_resident_gb": round(st.peak_bytes / 1e9, 2)}


SERVE_SWEEP_WARM = 2.0                     # seconds of arrivals before the measured ones


def serve_p99_sweep(G, pool, dev, duration, rates, p99_ms):
    """Highest arrival rate each path sustains with its p99 latency at or
    below p99_ms.  For each rate in increasing order, a fresh server (same
    pool, nothing resident) replays SERVE_SWEEP_WARM + `duration` s of the
    config-5 trace at that rate; the latencies of the requests arriving in
    the last `duration` s count (the first seconds are the server filling
    up).  A path stops at the first rate whose p99 exceeds the target or
    that leaves requests unfinished."""
    out = {}
    for mode, name in ((G.GmlxServeBatching, "batching"), (G.GmlxServeSerial, "serial")):
        runs, best = [], 0.0
        for rate in rates:
            srv = G.lib.GmlxServeNew(dev, 150e9, 8)
            nreq = int(rate * (SERVE_SWEEP_WARM + duration))
            req, _ = serve_trace(G, pool, srv, nreq, rate, np.random.default_rng(SEED))
            st = G.GmlxServeStats()
            G.lib.GmlxServeRun(srv, req, nreq, mode, ctypes.byref(st))
            G.lib.GmlxServeFree(srv)
            lat = sorted(req[i].finish - req[i].arrival for i in range(nreq)
                         if req[i].arrival >= SERVE_SWEEP_WARM and req[i].status == 1)
            nmeas = sum(1 for i in range(nreq) if req[i].arrival >= SERVE_SWEEP_WARM)
            p99 = lat[int(0.99 * (len(lat) - 1))] if lat else float("inf")
            p50 = lat[len(lat) // 2] if lat else float("inf")
            ok = st.failed == 0 and len(lat) == nmeas and p99 * 1e3 <= p99_ms
            runs.append({"rate": rate, "p50_ms": round(p50 * 1e3, 2), "p99_ms": round(p99 * 1e3, 2),
                         "throughput_rps": round(st.throughput, 2), "meets_p99": bool(ok)})
            if not ok:
                break
            best = float(rate)
        out[name] = {"max_rate_at_p99": best, "runs": runs}
    if out["serial"]["max_rate_at_p99"] > 0:
        out["batching_over_serial"] = round(out["batching"]["max_rate_at_p99"]
                                            / out["serial"]["max_rate_at_p99"], 2)
    else:
        # the serial path misses the target at the lowest rate tried, so its
        # sustainable rate is below that rate
        out["batching_over_serial_at_least"] = round(out["batching"]["max_rate_at_p99"]
                                                     / rates[0], 2)
    out["p99_target_ms"] = p99_ms
    out["seconds_per_run"] = duration
    out["warm_seconds"] = SERVE_SWEEP_WARM
    return out


def serve_measure(G, dev, rate, duration, serial_requests, saturate, sweep_s, pool=None):
    """Config 5 (see run_serve); returns the measured dict."""
    pool = pool or ServePool(G)
    rng = np.random.default_rng(SEED)
    srv = G.lib.GmlxServeNew(dev, 150e9, 8)
    nreq = int(rate * duration)
    req, added = serve_trace(G, pool, srv, nreq, rate, rng)
    stb = G.GmlxServeStats()
    clocks = Clocks(dev)
    clocks.start()
    G.lib.GmlxServeRun(srv, req, nreq, G.GmlxServeBatching, ctypes.byref(stb))
    clk = clocks.stop()
    nser = min(nreq, serial_requests)
    ser = (G.GmlxRequest * max(nser, 1))()
    for i in range(nser):
        ser[i].kind, ser[i].target, ser[i].arrival = req[i].kind, req[i].target, req[i].arrival
    sts = G.GmlxServeStats()
    G.lib.GmlxServeRun(srv, ser, nser, G.GmlxServeSerial, ctypes.byref(sts))
    # capacity: the first `saturate` requests of the trace all due at t = 0,
    # through each path (requests/s the path sustains when never idle), on a
    # second server with the same targets and none of them resident
    nsat = min(nreq, saturate)
    cap = {}
    srv2 = G.lib.GmlxServeNew(dev, 150e9, 8)
    for cls, b in added:
        pool.register(srv2, cls, b)
    for mode, name in ((G.GmlxServeBatching, "batching"), (G.GmlxServeSerial, "serial")):
        sat = (G.GmlxRequest * max(nsat, 1))()
        for i in range(nsat):
            sat[i].kind, sat[i].target, sat[i].arrival = req[i].kind, req[i].target, 0.0
        stc = G.GmlxServeStats()
        G.lib.GmlxServeRun(srv2, sat, nsat, mode, ctypes.byref(stc))
        cap[name] = {"requests": nsat, "completed": stc.completed, "seconds": round(stc.seconds, 3),
                     "throughput_rps": round(stc.throughput, 2)}
    G.lib.GmlxServeFree(srv2)
    if cap["serial"]["throughput_rps"] > 0:
        cap["batching_over_serial"] = round(cap["batching"]["throughput_rps"]
                                            / cap["serial"]["throughput_rps"], 2)

    def breakdown(reqs, n):
        """per kind: mean queueing delay (start - arrival) and service time
        (finish - start), split by whether the request loaded its target"""
        out = {}
        firsts = set()
        loaded = []
        for i in range(n):
            t = reqs[i].target
            loaded.append(t not in firsts)
            firsts.add(t)
        names = {G.GmlxReqQuality: "quality", G.GmlxReqSmooth: "smooth", G.GmlxReqSolve: "solve"}
        for k, name in names.items():
            for cold in (True, False):
                idx = [i for i in range(n) if reqs[i].kind == k and loaded[i] == cold
                       and reqs[i].status == 1]
                if not idx:
                    continue
                q = [reqs[i].start - reqs[i].arrival for i in idx]
                sv = sorted(reqs[i].finish - reqs[i].start for i in idx)
                out["%s_%s" % (name, "load" if cold else "resident")] = {
                    "n": len(idx), "queue_ms": round(1e3 * sum(q) / len(q), 2),
                    "service_ms": round(1e3 * sum(sv) / len(sv), 2),
                    "service_p99_ms": round(1e3 * sv[int(0.99 * (len(sv) - 1))], 2)}
        return out
    bd = breakdown(req, nreq)
    same = sum(1 for i in range(nser)
               if req[i].status == 1 and ser[i].status == 1
               and (req[i].NmbIte, req[i].RelRes, req[i].qal.MinQal, req[i].qal.MinIdx)
               == (ser[i].NmbIte, ser[i].RelRes, ser[i].qal.MinQal, ser[i].qal.MinIdx))
    G.lib.GmlxServeFree(srv)
    sweep = serve_p99_sweep(G, pool, dev, sweep_s, SERVE_SWEEP_RATES, SERVE_P99_MS) \
        if sweep_s > 0 else None
    return {"pool": pool, "batching": serve_stats(stb), "batching_by_kind": bd,
            "serial_prefix": serve_stats(sts), "capacity_saturated": cap,
            "capacity_at_p99": sweep, "same": same, "nser": nser, "clocks": clk}


def run_serve(args, dist):
    """Poisson arrivals (--rate per s for --duration s), 50/30/20 quality /
    10-sweep smoothing / CG requests on meshes of 1e4..1e7 tets (log-uniform)
    and on the SPD systems of their vertex graphs; a request targets a mesh
    seen before with probability 0.5, else a new one.  Distinct sizes come
    from a pool of size buckets (each new target is a separate resident
    copy).  Continuous batching with a 150 GB budget, then the serial plain
    path on the first --serial-requests requests of the same trace, the
    saturated capacity of both paths, and the highest rate each path
    sustains at the stated p99 (--sweep-seconds of arrivals per rate)."""
    import gmlib_gb300 as G
    m = serve_measure(G, dist.local, args.rate, args.duration, args.serial_requests,
                      args.saturate, args.sweep_seconds)
    pool = m["pool"]
    if dist.rank == 0:
        line = {"metric": "served requests/s at p99 (continuous batching)",
                "value": m["batching"]["throughput_rps"], "unit": "req/s", "n_gpus": dist.world,
                "higher_is_better": True, "dtype": "f32 / f64", "data": "synthetic",
                "config": {"workload": "Poisson %.0f req/s for %.0f s, 50/30/20 quality / "
                                       "10-sweep smoothing / CG (1e-10)" % (args.rate, args.duration),
                           "sizes_tets": [int(6 * n ** 3) for n in pool.ns], "reuse": 0.5,
                           "budget_gb": 150, "slots": 8, "pool_generation_s": round(pool.tgen, 1),
                           "vertex_tet_degrees": degree_summary([x[1] for x in pool.meshes])},
                "batching": m["batching"], "batching_by_kind": m["batching_by_kind"],
                "serial_prefix": m["serial_prefix"], "capacity_saturated": m["capacity_saturated"],
                "capacity_at_p99": m["capacity_at_p99"],
                "same_result_alone_and_in_mix": "%d of %d" % (m["same"], m["nser"]),
                "clocks": m["clocks"]}
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        elif args.workload == "solve":
            run_solve(args, dist)
        elif args.workload == "batch":
            run_batch(args, dist)
        elif args.workload == "serve":
            run_serve(args, dist)
        elif args.workload == "p2":
            run_p2(args, dist)
        elif args.workload == "quality":
            run_quality(args, dist)
        elif args.workload == "nodesmooth":
            run_nodesmooth(args, dist)
        else:
            run_gpu(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
