"""Benchmark of the neighbour-query -> pair-reduction path on one GB300.

Headline workload (pair evaluations per second): 102^3 = 1,061,208 points on a
simple-cubic lattice of spacing 1 with seeded Gaussian jitter sigma = 0.1, periodic
cubic box L = 102, float32; LinkCell(box, points, 3.0).query(points,
{r_max: 3.0, exclude_ii: True}).toNeighborList() in the reference's sorted order,
then RDF(300 bins, r_max 3.0) on that NeighborList. One step = both calls.
A pair evaluation is one accepted ordered bond.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

value      device-resident points, C-ABI calls, CUDA events around each step
e2e        the public Python API with host (pinned) points: H2D, build, query,
           RDF, D2H of the RDF; host wall clock around each synchronous step
roofline   the dominant kernel's algorithmic bytes / its event-timed duration
cpu_baseline  the CPU oracle (restatement of the reference, all host threads)
              on a bounded sample of the same workload (a prefix of the query points)
--impl reference  times that CPU path alone with the same metric.
Multi-GPU: independent replicas (the path has no exchange step); value sums ranks.
"""

import argparse
import ctypes
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

METRIC = "pair evals/s (RDF) & particles/s (Steinhardt l=6), batched vs plain, 1 GB300"
WORKLOAD = "large_n_nlist_rdf"
L2_BYTES = 129 * 1024 * 1024


def c2_system(seed=2024, n1=102):
    """n1^3 simple-cubic lattice (102^3 by default), spacing 1, N(0, 0.1) jitter,
    wrapped into the periodic cube of side L = n1."""
    L = float(n1)
    g = np.arange(n1, dtype=np.float64) - n1 / 2.0
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], 1)
    rng = np.random.default_rng(seed)
    pts = pts + rng.normal(0.0, 0.1, pts.shape)
    pts = (pts + L / 2) % L - L / 2
    return L, pts.astype(np.float32)


def read_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self._t is not None:
            self._t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(L, pts, r_max=3.0, bins=300, target_s=12.0, threads=None):
    """CPU oracle (restatement of the reference path, all host threads) on a bounded
    sample: the first M query points against all points, M scaled so the measured
    run takes about target_s seconds. Returns (bonds/s, sample description, cores)."""
    from oracle import oracle as O

    threads = threads or (os.cpu_count() or 1)
    box = (L, L, L, 0.0, 0.0, 0.0, 0.0)
    m = 20000
    t0 = time.perf_counter()
    ij, d, v = O.query(box, pts, query_points=pts[:m], r_max=r_max, exclude_ii=True, arith=O.ARITH_WRAP,
                       threads=threads)
    O.hist(d, bins, r_max)
    dt = time.perf_counter() - t0
    m2 = int(min(len(pts), max(m, m * target_s / max(dt, 1e-3))))
    t0 = time.perf_counter()
    ij, d, v = O.query(box, pts, query_points=pts[:m2], r_max=r_max, exclude_ii=True, arith=O.ARITH_WRAP,
                       threads=threads)
    O.hist(d, bins, r_max)
    dt = time.perf_counter() - t0
    return len(ij) / dt, ("LinkCell-arithmetic ball query r_max=3 + NeighborList sort + RDF histogram for the "
                          "first %d of %d query points against all points" % (m2, len(pts))), threads, dt


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    L, pts = c2_system(n1=args.n_side)
    vals = []
    desc = cores = None
    for _ in range(args.warmup):
        cpu_baseline(L, pts, target_s=2.0)
    for _ in range(args.steps):
        v, desc, cores, _dt = cpu_baseline(L, pts, target_s=8.0)
        vals.append(v)
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "pair evals/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "n_points": len(pts), "box_L": L, "cell_width": 3.0, "r_max": 3.0,
                   "bins": 300},
        "cpu_baseline": {"value": value, "unit": "pair evals/s", "cores": cores, "kind": "port", "sample": desc},
        "e2e": {"value": value, "unit": "pair evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--n-side", type=int, default=102,
                    help="lattice points per side; 102 is the benchmark workload, smaller sizes are for profiling")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from freud_gb300 import _lib

    import freud_gb300 as freud

    lib = _lib.lib
    # one dedicated stream for the library, the L2 flush and the timing events
    stream = torch.cuda.Stream()
    _lib.set_stream(stream.cuda_stream)
    torch.cuda.set_stream(stream)

    L, pts_host = c2_system(seed=2024 + rank, n1=args.n_side)
    n = len(pts_host)
    d_pts = torch.from_numpy(pts_host).cuda()
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    box = freud.box.Box.cube(L)
    cbox = box._c_box()
    qargs = _lib.make_args(_lib.MODE_BALL, r_max=3.0, exclude_ii=True)
    rdf = ctypes.c_void_p()
    _lib.check(lib.fg_rdf_create(300, 3.0, 0.0, ctypes.byref(rdf)))

    def step():
        nq = ctypes.c_void_p()
        _lib.check(lib.fg_nq_create_device(ctypes.byref(cbox), ctypes.c_void_p(d_pts.data_ptr()), n,
                                           _lib.NQ_LINKCELL, 3.0, ctypes.byref(nq)))
        nl = ctypes.c_void_p()
        _lib.check(lib.fg_nq_query_device(nq, None, n, ctypes.byref(qargs), 0, ctypes.byref(nl)))
        _lib.check(lib.fg_rdf_reset(rdf))
        _lib.check(lib.fg_rdf_accumulate_device(rdf, nq, None, n, nl, None))
        nb = ctypes.c_uint64()
        _lib.check(lib.fg_nlist_num_bonds(nl, ctypes.byref(nb)))
        lib.fg_nlist_destroy(nl)
        lib.fg_nq_destroy(nq)
        return nb.value

    for _ in range(max(args.warmup, 3)):
        bonds = step()
    torch.cuda.synchronize()

    # ---- timed region: device-resident inputs -------------------------------------
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = _lib.launch_count()
    _lib.profile_enable(True)
    times = []
    for _ in range(args.steps):
        flush.fill_(1.0)  # evict L2 between steps (outside the timed interval)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        bonds = step()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    prof = _lib.profile_report()
    _lib.profile_enable(False)
    launches = _lib.launch_count() - launches0 - 0
    clk = clocks.stop()
    total_ms = sum(times)
    if world > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = bonds * world * args.steps / (total_ms / 1e3)

    # roofline of the dominant kernel
    peak, peak_kind = read_peaks()
    dom = max(prof.items(), key=lambda kv: kv[1][1]) if prof else (None, (0, 0.0))
    dom_name, (dom_n, dom_ms) = dom
    per_launch_ms = dom_ms / max(dom_n, 1)
    if dom_name is not None and "EMIT" in dom_name:
        alg_bytes = 12.0 * n + 24.0 * bonds  # positions read + (i,j) 8 B + distance 4 B + vector 12 B per bond
        alg_desc = "12*N + 24*B (positions read; (i,j), distance, vector written; weights are lazy)"
    elif dom_name is not None and "COUNT" in dom_name:
        alg_bytes = 12.0 * n + 4.0 * n
        alg_desc = "12*N + 4*N (positions read, counts written)"
    elif dom_name is not None and "hist" in dom_name:
        alg_bytes = 4.0 * bonds
        alg_desc = "4*B (distances read)"
    else:
        alg_bytes = 12.0 * n
        alg_desc = "12*N"
    achieved = alg_bytes / (per_launch_ms / 1e3) / 1e9 if per_launch_ms > 0 else 0.0
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            traffic = json.load(f).get(dom_name)
    except (OSError, ValueError):
        pass

    # ---- e2e: public Python API with host (pinned) buffers --------------------------
    pinned = torch.from_numpy(pts_host).pin_memory().numpy()
    e2e_times = []
    for it in range(args.warmup + args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lc = freud.locality.LinkCell(box, pinned, 3.0)
        nlist = lc.query(pinned, {"r_max": 3.0, "exclude_ii": True}).toNeighborList()
        r = freud.density.RDF(300, 3.0).compute(lc, neighbors=nlist)
        g = r.rdf
        t1 = time.perf_counter()
        if it >= args.warmup:
            e2e_times.append(t1 - t0)
        del lc, nlist, r, g
    e2e_value = bonds * world / statistics.median(e2e_times)

    # ---- CPU baseline (rank 0, N=1 only) ---------------------------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, desc, cores, dt = cpu_baseline(L, pts_host)
        cpu = {"value": v, "unit": "pair evals/s", "cores": cores, "kind": "port", "sample": desc,
               "seconds": round(dt, 2)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "pair evals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered 102^3 lattice)",
            "config": {"workload": WORKLOAD if args.n_side == 102 else "%s_n%d" % (WORKLOAD, args.n_side), "n_points": n, "box_L": L, "cell_width": 3.0, "r_max": 3.0,
                       "bins": 300, "bonds_per_step": bonds, "l2": "flushed between steps (258 MB write)",
                       "parallelism": "replicas" if world > 1 else "single"},
            "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak,
                         "peak_source": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "algorithmic_bytes_per_launch": alg_bytes,
                         "algorithmic_bytes": alg_desc, "launch_ms": per_launch_ms},
            "kernels": {k: {"launches": v[0], "total_ms": round(v[1], 4)} for k, v in sorted(prof.items())},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "pair evals/s", "h2d_bytes_per_step": int(12 * n),
                    "d2h_bytes_per_step": int(300 * 4)},
            "gpu_launches": int(launches),
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    lib.fg_rdf_destroy(rdf)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
