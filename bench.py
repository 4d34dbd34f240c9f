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
e2e_nlist_readback  the same plus nlist[:], distances and vectors read to host
roofline   the NeighborList build (every kernel of the step except the RDF over
           the finished list): 12 N + 24 B bytes over the kernels' event time
cpu_baseline  the CPU oracle (restatement of the reference, all host threads)
              over the whole workload; its list is also the parity reference
parity     per workload: the GPU results against the oracle (bit-exact lists and
           counts; Steinhardt within the stated FP64 tolerances); a mismatch
           makes the run exit with status 1 after printing the line
--impl reference  times the CPU path alone with the same metric (a bounded sample).
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
PARITY_OK = ("bit-exact", "within tolerance")
WL_FLOOR = 1e-7  # absolute floor of the Wl tolerance (normalised Wl is O(0.01-0.1))


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


def c1_system(seed=1):
    """10,000 points uniform in a periodic cube of side 21.544 (number density 1)."""
    L = 21.544
    rng = np.random.default_rng(seed)
    pts = rng.uniform(-L / 2, L / 2, (10000, 3)).astype(np.float32)
    return L, pts


def c3_system(seed=3):
    """FCC crystal 4 * 40^3 = 256,000 points, lattice constant 1.5874 (density 1),
    seeded N(0, 0.05) displacements, periodic cube of side 63.496."""
    a, nc = 1.5874, 40
    L = a * nc
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]], np.float64)
    g = np.arange(nc, dtype=np.float64)
    cells = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 1, 3)
    pts = ((cells + basis[None]) * a).reshape(-1, 3) - L / 2
    rng = np.random.default_rng(seed)
    pts = pts + rng.normal(0.0, 0.05, pts.shape)
    pts = (pts + L / 2) % L - L / 2
    return np.float32(L), pts.astype(np.float32)


def c4_frames(freud, seed=4, nframes=64, density=0.85):
    """64 frames, N uniform-integer in [5,000, 500,000], points uniform in
    fractional coordinates at number density 0.85; 90% cubic boxes, 10%
    triclinic (xy = 0.2, xz = 0.1, yz = 0)."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(5000, 500001, nframes)
    tric = np.zeros(nframes, bool)
    tric[rng.permutation(nframes)[:int(round(0.1 * nframes))]] = True
    frames = []
    for n, t in zip(ns, tric):
        L = float((n / density) ** (1.0 / 3.0))
        box = freud.box.Box(L, L, L, 0.2 if t else 0.0, 0.1 if t else 0.0, 0.0)
        frac = rng.random((int(n), 3))
        frames.append((box, box.make_absolute(frac).astype(np.float32)))
    return frames


def c5_system(seed=5, blobs=4096, L=256.0):
    """4,096 isotropic Gaussian blobs (sigma 2.0, 1,024 points each) with centres
    uniform in a periodic cube of side 256: 4,194,304 points (a smaller profiling
    case keeps the blob density: 512 blobs in L = 128)."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.0, L, (blobs, 3))
    pts = (centres[:, None, :] + rng.normal(0.0, 2.0, (blobs, 1024, 3))).reshape(-1, 3)
    pts = (pts % L) - L / 2
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


def cpu_baseline(L, pts, r_max=3.0, bins=300, target_s=12.0, threads=None, sample=None):
    """CPU oracle (restatement of the reference path, all host threads): LinkCell
    arithmetic ball query + NeighborList in reference order + RDF histogram.
    sample=None runs the whole workload once (every query point) and also returns
    the oracle's list and counts for the parity check; sample=M times the first M
    query points against all points (a bounded sample; M = 0 scales M from a short
    probe so the run takes about target_s seconds).
    Returns (bonds/s, sample description, threads, seconds, (ij, d, v, counts) or None)."""
    from oracle import oracle as O

    threads = threads or (os.cpu_count() or 1)
    box = (L, L, L, 0.0, 0.0, 0.0, 0.0)
    if sample is None:
        t0 = time.perf_counter()
        ij, d, v = O.query(box, pts, r_max=r_max, exclude_ii=True, arith=O.ARITH_WRAP, threads=threads)
        counts = O.hist(d, bins, r_max)
        dt = time.perf_counter() - t0
        return (len(ij) / dt, "whole workload: LinkCell-arithmetic ball query r_max=%g over all %d query points + "
                "NeighborList sort + RDF histogram, one run" % (r_max, len(pts)), threads, dt, (ij, d, v, counts))
    m = sample if sample > 0 else 20000
    if sample == 0:
        t0 = time.perf_counter()
        O.query(box, pts, query_points=pts[:m], r_max=r_max, exclude_ii=True, arith=O.ARITH_WRAP, threads=threads)
        dt = time.perf_counter() - t0
        m = int(min(len(pts), max(m, m * target_s / max(dt, 1e-3))))
    t0 = time.perf_counter()
    ij, d, v = O.query(box, pts, query_points=pts[:m], r_max=r_max, exclude_ii=True, arith=O.ARITH_WRAP,
                       threads=threads)
    O.hist(d, bins, r_max)
    dt = time.perf_counter() - t0
    return len(ij) / dt, ("LinkCell-arithmetic ball query r_max=%g + NeighborList sort + RDF histogram for the "
                          "first %d of %d query points against all points" % (r_max, m, len(pts))), threads, dt, None


def _median_wall(fn, steps, warmup):
    for _ in range(warmup):
        fn()
    ts = []
    for _ in range(steps):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts)


def _device_ms(_lib, fn, steps):
    """Median device time of fn's kernels per call (CUDA events the library records
    on its stream around each launch) and the launches per call."""
    _lib.profile_enable(True)
    l0 = _lib.launch_count()
    for _ in range(steps):
        fn()
    prof = _lib.profile_report()
    launches = (_lib.launch_count() - l0) / steps
    _lib.profile_enable(False)
    ms = sum(v[1] for v in prof.values()) / steps
    per = {k: round(v[1] / steps, 4) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])}
    return ms, launches, per


def measure_c1(freud, _lib, steps, warmup, cpu=True):
    """Plain RDF: RDF(200, 4.0).compute((box, points)), 10,000 uniform points."""
    L, pts = c1_system()
    box = freud.box.Box.cube(L)
    rdf = freud.density.RDF(200, 4.0)

    def step():
        rdf.compute((box, pts))
        return rdf.bin_counts_u64

    pairs = int(step().sum())
    t = _median_wall(step, steps, warmup)
    dev_ms, launches, top = _device_ms(_lib, step, steps)
    out = {"workload": "plain_rdf_n10000_L21.544_rmax4_bins200", "pairs": pairs, "e2e_ms": t * 1e3,
           "e2e": pairs / t, "device_ms": dev_ms, "device": pairs / (dev_ms / 1e3), "unit": "pair evals/s",
           "launches_per_step": launches, "kernels_ms_per_step": top}
    if cpu:
        from oracle import oracle as O

        bx = (L, L, L, 0.0, 0.0, 0.0, 0.0)
        threads = os.cpu_count() or 1
        ts = []
        for _ in range(5):
            t0 = time.perf_counter()
            O.rdf_counts_query(bx, pts, 200, 4.0, arith=O.ARITH_AABB, threads=threads)
            ts.append(time.perf_counter() - t0)
        out["cpu_baseline"] = {"value": pairs / statistics.median(ts), "unit": "pair evals/s", "cores": threads,
                               "kind": "port", "sample": "whole workload, median of 5"}
    return out


def measure_cf(freud, _lib, steps, warmup, cpu=True):
    """CorrelationFunction(200, 4.0).compute((box, points), values) on the plain RDF
    system (10,000 uniform points) with complex values e^{i theta}: bonds found on
    the GPU, conj(values[j]) * values[i] summed per bin in FP64."""
    L, pts = c1_system()
    box = freud.box.Box.cube(L)
    rs = np.random.RandomState(5)
    vals = np.exp(1j * rs.random_sample(len(pts)) * 2.0 * np.pi)
    cf = freud.density.CorrelationFunction(200, 4.0)

    def step():
        cf.compute((box, pts), vals)
        return cf.bin_counts

    pairs = int(step().astype(np.int64).sum())
    t = _median_wall(step, steps, warmup)
    dev_ms, launches, top = _device_ms(_lib, step, steps)
    out = {"workload": "correlation_function_n10000_L21.544_rmax4_bins200_complex", "pairs": pairs,
           "e2e_ms": t * 1e3, "e2e": pairs / t, "device_ms": dev_ms, "device": pairs / (dev_ms / 1e3),
           "unit": "pair evals/s", "launches_per_step": launches, "kernels_ms_per_step": top}
    if cpu:
        from oracle import oracle as O

        bx = (L, L, L, 0.0, 0.0, 0.0, 0.0)
        threads = os.cpu_count() or 1
        ts = []
        for _ in range(5):
            t0 = time.perf_counter()
            ij, d, _ = O.query(bx, pts, r_max=4.0, exclude_ii=True, threads=threads)
            O.correlation(ij, d, vals, vals, 200, 4.0)
            ts.append(time.perf_counter() - t0)
        out["cpu_baseline"] = {"value": pairs / statistics.median(ts), "unit": "pair evals/s", "cores": threads,
                               "kind": "port", "sample": "whole workload (oracle query on all threads, numpy "
                                                         "FP64 sums), median of 5"}
    return out


def measure_pmft(freud, _lib, steps, warmup, cpu=True):
    """PMFTXYZ(1.5, 1.5, 1.5, 40) on the 256,000-particle FCC system with random
    unit-quaternion orientations (ball neighbours within sqrt(3) * 1.5)."""
    L, pts = c3_system()
    box = freud.box.Box.cube(float(L))
    rs = np.random.RandomState(6)
    q = rs.standard_normal((len(pts), 4))
    q = (q / np.linalg.norm(q, axis=1, keepdims=True)).astype(np.float32)
    pm = freud.pmft.PMFTXYZ(1.5, 1.5, 1.5, 40)

    def step():
        pm.compute((box, pts), q)
        return pm.bin_counts

    bonds = int(step().astype(np.int64).sum())
    t = _median_wall(step, steps, warmup)
    dev_ms, launches, top = _device_ms(_lib, step, steps)
    out = {"workload": "pmftxyz_fcc_256000_xyz1.5_bins40", "binned_bonds": bonds, "e2e_ms": t * 1e3,
           "e2e": bonds / t, "device_ms": dev_ms, "device": bonds / (dev_ms / 1e3), "unit": "pair evals/s",
           "launches_per_step": launches, "kernels_ms_per_step": top}
    if cpu:
        from oracle import oracle as O

        bx = (float(L),) * 3 + (0.0, 0.0, 0.0, 0.0)
        rm = float(np.float32(np.sqrt(3 * 1.5 ** 2)))
        t0 = time.perf_counter()
        ij, d, v = O.query(bx, pts, r_max=rm, exclude_ii=True)
        tq = time.perf_counter() - t0
        t0 = time.perf_counter()
        O.pmft_counts(3, [1.5, 1.5, 1.5], [40, 40, 40], ij, d, v, q_quat=q,
                      equiv=np.array([[1, 0, 0, 0]], np.float32))
        tb = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": bonds / (tq + tb), "unit": "pair evals/s", "cores": os.cpu_count() or 1,
                               "kind": "port", "sample": "whole workload: oracle ball query (all threads) + PMFT "
                                                         "binning (1 thread)"}
    return out


def measure_c3(freud, _lib, steps, warmup, cpu=True):
    """Steinhardt([4, 6, 8, 10, 12], average, wl, wl_normalize) with 12 nearest
    neighbours on a 256,000-point noisy FCC crystal. Parity: every particle's
    averaged Ql and normalised Wl and the system order against the FP64 oracle
    (whose run over the whole workload is also the CPU baseline)."""
    L, pts = c3_system()
    box = freud.box.Box.cube(float(L))
    ls = [4, 6, 8, 10, 12]
    st = freud.order.Steinhardt(ls, average=True, wl=True, wl_normalize=True)

    def step():
        st.compute((box, pts), neighbors={"num_neighbors": 12})
        return st.particle_order

    step()
    t = _median_wall(step, steps, warmup)
    dev_ms, launches, top = _device_ms(_lib, step, steps)
    n = len(pts)
    out = {"workload": "steinhardt_fcc_256000_k12_l4-12_ave_wl", "particles": n, "e2e_ms": t * 1e3, "e2e": n / t,
           "device_ms": dev_ms, "device": n / (dev_ms / 1e3), "unit": "particles/s", "launches_per_step": launches,
           "kernels_ms_per_step": top}
    # roofline of the step: 12 N + 8 B + 8 N sum(2l+1) (1 + average) + 4 N n_l (1 + average + wl)
    peak, peak_kind = read_peaks()
    stride = sum(2 * l + 1 for l in ls)
    alg = 12.0 * n + 8.0 * 12 * n + 8.0 * n * stride * 2 + 4.0 * n * len(ls) * 3
    out["roofline"] = {"bound": "hbm", "algorithmic_bytes": alg, "achieved": alg / (dev_ms / 1e3) / 1e9,
                       "peak": peak, "peak_source": peak_kind, "unit": "GB/s",
                       "frac": alg / (dev_ms / 1e3) / 1e9 / peak,
                       "formula": "12 N + 8 B + 8 N sum(2l+1) (1 + average) + 4 N n_l (1 + average + wl), B = 12 N"}
    if cpu:
        from oracle import oracle as O

        bx = (float(L),) * 3 + (0.0, 0.0, 0.0, 0.0)
        threads = os.cpu_count() or 1
        t0 = time.perf_counter()
        ij, d, _v = O.query(bx, pts, num_neighbors=12, exclude_ii=True, threads=threads)
        o = O.steinhardt(ls, bx, pts, ij, d, average=True, wl=True, wl_normalize=True, threads=threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": n / dt, "unit": "particles/s", "cores": threads, "kind": "port",
                               "sample": "whole workload: kNN query (k = 12) + FP64 Steinhardt l = 4..12, "
                                         "average, wl, wl_normalize, one run", "seconds": round(dt, 2)}
        out["parity"] = steinhardt_parity(st, o, ls)
    return out


def steinhardt_parity(st, o, ls, wl=True):
    """Errors of a computed Steinhardt against the FP64 oracle: Ql (averaged) 1e-5
    relative; Wl |dw| <= 1e-5 |w| + WL_FLOOR (normalised Wl, absolute floor for
    values near zero); system order 1e-5 relative (Wl order: + WL_FLOOR)."""
    ql = np.asarray(st.ql, np.float64).reshape(o["ql_ave"].shape)
    ref_ql = o["ql_ave"]
    ok = np.isfinite(ref_ql)
    ql_rel = float(np.max(np.abs(ql[ok] - ref_ql[ok]) / np.abs(ref_ql[ok])))
    res = {"particles": int(ql.shape[0]), "ql_max_rel": ql_rel, "ql_tol_rel": 1e-5}
    good = ql_rel <= 1e-5
    if wl:
        w = np.asarray(st.particle_order, np.float64).reshape(o["wl"].shape)
        ref_w = o["wl"]
        okw = np.isfinite(ref_w)
        err = np.abs(w[okw] - ref_w[okw])
        bound = 1e-5 * np.abs(ref_w[okw]) + WL_FLOOR
        res.update(wl_max_rel=float(np.max(err / np.abs(ref_w[okw]))),
                   wl_max_abs=float(np.max(err)), wl_tol="1e-5 |w| + %g" % WL_FLOOR,
                   wl_within=bool(np.all(err <= bound)),
                   wl_max_over_bound=float(np.max(err / bound)))
        per_l = np.max(np.abs(w - ref_w) / (1e-5 * np.abs(ref_w) + WL_FLOOR), axis=0)
        res["wl_max_over_bound_per_l"] = {str(l): float(x) for l, x in zip(ls, np.atleast_1d(per_l))}
        good = good and res["wl_within"]
    order = np.atleast_1d(np.asarray(st.order, np.float64))
    ref_o = np.atleast_1d(o["order"])
    oerr = np.abs(order - ref_o)
    res["order_max_rel"] = float(np.max(oerr / np.abs(ref_o)))
    good = good and bool(np.all(oerr <= 1e-5 * np.abs(ref_o) + (WL_FLOOR if wl else 0.0)))
    res["status"] = "within tolerance" if good else "MISMATCH"
    return res


def measure_c4(freud, _lib, steps, warmup, nframes=64):
    """64 uneven frames: RDF(200, 4.0) accumulated over the frames (reset=False)
    plus Steinhardt(6, average=True) on r_max = 1.5 ball neighbours, per frame
    (plain) and as one FrameBatch (batched), both through the public API with
    host points, results read back every step."""
    frames = c4_frames(freud, nframes=nframes)
    n_total = sum(len(p) for _, p in frames)
    rdf = freud.density.RDF(200, 4.0)
    st = freud.order.Steinhardt(6, average=True)

    def plain():
        for f, (box, p) in enumerate(frames):
            rdf.compute((box, p), reset=(f == 0))
            st.compute((box, p), neighbors={"r_max": 1.5})
            st.ql
        return rdf.bin_counts_u64

    def batched():
        batch = freud.locality.FrameBatch(frames)
        rdf.compute(batch)
        st.compute(batch, neighbors={"r_max": 1.5})
        st.ql
        return rdf.bin_counts_u64

    ref = plain()
    got = batched()
    assert np.array_equal(ref, got), "batched RDF counts differ from the per-frame path"
    parity, cpu = c4_oracle_check(freud, frames)
    small = measure_small_frames(freud, _lib, max(1, min(steps, 5)), max(1, warmup))
    pairs = int(got.sum())
    k = max(1, min(steps, 5))
    t_plain = _median_wall(plain, k, 1)
    t_batch = _median_wall(batched, k, max(1, warmup))
    dev_plain, l_plain, top_plain = _device_ms(_lib, plain, 2)
    dev_batch, l_batch, top_batch = _device_ms(_lib, batched, 2)
    return {"workload": "batched_uneven_%d_frames_rdf_rmax4_bins200_steinhardt6_rmax1.5" % len(frames),
            "frames": len(frames),
            "particles": n_total, "pairs": pairs,
            "plain": {"e2e_ms": t_plain * 1e3, "pair_evals_per_s": pairs / t_plain, "particles_per_s": n_total / t_plain,
                      "device_ms": dev_plain, "launches_per_step": l_plain, "kernels_ms_per_step": top_plain},
            "batched": {"e2e_ms": t_batch * 1e3, "pair_evals_per_s": pairs / t_batch,
                        "particles_per_s": n_total / t_batch, "device_ms": dev_batch, "launches_per_step": l_batch,
                        "kernels_ms_per_step": top_batch},
            "speedup_e2e": t_plain / t_batch, "speedup_device": dev_plain / dev_batch if dev_batch else None,
            "small_frames": small,
            "autotune": _lib.autotune_report().strip().splitlines(),
            "parity": parity, "cpu_baseline": cpu}


def c4_oracle_check(freud, frames, max_frames=8):
    """Oracle parity on a sample of the trajectory's frames (every triclinic frame,
    then the smallest and largest cubic ones, up to max_frames): per frame the RDF
    counts (RDF(200, 4.0) on (box, points), bit-exact) and Steinhardt(6, average)
    on r_max = 1.5 ball neighbours (1e-5 relative to the FP64 oracle), through the
    public API on the GPU. The same oracle runs, timed, are the CPU baseline."""
    from oracle import oracle as O

    tric = [f for f, (b, _) in enumerate(frames) if b.xy != 0.0 or b.xz != 0.0]
    cubic = sorted((f for f in range(len(frames)) if f not in tric), key=lambda f: len(frames[f][1]))
    pick = (tric + cubic[:1] + cubic[-1:] + cubic[1:])[:max_frames]
    threads = os.cpu_count() or 1
    rdf = freud.density.RDF(200, 4.0)
    st = freud.order.Steinhardt(6, average=True)
    rows, cpu_s, pairs, parts = [], 0.0, 0, 0
    ok = True
    for f in pick:
        box, p = frames[f]
        c_gpu = np.asarray(rdf.compute((box, p)).bin_counts_u64)
        q_gpu = np.asarray(st.compute((box, p), neighbors={"r_max": 1.5}).ql, np.float64)
        bx = O.box7(box)
        t0 = time.perf_counter()
        c_ref = O.rdf_counts_query(bx, p, 200, 4.0, threads=threads)
        ij, d, _ = O.query(bx, p, r_max=1.5, exclude_ii=True, threads=threads)
        o = O.steinhardt([6], bx, p, ij, d, average=True, threads=threads)
        cpu_s += time.perf_counter() - t0
        q_ref = o["ql_ave"][:, 0]
        fin = np.isfinite(q_ref)
        same_nan = bool(np.array_equal(np.isfinite(q_gpu), fin))
        q_rel = float(np.max(np.abs(q_gpu[fin] - q_ref[fin]) / np.abs(q_ref[fin]))) if fin.any() else 0.0
        counts_ok = bool(np.array_equal(c_gpu, c_ref))
        ok = ok and counts_ok and same_nan and q_rel <= 1e-5
        pairs += int(c_ref.sum())
        parts += len(p)
        rows.append({"frame": int(f), "n": int(len(p)), "triclinic": f in tric, "rdf_counts_equal": counts_ok,
                     "q6_max_rel": q_rel})
    parity = {"frames": rows, "status": "within tolerance" if ok else "MISMATCH",
              "what": "RDF counts bit-exact, averaged q6 within 1e-5 relative of the FP64 oracle, per frame"}
    cpu = {"value": pairs / cpu_s, "unit": "pair evals/s", "particles_per_s": parts / cpu_s, "cores": threads,
           "kind": "port", "seconds": round(cpu_s, 2),
           "sample": "%d of the %d frames (%d points): RDF counts + ball query r_max 1.5 + FP64 Steinhardt "
                     "l = 6 average" % (len(pick), len(frames), parts)}
    return parity, cpu


def measure_small_frames(freud, _lib, steps, warmup, nframes=1024, seed=44):
    """Where batching pays most: 1,024 frames of 1,000-4,000 points (same density
    and computes as the uneven trajectory), per frame vs one FrameBatch."""
    rng = np.random.default_rng(seed)
    frames = []
    for n in rng.integers(1000, 4001, nframes):
        L = float((n / 0.85) ** (1.0 / 3.0))
        box = freud.box.Box.cube(L)
        frames.append((box, box.make_absolute(rng.random((int(n), 3))).astype(np.float32)))
    rdf = freud.density.RDF(200, 4.0)
    st = freud.order.Steinhardt(6, average=True)

    def plain():
        for f, (box, p) in enumerate(frames):
            rdf.compute((box, p), reset=(f == 0))
            st.compute((box, p), neighbors={"r_max": 1.5})
            st.ql
        return rdf.bin_counts_u64

    def batched():
        batch = freud.locality.FrameBatch(frames)
        rdf.compute(batch)
        st.compute(batch, neighbors={"r_max": 1.5})
        st.ql
        return rdf.bin_counts_u64

    assert np.array_equal(plain(), batched()), "batched RDF counts differ from the per-frame path"
    t_plain = _median_wall(plain, steps, 1)
    t_batch = _median_wall(batched, steps, warmup)
    return {"workload": "1024_frames_1000-4000_points", "particles": int(sum(len(p) for _, p in frames)),
            "plain_e2e_ms": t_plain * 1e3, "batched_e2e_ms": t_batch * 1e3, "speedup_e2e": t_plain / t_batch}


def measure_c5(freud, _lib, steps, warmup, small=False):
    """4,194,304 points in 4,096 Gaussian blobs: RDF(500, 5.0) with uint64 counts
    and FP64 normalisation, Steinhardt(6) on r_max = 1.2 ball neighbours."""
    L, pts = c5_system(blobs=512, L=128.0) if small else c5_system()
    box = freud.box.Box.cube(L)
    rdf = freud.density.RDF(500, 5.0)
    st = freud.order.Steinhardt(6)

    def step():
        rdf.compute((box, pts))
        c = rdf.bin_counts_u64
        st.compute((box, pts), neighbors={"r_max": 1.2})
        st.ql
        return c

    c = step()
    pairs = int(c.sum())
    k = max(1, min(steps, 3))
    t = _median_wall(step, k, 1)
    dev_ms, launches, top = _device_ms(_lib, step, 1)
    g32, g64 = rdf.rdf.astype(np.float64), rdf.rdf_fp64
    nz = g64 > 0
    # Steinhardt error against the FP64 oracle on the first 16,384 particles (their
    # q6 needs only their own bonds: no averaging)
    from oracle import oracle as O

    m = min(16384, len(pts))
    bx = (L, L, L, 0.0, 0.0, 0.0, 0.0)
    ij, d, _ = O.query(bx, pts, query_points=pts[:m], r_max=1.2, exclude_ii=True, arith=O.ARITH_AABB)
    ref = O.steinhardt([6], bx, pts, ij, d)["ql"][:m, 0]
    got = np.asarray(st.ql, np.float64)[:m]
    ok = np.isfinite(ref)
    ql_err = float(np.max(np.abs(got[ok] - ref[ok]) / np.abs(ref[ok])))
    # RDF counts of a spread sample of query points (every 64th point, exclude_ii off
    # so query i need not be point i) against the oracle; its timed run is the CPU baseline
    qs = np.ascontiguousarray(pts[::64])
    r2 = freud.density.RDF(500, 5.0).compute((box, pts), query_points=qs,
                                               neighbors={"r_max": 5.0, "exclude_ii": False})
    c_gpu = np.asarray(r2.bin_counts_u64)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    c_ref = O.rdf_counts_query(bx, pts, 500, 5.0, query_points=qs, exclude_ii=False, threads=threads)
    cpu_s = time.perf_counter() - t0
    counts_ok = bool(np.array_equal(c_gpu, c_ref))
    parity = {"rdf_counts_equal": counts_ok, "query_points": int(len(qs)), "pairs": int(c_ref.sum()),
              "q6_max_rel": ql_err, "q6_particles": int(m),
              "status": "within tolerance" if counts_ok and ql_err <= 1e-5 else "MISMATCH",
              "what": "RDF counts of every 64th point as a query point, bit-exact; q6 of the first 16,384 "
                      "particles within 1e-5 relative of the FP64 oracle"}
    cpu = {"value": float(c_ref.sum()) / cpu_s, "unit": "pair evals/s", "cores": threads, "kind": "port",
           "seconds": round(cpu_s, 2),
           "sample": "RDF(500, 5.0) counts of %d query points (every 64th) against all %d points"
                     % (len(qs), len(pts))}
    # occupancy skew of the r_max = 5 cell grid (51^3 cells)
    nc = int(L // 5.0)
    idx = np.floor((pts.astype(np.float64) + L / 2) / L * nc).astype(np.int64) % nc
    occ = np.bincount((idx[:, 0] * nc + idx[:, 1]) * nc + idx[:, 2], minlength=nc ** 3)
    return {"workload": "blobs_%dx1024_L%d_rdf_rmax5_bins500_steinhardt6_rmax1.2" % (len(pts) // 1024, int(L)),
            "particles": len(pts),
            "pairs": pairs, "pairs_above_2^32": pairs >= 2 ** 32, "e2e_ms": t * 1e3, "e2e": pairs / t,
            "device_ms": dev_ms, "device": pairs / (dev_ms / 1e3), "unit": "pair evals/s (RDF + Steinhardt step)",
            "launches_per_step": launches, "kernels_ms_per_step": top,
            "rdf_f32_vs_fp64_max_rel": float(np.max(np.abs(g32[nz] - g64[nz]) / g64[nz])),
            "q6_vs_fp64_oracle_max_rel": ql_err, "q6_checked_particles": int(m),
            "cell_occupancy": {"mean": float(occ.mean()), "max": int(occ.max()),
                               "skew_max_over_mean": float(occ.max() / occ.mean())},
            "parity": parity, "cpu_baseline": cpu}


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
        cpu_baseline(L, pts, target_s=2.0, sample=0)
    for _ in range(args.steps):
        v, desc, cores, _dt, _ = cpu_baseline(L, pts, target_s=8.0, sample=0)
        vals.append(v)
    value = statistics.median(vals)
    # the whole step (every query point) at the sampled rate: 108 bonds per point on
    # the jittered lattice at r_max 3 (114,643,150 bonds for 102^3 points)
    bonds_full = 114643150 * len(pts) / 1061208.0
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "pair evals/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * bonds_full / value,
        "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "n_points": len(pts), "box_L": L, "cell_width": 3.0, "r_max": 3.0,
                   "bins": 300},
        "cpu_baseline": {"value": value, "unit": "pair evals/s", "cores": cores, "kind": "port", "sample": desc},
        "e2e": {"value": value, "unit": "pair evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_only(args):
    import torch

    torch.cuda.set_device(0)
    from freud_gb300 import _lib

    import freud_gb300 as freud

    stream = torch.cuda.Stream()
    _lib.set_stream(stream.cuda_stream)
    torch.cuda.set_stream(stream)
    if args.batch_config:
        _lib.set_batch_config(*[int(x) for x in args.batch_config.split(",")])
    fns = {"plain_rdf": lambda: measure_c1(freud, _lib, args.steps, args.warmup, cpu=False),
           "steinhardt": lambda: measure_c3(freud, _lib, args.steps, args.warmup, cpu=not args.no_cpu_baseline),
           "correlation_function": lambda: measure_cf(freud, _lib, args.steps, args.warmup, cpu=False),
           "pmft": lambda: measure_pmft(freud, _lib, args.steps, args.warmup, cpu=False),
           "batched_frames": lambda: measure_c4(freud, _lib, args.steps, args.warmup, 8 if args.small else 64),
           "precision_stress": lambda: measure_c5(freud, _lib, args.steps, args.warmup, args.small)}
    print(json.dumps({"only": args.only, "result": fns[args.only]()}), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true",
                    help="skip the plain-RDF, Steinhardt, batched-frames and stress workloads")
    ap.add_argument("--n-side", type=int, default=102,
                    help="lattice points per side; 102 is the benchmark workload, smaller sizes are for profiling")
    ap.add_argument("--only", default=None, choices=["plain_rdf", "steinhardt", "correlation_function", "pmft",
                                                     "batched_frames", "precision_stress"],
                    help="run one of the other workloads alone and print its result (profiling)")
    ap.add_argument("--small", action="store_true",
                    help="with --only: the profiling-size case (8 frames; 512 blobs in L = 128)")
    ap.add_argument("--batch-config", default=None,
                    help="SHELL,WARPS,COPIES: fix the batched histogram's launch shape instead of autotuning "
                         "(profiling: no trial launches)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.only:
        return run_only(args)

    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from freud_gb300 import _lib

    import freud_gb300 as freud

    bad = []
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

    # roofline: the NeighborList build (every kernel of the step but the RDF over the
    # finished list) against its algorithmic bytes, 12 N (positions read) + 24 B
    # ((i, j) 8 B, distance 4 B, vector 12 B written per bond; weights are lazy)
    peak, peak_kind = read_peaks()
    rdf_names = ("k_hist_distances",)
    build = {k: v for k, v in prof.items() if not k.startswith(rdf_names)}
    build_ms = sum(v[1] for v in build.values()) / max(args.steps, 1)
    build_bytes = 12.0 * n + 24.0 * bonds
    build_gbs = build_bytes / (build_ms / 1e3) / 1e9 if build_ms > 0 else 0.0
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            tj = json.load(f)
        # DRAM bytes per launch x launches per step, over the build's kernels
        per_kernel = [None if tj.get(k) is None else tj[k] * v[0] / max(args.steps, 1) for k, v in build.items()]
        if per_kernel and all(x is not None for x in per_kernel):
            traffic = float(sum(per_kernel))
    except (OSError, ValueError):
        pass
    dom_name, (dom_n, dom_ms) = max(prof.items(), key=lambda kv: kv[1][1]) if prof else (None, (0, 0.0))

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

    # ---- e2e with the NeighborList read back: nlist[:], distances, vectors as a freud
    # user reads them (24 B per bond device -> host; weights are read only when asked for)
    rb_times = []
    gpu_list = None
    n_rb = 1 + max(1, min(args.steps, 3))
    for it in range(n_rb):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lc = freud.locality.LinkCell(box, pinned, 3.0)
        nlist = lc.query(pinned, {"r_max": 3.0, "exclude_ii": True}).toNeighborList()
        r = freud.density.RDF(300, 3.0).compute(lc, neighbors=nlist)
        counts = r.bin_counts
        ij, d, v = nlist[:], nlist.distances, nlist.vectors
        t1 = time.perf_counter()
        if it >= 1:
            rb_times.append(t1 - t0)
        if it == n_rb - 1:
            gpu_list = (ij, d, v, counts)  # kept for the parity check
        del lc, nlist, r, ij, d, v  # a user's arrays go before the next step's come back
    rb_value = bonds * world / statistics.median(rb_times)

    # ---- CPU baseline (rank 0, N=1 only): the oracle over the whole workload, whose
    # list is also the parity reference (identical neighbour sets, distances, vectors
    # and RDF counts, in the reference's order) ------------------------------------------
    cpu = None
    parity = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, desc, cores, dt, ref = cpu_baseline(L, pts_host)
        cpu = {"value": v, "unit": "pair evals/s", "cores": cores, "kind": "port", "sample": desc,
               "seconds": round(dt, 2)}
        ij, d, vv, counts = gpu_list
        rij, rd, rv, rcounts = ref
        same_n = len(ij) == len(rij)
        checks = {"bonds_gpu": int(len(ij)), "bonds_oracle": int(len(rij)),
                  "ij": bool(same_n and np.array_equal(ij, rij)),
                  "distances": bool(same_n and np.array_equal(d.view(np.uint32), rd.view(np.uint32))),
                  "vectors": bool(same_n and np.array_equal(vv.view(np.uint32), rv.view(np.uint32))),
                  "rdf_counts": bool(np.array_equal(np.asarray(counts, np.uint64), rcounts))}
        ok = all(checks[k] for k in ("ij", "distances", "vectors", "rdf_counts"))
        parity = dict(checks, status="bit-exact" if ok else "MISMATCH",
                      what="full NeighborList (every query point) and RDF counts, GPU through the public API "
                           "vs the CPU oracle, bitwise")
        del ref, rij, rd, rv
    del gpu_list

    # ---- the other workloads (rank 0, N=1): plain RDF, Steinhardt, batched frames, stress
    secondary = None
    if rank == 0 and world == 1 and not args.no_secondary:
        secondary = {}
        for name, fn in (("plain_rdf", lambda: measure_c1(freud, _lib, args.steps, args.warmup,
                                                            cpu=not args.no_cpu_baseline)),
                         ("steinhardt", lambda: measure_c3(freud, _lib, args.steps, args.warmup,
                                                            cpu=not args.no_cpu_baseline)),
                         ("correlation_function", lambda: measure_cf(freud, _lib, args.steps, args.warmup,
                                                                     cpu=not args.no_cpu_baseline)),
                         ("pmft", lambda: measure_pmft(freud, _lib, args.steps, args.warmup,
                                                       cpu=not args.no_cpu_baseline)),
                         ("batched_frames", lambda: measure_c4(freud, _lib, args.steps, args.warmup)),
                         ("precision_stress", lambda: measure_c5(freud, _lib, args.steps, args.warmup))):
            try:
                secondary[name] = fn()
            except Exception as e:  # report, do not hide, a failing secondary workload
                secondary[name] = {"error": "%s: %s" % (type(e).__name__, e)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "pair evals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered 102^3 lattice)",
            "config": {"workload": WORKLOAD if args.n_side == 102 else "%s_n%d" % (WORKLOAD, args.n_side), "n_points": n, "box_L": L, "cell_width": 3.0, "r_max": 3.0,
                       "bins": 300, "bonds_per_step": bonds, "l2": "flushed between steps (258 MB write)",
                       "parallelism": "replicas" if world > 1 else "single"},
            "roofline": {"bound": "hbm", "kernel": "NeighborList build: " + ", ".join(sorted(build)),
                         "achieved": build_gbs, "peak": peak, "peak_source": peak_kind, "unit": "GB/s",
                         "frac": build_gbs / peak, "traffic": traffic, "algorithmic_bytes_per_launch": build_bytes,
                         "algorithmic_bytes": "12*N + 24*B (positions read; (i,j), distance, vector written per "
                                              "bond; weights are lazy)",
                         "launch_ms": build_ms, "dominant_kernel": dom_name,
                         "dominant_kernel_ms": dom_ms / max(dom_n, 1)},
            "kernels": {k: {"launches": v[0], "total_ms": round(v[1], 4)} for k, v in sorted(prof.items())},
            "secondary": secondary,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "pair evals/s", "h2d_bytes_per_step": int(12 * n),
                    "d2h_bytes_per_step": int(300 * 4)},
            "e2e_nlist_readback": {"value": rb_value, "unit": "pair evals/s", "h2d_bytes_per_step": int(12 * n),
                                   "d2h_bytes_per_step": int(24 * bonds + 300 * 4),
                                   "what": "the e2e step plus nlist[:], distances and vectors read to host"},
            "parity": {"large_n_nlist_rdf": parity},
            "gpu_launches": int(launches),
            "clocks": clk,
        }
        if secondary:
            for k, sec in secondary.items():
                if isinstance(sec, dict) and "parity" in sec:
                    line["parity"][k] = sec["parity"]
        print(json.dumps(line), flush=True)
        bad = [k for k, v in line["parity"].items() if v is not None and v.get("status") not in PARITY_OK]
        if bad:
            print("parity check failed for: " + ", ".join(bad), file=sys.stderr)
    lib.fg_rdf_destroy(rdf)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 1 if rank == 0 and bad else 0


if __name__ == "__main__":
    sys.exit(main())
