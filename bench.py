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
    neighbours on a 256,000-point noisy FCC crystal."""
    L, pts = c3_system()
    box = freud.box.Box.cube(float(L))
    st = freud.order.Steinhardt([4, 6, 8, 10, 12], average=True, wl=True, wl_normalize=True)

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
    if cpu:
        from oracle import oracle as O

        bx = (float(L),) * 3 + (0.0, 0.0, 0.0, 0.0)
        m = 32000
        t0 = time.perf_counter()
        ij, d, v = O.query(bx, pts, query_points=pts[:m], num_neighbors=12, exclude_ii=True)
        tq = time.perf_counter() - t0
        ij_all, d_all, _ = O.query(bx, pts, num_neighbors=12, exclude_ii=True)
        t0 = time.perf_counter()
        O.steinhardt([4, 6, 8, 10, 12], bx, pts, ij_all, d_all, average=True, wl=True, wl_normalize=True)
        ts = time.perf_counter() - t0
        per_particle = tq / m + ts / n
        out["cpu_baseline"] = {"value": 1.0 / per_particle, "unit": "particles/s", "cores": os.cpu_count() or 1,
                               "kind": "port",
                               "sample": "kNN query of %d query points (all threads) + FP64 Steinhardt of all %d "
                                         "particles (1 thread)" % (m, n)}
    return out


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
            "autotune": _lib.autotune_report().strip().splitlines()[-1:] }


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
                               "skew_max_over_mean": float(occ.max() / occ.mean())}}


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
           "steinhardt": lambda: measure_c3(freud, _lib, args.steps, args.warmup, cpu=False),
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
    if dom_name is not None and ("EMIT" in dom_name or "emit" in dom_name):
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
    # the whole NeighborList build (grid + scan + write passes) against its output bytes
    build_names = ("k_assign", "k_scatter", "k_sort_cells", "k_tile_scan", "k_tile_sums", "k_cell_scan<COUNT>",
                   "k_cell_emit", "k_seg_from_offsets")
    build_ms = sum(v[1] for k, v in prof.items() if k.startswith(build_names)) / max(args.steps, 1)
    build_bytes = 12.0 * n + 24.0 * bonds
    build_gbs = build_bytes / (build_ms / 1e3) / 1e9 if build_ms > 0 else 0.0
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
            "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": peak,
                         "peak_source": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "algorithmic_bytes_per_launch": alg_bytes,
                         "algorithmic_bytes": alg_desc, "launch_ms": per_launch_ms,
                         "note": ("the scan pass reads positions and writes counts only (its masks and "
                                  "sorted candidate lists stay in L2): HBM is not what bounds it; ncu shows "
                                  "it instruction-bound (66% issue-active, "
                                  "profiles/k_cell_scan_k_cell_emit_k_hist_distances_262k.md); "
                                  "roofline_build gives the whole NeighborList build against its output bytes")
                         if dom_name is not None and "COUNT" in dom_name else None},
            "roofline_build": {"bound": "hbm", "what": "NeighborList build: grid + scan + write passes",
                               "achieved": build_gbs, "peak": peak, "unit": "GB/s", "frac": build_gbs / peak,
                               "algorithmic_bytes": "12*N + 24*B", "ms_per_step": build_ms},
            "kernels": {k: {"launches": v[0], "total_ms": round(v[1], 4)} for k, v in sorted(prof.items())},
            "secondary": secondary,
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
