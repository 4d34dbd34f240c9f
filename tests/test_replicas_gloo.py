"""Several processes (one GPU each in production; the path has no device
collective): frame ranges and the host combination of RDF states, run as
world_size 2 over gloo on the CPU with each rank's counts from the oracle. The
combined state must equal one process accumulating every frame in order."""

import os
import socket

import numpy as np
import pytest

from oracle import oracle as O


def _frames():
    rs = np.random.RandomState(77)
    frames = []
    for f, n in enumerate([400, 250, 600, 330, 512]):
        L = (n / 0.9) ** (1.0 / 3.0)
        box = (L, L, L, 0.1 * (f % 2), 0.0, 0.0, 0.0)
        frac = rs.random_sample((n, 3))
        lo = -np.float32(L) / np.float32(2)
        pts = (lo + frac * np.float32(L)).astype(np.float32)
        pts[:, 0] += np.float32(box[3]) * pts[:, 1]
        frames.append((box, pts.astype(np.float32)))
    return frames


def _state_for(frames, lo, hi, bins, r_max):
    from freud_gb300.replicas import RDFState

    counts = np.zeros(bins, np.uint64)
    for f in range(lo, hi):
        box, pts = frames[f]
        O.rdf_counts_query(box, pts, bins, r_max, counts=counts, threads=1)
    if hi > lo:
        box, pts = frames[hi - 1]
        return RDFState(counts, hi - lo, tuple(box), len(pts), len(pts))
    return RDFState(counts, 0, (1.0, 1.0, 1.0, 0.0, 0.0, 0.0, 0), 0, 0)


def _rank_main(rank, world, port, queue):
    import torch.distributed as dist

    from freud_gb300.replicas import allgather_rdf_state, frame_range

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        frames = _frames()
        lo, hi = frame_range(len(frames), rank, world)
        merged = allgather_rdf_state(_state_for(frames, lo, hi, 60, 1.4))
        if rank == 0:
            queue.put(tuple(merged))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world", [1, 2, 3, 5, 7])
def test_frame_range_partitions(world):
    from freud_gb300.replicas import frame_range

    covered = []
    for r in range(world):
        lo, hi = frame_range(17, r, world)
        covered.extend(range(lo, hi))
        assert hi - lo in (17 // world, 17 // world + 1)
    assert covered == list(range(17))
    with pytest.raises(ValueError):
        frame_range(5, 3, 3)


def test_combine_keeps_last_nonempty_frame():
    from freud_gb300.replicas import RDFState, combine_rdf_states

    a = RDFState(np.array([1, 2], np.uint64), 2, (3.0, 3.0, 3.0, 0, 0, 0, 0), 10, 10)
    b = RDFState(np.array([5, 0], np.uint64), 1, (4.0, 4.0, 4.0, 0, 0, 0, 0), 12, 12)
    empty = RDFState(np.zeros(2, np.uint64), 0, (1.0, 1.0, 1.0, 0, 0, 0, 0), 0, 0)
    m = combine_rdf_states([a, b, empty])
    np.testing.assert_array_equal(m.counts, [6, 2])
    assert m.n_frames == 3 and m.box[0] == 4.0 and m.n_points == 12


def test_gloo_two_ranks_equal_one_process():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    del torch
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        merged = queue.get(timeout=180)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert all(p.exitcode == 0 for p in procs)
    frames = _frames()
    whole = _state_for(frames, 0, len(frames), 60, 1.4)
    counts, n_frames, box, n_points, n_query = merged
    np.testing.assert_array_equal(counts, whole.counts)
    assert n_frames == len(frames) and tuple(box) == tuple(whole.box) and n_points == whole.n_points
    # the float32 normalisation of the combined state equals the single-process one
    vol = np.float32(box[0]) * np.float32(box[1]) * np.float32(box[2])
    g1, n1 = O.rdf_reduce(counts, 1.4, 0.0, n_frames, n_points, n_query, vol)
    g2, n2 = O.rdf_reduce(whole.counts, 1.4, 0.0, whole.n_frames, whole.n_points, whole.n_query, vol)
    np.testing.assert_array_equal(g1, g2)
    np.testing.assert_array_equal(n1, n2)
