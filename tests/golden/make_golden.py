"""Generates the golden fixtures in tests/golden/ from the reference's own CPU
sources (compiled in place by oracle/build_ref.sh into oracle/_ref/).

Run here, where the reference tree exists:  python tests/golden/make_golden.py
Each fixture stores its seeded inputs and the reference outputs; the CPU tests
pin the oracle to them bit for bit, the GPU tests pin the CUDA path.
"""

import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref as R  # noqa: E402


def absolute(box, frac):
    """Box::makeAbsolute in float32 (box = (Lx, Ly, Lz, xy, xz, yz, is2D))."""
    b = np.asarray(box, np.float32)
    L = b[:3].copy()
    if box[6]:
        L[2] = 0
    lo = -(L / np.float32(2))
    f = np.asarray(frac, np.float32)
    v = lo + f * L
    x = v[:, 0] + (b[3] * v[:, 1] + b[4] * v[:, 2])
    y = v[:, 1] + b[5] * v[:, 2]
    z = v[:, 2] if not box[6] else np.zeros_like(x)
    return np.stack([x, y, z], 1).astype(np.float32)


def random_system(L, n, seed, tilt=(0.0, 0.0, 0.0), is2d=False):
    rs = np.random.RandomState(seed)
    f = rs.random_sample((n, 3))
    if is2d:
        f[:, 2] = 0
    box = (L, L, 0.0 if is2d else L, tilt[0], 0.0 if is2d else tilt[1], 0.0 if is2d else tilt[2], 1 if is2d else 0)
    return box, absolute(box, f)


def fcc(ncell, a, sigma, seed):
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(*(np.arange(ncell),) * 3, indexing="ij"), -1).reshape(-1, 3)
    L = ncell * a
    pts = ((basis[:, None, :] + g[None]).reshape(-1, 3) + 0.25) * a - L / 2
    rs = np.random.RandomState(seed)
    pts = pts + rs.normal(0, sigma, pts.shape)
    pts = (pts + L / 2) % L - L / 2
    return (L, L, L, 0.0, 0.0, 0.0, 0), pts.astype(np.float32)


def save(name, **arrays):
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **arrays)
    print("wrote", path, os.path.getsize(path), "bytes")


def main():
    subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh")])
    assert R.available(), "oracle/_ref/libfreud_ref.so missing"

    # ball queries: AABB (RawPoints default) and LinkCell arithmetic, cubic / triclinic / 2D
    cases = [
        ("ball_aabb_cubic", R.KIND_RAW, random_system(8.0, 400, 11), 2.0, 0.0, 0.0),
        ("ball_aabb_triclinic", R.KIND_AABB, random_system(9.0, 400, 12, (0.2, 0.1, 0.0)), 2.0, 0.0, 0.0),
        ("ball_aabb_2d", R.KIND_AABB, random_system(10.0, 300, 13, is2d=True), 1.7, 0.0, 0.0),
        ("ball_lc_cubic", R.KIND_LINKCELL, random_system(8.0, 400, 14), 2.0, 0.5, 2.0),
        ("ball_lc_triclinic", R.KIND_LINKCELL, random_system(9.0, 400, 15, (0.5, -0.3, 0.25)), 2.2, 0.0, 2.2),
        ("ball_lc_2d", R.KIND_LINKCELL, random_system(10.0, 300, 16, (0.3, 0, 0), is2d=True), 1.5, 0.0, 1.0),
        ("ball_lc_small_box", R.KIND_LINKCELL, random_system(5.0, 60, 17), 2.45, 0.0, 1.0),
    ]
    for name, kind, (box, pts), r_max, r_min, cw in cases:
        for by_dist in (False, True):
            ij, d, w, v = R.query(kind, box, pts, pts, mode=R.MODE_BALL, r_max=r_max, r_min=r_min,
                                  exclude_ii=True, cell_width=cw, sort_by_distance=by_dist)
            save(name + ("_bydist" if by_dist else ""), box=np.asarray(box, np.float32), points=pts, kind=kind,
                 r_max=np.float32(r_max), r_min=np.float32(r_min), cell_width=np.float32(cw), ij=ij, d=d, v=v)

    # CellQuery (ghost copies; third arithmetic): cubic / triclinic with some points
    # outside the box (their copies beyond the padded grid are dropped) / 2D
    def spill_system(L, n, seed, tilt, spill):
        rs = np.random.RandomState(seed)
        f = rs.random_sample((n, 3)) * (1 + 2 * spill) - spill
        box = (L, L, L, tilt[0], tilt[1], tilt[2], 0)
        return box, absolute(box, f)

    cq_cases = [
        ("ball_cq_cubic", random_system(8.0, 400, 61), 2.0, 0.0),
        ("ball_cq_triclinic_spill", spill_system(9.0, 400, 62, (0.3, -0.2, 0.1), 0.06), 2.2, 0.4),
        ("ball_cq_2d", random_system(10.0, 300, 63, (0.25, 0, 0), is2d=True), 1.7, 0.0),
    ]
    for name, (box, pts), r_max, r_min in cq_cases:
        for by_dist in (False, True):
            ij, d, w, v = R.query(R.KIND_CELLQUERY, box, pts, pts, mode=R.MODE_BALL, r_max=r_max, r_min=r_min,
                                  exclude_ii=True, sort_by_distance=by_dist)
            save(name + ("_bydist" if by_dist else ""), box=np.asarray(box, np.float32), points=pts,
                 kind=R.KIND_CELLQUERY, r_max=np.float32(r_max), r_min=np.float32(r_min), ij=ij, d=d, v=v)
    box, pts = random_system(8.0, 300, 64, (0.1, 0.2, 0.0))
    _, qpts = spill_system(8.0, 120, 65, (0.1, 0.2, 0.0), 0.1)
    ij, d, w, v = R.query(R.KIND_CELLQUERY, box, pts, qpts, mode=R.MODE_BALL, r_max=1.9, exclude_ii=False)
    save("ball_cq_query_points", box=np.asarray(box, np.float32), points=pts, query_points=qpts,
         kind=R.KIND_CELLQUERY, r_max=np.float32(1.9), ij=ij, d=d, v=v)
    box, pts = random_system(9.0, 800, 66, (0.2, 0.0, 0.1))
    c, g, nr = R.rdf(90, 2.5, [(box, pts)], kind=R.KIND_CELLQUERY)
    save("rdf_cellquery", box=np.asarray(box, np.float32), points=pts, bins=90, r_max=np.float32(2.5), counts=c,
         rdf=g, n_r=nr)

    # query points different from the points
    box, pts = random_system(8.0, 300, 21)
    _, qpts = random_system(8.0, 100, 22)
    ij, d, w, v = R.query(R.KIND_AABB, box, pts, qpts, mode=R.MODE_BALL, r_max=1.8, exclude_ii=False)
    save("ball_aabb_query_points", box=np.asarray(box, np.float32), points=pts, query_points=qpts,
         kind=R.KIND_AABB, r_max=np.float32(1.8), ij=ij, d=d, v=v)

    # k nearest neighbours
    box, pts = fcc(4, 1.5874, 0.05, 31)
    for name, kind in (("knn_aabb_fcc", R.KIND_AABB), ("knn_lc_fcc", R.KIND_LINKCELL)):
        ij, d, w, v = R.query(kind, box, pts, pts, mode=R.MODE_NEAREST, num_neighbors=12, exclude_ii=True,
                              cell_width=1.6)
        save(name, box=np.asarray(box, np.float32), points=pts, kind=kind, k=12, ij=ij, d=d, v=v)
    box, pts = random_system(6.0, 200, 32, (0.2, 0.0, 0.1))
    ij, d, w, v = R.query(R.KIND_AABB, box, pts, pts, mode=R.MODE_NEAREST, num_neighbors=7, r_max=1.2,
                          exclude_ii=False)
    save("knn_aabb_rmax", box=np.asarray(box, np.float32), points=pts, kind=R.KIND_AABB, k=7,
         r_max=np.float32(1.2), ij=ij, d=d, v=v)

    # RDF: plain (default (box, points) query) and multi-frame reset=False with uneven N
    box, pts = random_system(10.0, 1000, 41)
    c, g, nr = R.rdf(100, 3.0, [(box, pts)])
    save("rdf_plain", box=np.asarray(box, np.float32), points=pts, bins=100, r_max=np.float32(3.0), counts=c,
         rdf=g, n_r=nr)
    frames = [random_system(8.0, 500, 42), random_system(9.0, 700, 43, (0.2, 0.1, 0.0)),
              random_system(7.5, 350, 44)]
    c, g, nr = R.rdf(80, 2.5, frames, r_min=0.5)
    arr = {}
    for f, (b, p) in enumerate(frames):
        arr["box%d" % f] = np.asarray(b, np.float32)
        arr["points%d" % f] = p
    save("rdf_frames", nframes=len(frames), bins=80, r_max=np.float32(2.5), r_min=np.float32(0.5), counts=c,
         rdf=g, n_r=nr, **arr)
    c, g, nr = R.rdf(60, 2.0, [random_system(6.0, 300, 45)], finite_size=True, exclude_ii=False)
    b, p = random_system(6.0, 300, 45)
    save("rdf_finite_size", box=np.asarray(b, np.float32), points=p, bins=60, r_max=np.float32(2.0), counts=c,
         rdf=g, n_r=nr)

    # Steinhardt (fsph stand-in values; compared with tolerance)
    box, pts = fcc(4, 1.5874, 0.05, 51)
    ls = np.array([4, 6, 8, 10, 12], np.uint32)
    for name, kw in (("st_knn_avg_wl", dict(average=True, wl=True, wl_normalize=True)),
                     ("st_knn_plain", dict())):
        o = R.steinhardt(ls, box, pts, mode=R.MODE_NEAREST, num_neighbors=12, **kw)
        save(name, box=np.asarray(box, np.float32), points=pts, ls=ls, ql=o["ql"], particle_order=o["particle_order"],
             order=o["order"], qlm=np.concatenate([q.reshape(-1) for q in o["qlm"]]),
             average=int(kw.get("average", False)), wl=int(kw.get("wl", False)),
             wl_normalize=int(kw.get("wl_normalize", False)))
    o = R.steinhardt([6], box, pts, mode=R.MODE_BALL, r_max=1.5)
    save("st_ball_l6", box=np.asarray(box, np.float32), points=pts, ls=np.array([6], np.uint32), r_max=np.float32(1.5),
         ql=o["ql"], particle_order=o["particle_order"], order=o["order"], qlm=o["qlm"][0].reshape(-1))


if __name__ == "__main__":
    main()
