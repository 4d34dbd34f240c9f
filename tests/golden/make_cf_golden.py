"""Generates the CorrelationFunction fixtures tests/golden/cf_*.npz from the
reference's own CPU sources (oracle/_ref, CorrelationFunction.cc compiled in
place). Counts are exact; the FP64 correlation sums depend on summation order,
so the tests compare them with a tolerance.

Run here, where the reference tree exists:  python tests/golden/make_cf_golden.py
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from make_golden import fcc, random_system, save  # noqa: E402
from oracle import ref as R  # noqa: E402


def phases(n, seed):
    rs = np.random.RandomState(seed)
    return np.exp(1j * rs.random_sample(n) * 2.0 * np.pi)


def main():
    # two 2D frames, complex values, default query (ball r_max, exclude_ii)
    frames = [random_system(20.0, 400, 71, is2d=True), random_system(22.0, 450, 72, is2d=True)]
    vals = [phases(400, 73), phases(450, 74)]
    c, g = R.cf(20, 5.0, frames, vals)
    arr = {}
    for f, (b, p) in enumerate(frames):
        arr["box%d" % f] = np.asarray(b, np.float32)
        arr["points%d" % f] = p
        arr["values%d" % f] = vals[f]
    save("cf_complex_2d", nframes=2, bins=20, r_max=np.float32(5.0), counts=c, correlation=g, **arr)

    # 3D triclinic, real values, distinct query points with their own values
    box, pts = random_system(10.0, 500, 75, (0.1, 0.0, 0.2))
    _, qpts = random_system(10.0, 200, 76, (0.1, 0.0, 0.2))
    rs = np.random.RandomState(77)
    v = rs.standard_normal(500).astype(np.complex128)
    qv = rs.standard_normal(200).astype(np.complex128)
    c, g = R.cf(15, 3.0, [(box, pts)], [v], query_frames=[qpts], query_values=[qv], exclude_ii=False)
    save("cf_real_query_points", box=np.asarray(box, np.float32), points=pts, query_points=qpts, values=v,
         query_values=qv, bins=15, r_max=np.float32(3.0), counts=c, correlation=g)

    # k nearest neighbours (FCC), complex values
    box, pts = fcc(4, 1.5874, 0.05, 78)
    v = phases(len(pts), 79)
    c, g = R.cf(12, 2.4, [(box, pts)], [v], mode=R.MODE_NEAREST, num_neighbors=8, q_r_max=-1.0)
    save("cf_knn", box=np.asarray(box, np.float32), points=pts, values=v, k=8, bins=12, r_max=np.float32(2.4),
         counts=c, correlation=g)

    # LinkCell (wrap arithmetic), complex values
    box, pts = random_system(9.0, 700, 80, (0.2, 0.1, 0.0))
    v = phases(700, 81)
    c, g = R.cf(25, 2.5, [(box, pts)], [v], kind=R.KIND_LINKCELL, cell_width=2.5)
    save("cf_linkcell", box=np.asarray(box, np.float32), points=pts, values=v, cell_width=np.float32(2.5),
         bins=25, r_max=np.float32(2.5), counts=c, correlation=g)


if __name__ == "__main__":
    main()
