"""Generates the PMFT fixtures tests/golden/pmft_*.npz from the reference's own
CPU sources (oracle/_ref: PMFTR12.cc, PMFTXYT.cc, PMFTXY.cc, PMFTXYZ.cc compiled in
place): inputs, bin counts and float32 pair correlation functions.

Run here, where the reference tree exists:  python tests/golden/make_pmft_golden.py
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from make_golden import random_system, save  # noqa: E402
from oracle import ref as R  # noqa: E402


def angles(n, seed):
    return (np.random.RandomState(seed).random_sample(n) * 2 * np.pi).astype(np.float32)


def unit_quats(n, seed):
    q = np.random.RandomState(seed).standard_normal((n, 4))
    return (q / np.linalg.norm(q, axis=1, keepdims=True)).astype(np.float32)


def frames_arrays(frames, orient=None):
    arr = {}
    for f, (b, p) in enumerate(frames):
        arr["box%d" % f] = np.asarray(b, np.float32)
        arr["points%d" % f] = p
        if orient is not None:
            arr["orient%d" % f] = orient[f]
    return arr


def main():
    # R12: two 2D frames accumulated, self query
    frames = [random_system(16.0, 600, 91, is2d=True), random_system(15.0, 550, 92, (0.1, 0, 0), is2d=True)]
    orient = [angles(600, 93), angles(550, 94)]
    c, g = R.pmft(0, [3.0], [10, 8, 8], frames, orientations=orient, r_max=3.0)
    save("pmft_r12", nframes=2, maxes=np.float32([3.0]), bins=np.uint32([10, 8, 8]), counts=c, pcf=g,
         **frames_arrays(frames, orient))

    # XYT: self query, ball r_max = sqrt(x_max^2 + y_max^2)
    box, pts = random_system(14.0, 700, 95, is2d=True)
    o = angles(700, 96)
    rm = float(np.float32(np.sqrt(3.0 ** 2 + 2.5 ** 2)))
    c, g = R.pmft(1, [3.0, 2.5], [12, 10, 6], [(box, pts)], orientations=[o], r_max=rm)
    save("pmft_xyt", nframes=1, maxes=np.float32([3.0, 2.5]), bins=np.uint32([12, 10, 6]), counts=c, pcf=g,
         r_max=np.float32(rm), **frames_arrays([(box, pts)], [o]))

    # XY: query points with their own orientations
    box, pts = random_system(12.0, 500, 97, is2d=True)
    _, qpts = random_system(12.0, 200, 98, is2d=True)
    qo = angles(200, 99)
    rm = float(np.float32(np.sqrt(18.0)))
    c, g = R.pmft(2, [3.0, 3.0], [16, 16], [(box, pts)], query_frames=[qpts], query_orientations=[qo], r_max=rm,
                  exclude_ii=False)
    save("pmft_xy", nframes=1, maxes=np.float32([3.0, 3.0]), bins=np.uint32([16, 16]), counts=c, pcf=g,
         r_max=np.float32(rm), query_points=qpts, query_orient=qo, **frames_arrays([(box, pts)]))

    # XYZ: quaternion orientations, two equivalent orientations, shifted query points
    box, pts = random_system(9.0, 700, 100, (0.1, 0.0, 0.2))
    qq = unit_quats(700, 101)
    equiv = np.array([[1, 0, 0, 0], [np.cos(np.pi / 4), 0, 0, np.sin(np.pi / 4)]], np.float32)
    shift = np.float32([0.1, 0.0, -0.05])
    qpts = (pts - shift.reshape(1, 3)).astype(np.float32)
    rm = float(np.float32(np.sqrt(3 * 2.5 ** 2)))
    c, g = R.pmft(3, [2.5, 2.5, 2.5], [10, 10, 10], [(box, pts)], query_frames=[qpts], query_orientations=[qq],
                  equiv=equiv, r_max=rm, exclude_ii=True)
    save("pmft_xyz", nframes=1, maxes=np.float32([2.5, 2.5, 2.5]), bins=np.uint32([10, 10, 10]), counts=c,
         pcf=g, r_max=np.float32(rm), query_quats=qq, equiv=equiv, shiftvec=shift,
         **frames_arrays([(box, pts)]))


if __name__ == "__main__":
    main()
