"""Generates tests/golden/lj_traj.npz and tests/golden/gc_config.npz from the
reference's trajectory fixtures, read with freud_gb300.gsd, and from the
reference's own CPU sources (oracle/_ref).

* lj_traj.npz - the 10-frame Lennard-Jones trajectory of
  tests/integration/files/lj/lj.gsd (1000 particles, L = 20) with the known RDF
  of tests/integration/files/lj/rdf.npz (RDF(bins=100, r_max=5) accumulated over
  every frame, tests/integration/test_reader_integrations.py:34-41) and the
  compiled reference's bin counts, rdf, n_r and Steinhardt(6) with 6 nearest
  neighbours on the last frame.
* gc_config.npz - tests/validation/files/steinhardt_average/Test_Configuration.gsd
  (3288 particles) with the "GC" code's q4, q6, w4, w6 and their averaged forms
  (GC_rc1.4_*.txt; tests/validation/test_steinhardt_average.py:83-109) and the
  compiled reference's values for the same four parameter sets.

Run here, where the reference tree exists:
    python tests/golden/make_trajectory_fixtures.py
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from freud_gb300 import gsd  # noqa: E402
from oracle import ref as R  # noqa: E402

# the reference tree (FREUD_REFERENCE_DIR); this script only runs where it exists
REF = os.path.join(os.environ.get("FREUD_REFERENCE_DIR", "/root/reference"), "tests")
LJ_GSD = os.path.join(REF, "integration", "files", "lj", "lj.gsd")
LJ_RDF = os.path.join(REF, "integration", "files", "lj", "rdf.npz")
GC_DIR = os.path.join(REF, "validation", "files", "steinhardt_average")


def box7(frame):
    b = [float(x) for x in frame.configuration.box]
    is2d = frame.configuration.dimensions == 2
    if is2d:
        b[2] = b[4] = b[5] = 0.0
    return tuple(b) + (1 if is2d else 0,)


def gc_params(average):
    return [dict(ls=[4], average=average), dict(ls=[6], average=average),
            dict(ls=[4], average=average, wl=True, wl_normalize=True),
            dict(ls=[6], average=average, wl=True, wl_normalize=True)]


def main():
    with gsd.open(LJ_GSD) as traj:
        frames = list(traj)
    pos = np.stack([f.particles.position for f in frames]).astype(np.float32)
    boxes = np.array([box7(f) for f in frames], np.float64)
    steps = np.array([f.configuration.step for f in frames], np.int64)
    known = np.load(LJ_RDF)["rdf"].astype(np.float32)
    systems = [(tuple(b), p) for b, p in zip(boxes, pos)]
    counts, g, nr = R.rdf(100, 5.0, systems)
    np.testing.assert_allclose(g, known, rtol=1e-5, atol=1e-5)
    st = R.steinhardt([6], systems[-1][0], systems[-1][1], mode=R.MODE_NEAREST, num_neighbors=6)
    out = os.path.join(HERE, "lj_traj.npz")
    np.savez_compressed(out, positions=pos, boxes=boxes, steps=steps, rdf_known=known, ref_counts=counts,
                        ref_rdf=g, ref_n_r=nr, ref_q6_last=st["particle_order"][:, 0])
    print("wrote", out, os.path.getsize(out), "bytes")

    with gsd.open(os.path.join(GC_DIR, "Test_Configuration.gsd")) as traj:
        frame = traj[-1]
    b = box7(frame)
    p = frame.particles.position.astype(np.float32)
    gc = np.genfromtxt(os.path.join(GC_DIR, "GC_rc1.4_q4q6w4w6.txt")).astype(np.float32)
    gc_ave = np.genfromtxt(os.path.join(GC_DIR, "GC_rc1.4_avq4avq6avw4avw6.txt")).astype(np.float32)
    refs = {}
    for name, average, data in (("ref", False, gc), ("ref_ave", True, gc_ave)):
        cols = []
        for kw in gc_params(average):
            ls = kw.pop("ls")
            o = R.steinhardt(ls, b, p, kind=R.KIND_AABB, mode=R.MODE_BALL, r_max=1.4, exclude_ii=True, **kw)
            cols.append(o["particle_order"][:, 0])
        refs[name] = np.stack(cols, 1)
        np.testing.assert_allclose(refs[name], data, atol=2e-5)
    out = os.path.join(HERE, "gc_config.npz")
    np.savez_compressed(out, positions=p, box=np.array(b, np.float64), gc=gc, gc_ave=gc_ave, ref=refs["ref"],
                        ref_ave=refs["ref_ave"])
    print("wrote", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main()
