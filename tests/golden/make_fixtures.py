"""Make tests/golden/ref_data.npz: the reference's example problems, parsed.

The GPU machine has no reference checkout, so the reference's own example files
that pin the solver on real data -- data/7camsvarK.txt + 7pts.txt,
data/54camsvarK.txt + 54pts.txt and data/Trafalgar-21-11315-{cams,pts}.txt,
the files PSBA/main.cpp:40-65 selects between -- travel as the arrays this
repository's reader makes of them (psba_gb300.io.load_scene, pinned
bit-for-bit to the reference's own reader by tests/test_io.py).  The
numbers are the files' own; this script only re-encodes them.

    python tests/golden/make_fixtures.py     (needs the reference checkout)
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import build  # noqa: E402
from psba_gb300 import io as pio  # noqa: E402

# name: (camera file, point file, points, observations) -- the counts the
# files hold (one observation per listed frame)
FIXTURES = {
    "7cams": ("7camsvarK.txt", "7pts.txt", 465, 1916),
    "54cams": ("54camsvarK.txt", "54pts.txt", 5207, 24609),
    "trafalgar21": ("Trafalgar-21-11315-cams.txt", "Trafalgar-21-11315-pts.txt", 11315, 36455),
}
OUT = os.path.join(ROOT, "tests", "golden", "ref_data.npz")


def load(name, data_dir):
    cams, pts, n_pts, n_obs = FIXTURES[name]
    sc = pio.load_scene(os.path.join(data_dir, cams), os.path.join(data_dir, pts), cnp=6, name=name)
    assert (sc.n_pts, sc.n_obs) == (n_pts, n_obs), (name, sc.n_pts, sc.n_obs)
    return sc


def main():
    d = build.reference_data_dir()
    if d is None:
        raise SystemExit("the reference checkout is not present (set PSBA_REFERENCE_DIR)")
    arrays = {}
    for name in FIXTURES:
        sc = load(name, d)
        assert sc.cov is None
        for k in ("K", "q0", "cams", "pts", "meas"):
            arrays["%s_%s" % (name, k)] = np.ascontiguousarray(getattr(sc, k), dtype=np.float64)
        arrays[name + "_obs_pt"] = sc.obs_pt.astype(np.int32)
        arrays[name + "_obs_cam"] = sc.obs_cam.astype(np.int32)
    np.savez_compressed(OUT, **arrays)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
