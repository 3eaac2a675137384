"""Regenerate tests/golden/tracks_3x2.moctrk, the golden track file.

Run from the repository root:

    python tests/golden/make_trackfile.py

Everything comes from the oracle, not the product: the oracle's plan of a 3 x 2 lattice
(1.26 cm pitch, 3 rings, 10 cm in 2 axial regions of 5 fine intervals; 4 azimuths, 2 polar
bins, 0.4 cm radial and 2 cm axial spacing), its sort-all-crossings tracer, and its own
writer of the format of include/moc_trackfile.h. tests/test_trackfile.py checks that the
library reads this file to the same descriptors and writes the same bytes from them.
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "simplemoc-kernel_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import mocatt  # noqa: E402  (the geometry structs)
import oracle  # noqa: E402

GEOMETRY = dict(nx=3, ny=2, n_axial=2, height=10.0)
QUADRATURE = dict(n_azim=4, n_polar=2, spacing=0.4, axial_spacing=2.0)
PATH = os.path.join(HERE, "tracks_3x2.moctrk")


def main():
    oracle.build()
    g, q = mocatt.geometry(**GEOMETRY), mocatt.quadrature(**QUADRATURE)
    plan = oracle.tracks_plan(g, q)
    off, reg, itv, ds = oracle.trace(g, plan)
    R = g.nx * g.ny * (g.n_rings + 1) * g.n_axial
    with open(PATH, "wb") as f:
        f.write(oracle.trackfile_bytes(R, g.n_intervals, off, reg, itv, ds))
    print(f"{PATH}: {len(plan)} tracks, {off[-1]} segments")


if __name__ == "__main__":
    main()
