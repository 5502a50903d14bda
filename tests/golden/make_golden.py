"""Generate the golden fixtures of tests/test_golden.py from the oracle.

The reference cannot be built here and ships no golden vectors, so these fixtures are
oracle outputs on seeded small models: they pin the oracle against regressions and let
the GPU tests check the CUDA path without re-running the oracle.  Each fixture holds the
receiver seismograms after 16 steps (two full 8-step F/B cycles), per-component interior
checksums, and the full interior of Vz.

Run from the repository root: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from helpers import feed, interior, small_model  # noqa: E402
from oracle import oracle as O  # noqa: E402

KINDS = ["surface", "buried", "nofree", "moment", "water"]
NSTEPS = 16


def run(kind):
    m = small_model(kind)
    met = O.metric(m.x, m.y, m.z)
    o = feed(O.Oracle(m.ni, m.nj, m.nk, m.stept, free_surface=m.free_surface), m, met, kind)
    o.run(NSTEPS)
    fields = [interior(o.get_field(c)).astype(np.float32) for c in range(9)]
    sums = np.array([[f.astype(np.float64).sum(), (f.astype(np.float64) ** 2).sum(), np.abs(f).max()] for f in fields])
    return dict(seismo=o.get_seismo().astype(np.float32), checksums=sums, vz=fields[2])


if __name__ == "__main__":
    O.build()
    for kind in KINDS:
        np.savez_compressed(os.path.join(HERE, f"oracle_{kind}_16steps.npz"), **run(kind))
        print("wrote", kind)
