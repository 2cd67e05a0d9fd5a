"""Writes tests/golden/restart/: a restart directory of a seeded 5 x 4 x 3
grid with five species (two tiles along x plus master.hdf), made by the
library's restart writer (include/htr_restart.h) from host arrays.  The
files pin the writer's bytes: tests/test_restart.py rewrites the same
directory and compares byte for byte, and reads these files back with the
independent oracle reader.

    python tests/golden/make_restart_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "restart")
SPECIES = ["N2", "O2", "NO", "N", "O"]


def fields():
    """The seeded restart fields, by name, shaped (z, y, x[, comp])."""
    from htr_gb300 import fluid, restart
    f = fluid.Fluid((5, 4, 3), 5, fields=list(restart.IO_FIELDS))
    rng = np.random.default_rng(2024)
    for n in restart.IO_FIELDS:
        f[n] = rng.standard_normal(f[n].shape)
    return f


def write(out):
    from htr_gb300 import restart
    f = fields()
    restart.dump(out, f, tiles=(2, 1, 1), time_step=1234, sim_time=0.5, channel_forcing=0.0,
                 species_names=SPECIES, versions=["golden-1", "legion-x"])
    return f


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import __graft_entry__
    __graft_entry__.load_package()
    write(OUT)
    print("\n".join(sorted(os.listdir(OUT))))
