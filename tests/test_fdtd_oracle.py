"""The finite-difference heat solver's oracle (oracle/fdtd_oracle.py) pinned
to the reference: the cell vectors of FDTDSolver (src/omd/fdtd.cpp compiled
from the reference tree, oracle/_ref/fdtd_driver) after every step of three
specs (tests/golden/fdtd_cases.npz), equal bit for bit.  The specs cover a 3D
slab with per-symbol and block values, ranged, future and external sources
and a cell outside the symbol map; the flags one all-'+' symbol loses at the
grid's edges; and a 2D grid (nz = 2) with periodic x, free y and cells of
zero conductivity."""
import os

import numpy as np
import pytest

from oracle import fdtd_oracle as fo

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fdtd_cases.npz")
SPECS = ("slab3d", "flat2d_cleared", "edges2d")


@pytest.mark.parametrize("name", SPECS)
def test_oracle_equals_the_reference(name):
    d = np.load(GOLD)
    rows = fo.run_spec(str(d[name + "_spec"]))
    assert np.array_equal(rows, d[name + "_rows"])


def test_periodic_grid_conserves_heat():
    """All faces periodic, no source: sum cap A is kept (to rounding) and
    the field relaxes toward its mean."""
    g = fo.Grid(5, 4, 6, "a pppppp", "a" * 120)
    g.set_spacestep(1.0)
    g.set_timestep(0.05)
    rng = np.random.default_rng(3)
    g.A = rng.uniform(100, 500, 120)
    g.set_capacity("@ 0,0,0,4,3,2=2.0")
    g.set_conductivity("@ 1,1,1,3,2,4=0.5")
    total0 = (g.A * g.cap).sum()
    spread0 = g.A.std()
    for _ in range(50):
        g.run_step()
    assert abs((g.A * g.cap).sum() - total0) < 1e-9 * total0
    assert g.A.std() < 0.5 * spread0
