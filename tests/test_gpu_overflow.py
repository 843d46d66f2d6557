"""Neighbour rows that overflow inside queued steps.

The reference grows each atom's row as it fills (VerletListFull.cpp:127-136),
so a run never stops for lack of room.  Here rows have a fixed capacity; when
a rebuild inside queued steps needs more, omdg_sync restores the state that
rebuild started from, grows the rows, redoes the step and replays the rest.
The test starts a converging flow (atoms of an EAM Al box driven toward its
centre, so the density and the row lengths grow) with a row capacity just
above the initial longest row, and compares it with the same run with ample
rows: positions, velocities, forces and the ledger must be equal bit for bit.
"""
import os

import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu

EAM_TABLE = os.path.join(TABLES, "eam.aluminum5000")


def converging_box():
    from objectmd_gb300 import inputs

    x, v, (lo, hi) = inputs.eam_aluminium(ncell=10, a=4.05, sigma=0.05, temp=300.0, seed_pos=51, seed_vel=52)
    c = 0.5 * (np.array(lo) + np.array(hi))
    d = x - c
    r = np.linalg.norm(d, axis=1)
    inner = r < 15.0
    v = v.copy()
    v[inner] -= 1.5 * d[inner]  # up to ~22 A/ps toward the centre
    return x, v, lo, hi


def run(omdg, capacity, batches):
    from objectmd_gb300 import inputs

    x, v, lo, hi = converging_box()
    ctx = omdg.Context(0)
    ctx.set_box(lo, hi)
    ctx.set_atoms(x, v, masses=[inputs.md_mass("aluminum")], znum=[13.0])
    ctx.add_eam(EAM_TABLE)
    if capacity:
        ctx.set_launch("nbr_capacity", capacity)
    ctx.set_neighbor(0.3, 0)
    ctx.set_timestep(0.002)
    kin, pot = [], []
    for nb in batches:
        ctx.step(nb)
        k, p = ctx.ledger_history()
        kin.append(k)
        pot.append(p)
    st = ctx.get_state()
    off = ctx.neighbors()[0]
    ctx.close()
    return st, np.concatenate(kin), np.concatenate(pot), np.diff(off)


def test_row_overflow_replays_to_the_ample_trajectory(omdg_lib):
    from objectmd_gb300 import inputs

    x, v, lo, hi = converging_box()
    with omdg_lib.Context(0) as ctx:
        ctx.set_box(lo, hi)
        ctx.set_atoms(x, v, masses=[inputs.md_mass("aluminum")], znum=[13.0])
        ctx.add_eam(EAM_TABLE)
        ctx.set_neighbor(0.3, 0)
        ctx.build_neighbors()
        first_max = int(np.diff(ctx.neighbors()[0]).max())
    batches = (60, 25, 15)
    ample, kin_a, pot_a, rows_a = run(omdg_lib, 0, batches)
    tight, kin_t, pot_t, rows_t = run(omdg_lib, first_max + 1, batches)
    # the compression lengthened the rows past the tight capacity: rows grew in the run
    assert rows_t.max() > first_max + 1, (rows_t.max(), first_max)
    assert np.array_equal(rows_t, rows_a)
    for k in ("x", "v", "f", "pot"):
        assert np.array_equal(tight[k], ample[k]), k
    assert np.array_equal(kin_t, kin_a)
    assert np.array_equal(pot_t, pot_a)
