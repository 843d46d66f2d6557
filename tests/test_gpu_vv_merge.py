"""Queued steps with each step boundary in one pass (k_kick_next: one
step's second half-kick and ledger row, then the next step's first
half-kick and drift) against the same steps with the two kernels apart
(launch key vv_merge).  The kernel applies the same operations to each atom
in the same order, so positions, velocities, forces and the ledger agree
bit for bit, rebuilds included; the merged batch launches one kernel fewer
per step boundary.
"""
import os

import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu


def run(omdg, make, merge, batches):
    with omdg.Context(0) as ctx:
        make(ctx)
        ctx.set_launch("vv_merge", merge)
        for n in batches:
            ctx.step(n)
        kin, pot = ctx.ledger_history()
        return ctx.get_state(), kin, pot, ctx.stats()


def check_same(a, b):
    (sa, ka, pa, ta), (sb, kb, pb, tb) = a, b
    for k in ("x", "v", "f", "pot", "vir"):
        assert np.array_equal(sa[k], sb[k]), k
    assert np.array_equal(ka, kb) and np.array_equal(pa, pb)
    assert ta["rebuilds"] == tb["rebuilds"] and ta["rebuilds"] >= 2
    return ta, tb


def test_eam_steps_merged_equal_apart(omdg_lib):
    from objectmd_gb300 import inputs

    x, v, (lo, hi) = inputs.eam_aluminium(ncell=12, a=4.05, sigma=0.05, temp=600.0, seed_pos=81, seed_vel=82)

    def make(ctx):
        ctx.set_box(lo, hi)
        ctx.set_atoms(x, v, masses=[inputs.md_mass("aluminum")], znum=[13.0])
        ctx.add_eam(os.path.join(TABLES, "eam.aluminum5000"))
        ctx.set_neighbor(0.1, 0)
        ctx.set_timestep(0.002)

    batches = (1, 17, 2, 20)
    ta, tb = check_same(run(omdg_lib, make, 1, batches), run(omdg_lib, make, 0, batches))
    # step boundaries inside the batches of two or more steps: 16 + 1 + 19
    assert tb["launches"] - ta["launches"] == 36


def test_tersoff_steps_merged_equal_apart(omdg_lib):
    from objectmd_gb300 import inputs

    x, v, (lo, hi) = inputs.diamond_silicon(ncell=6, a=5.431, sigma=0.03, temp=1500.0, seed_pos=83, seed_vel=84)

    def make(ctx):
        ctx.set_box(lo, hi)
        ctx.set_atoms(x, v, masses=[inputs.md_mass("silicon")], znum=[14.0])
        ctx.add_tersoff(os.path.join(TABLES, "tersoff.silicon27"))
        ctx.set_neighbor(0.1, 0)
        ctx.set_timestep(0.001)

    check_same(run(omdg_lib, make, 1, (30,)), run(omdg_lib, make, 0, (30,)))


def test_thermostat_keeps_the_kernels_apart(omdg_lib):
    """A Berendsen thermostat acts between the two half-kicks (its factor
    needs the whole kinetic energy): the batch runs the separate kernels."""
    from objectmd_gb300 import inputs

    x, v, (lo, hi) = inputs.eam_aluminium(ncell=8, a=4.05, sigma=0.05, temp=300.0, seed_pos=85, seed_vel=86)

    def make(ctx):
        ctx.set_box(lo, hi)
        ctx.set_atoms(x, v, masses=[inputs.md_mass("aluminum")], znum=[13.0])
        ctx.add_eam(os.path.join(TABLES, "eam.aluminum5000"))
        ctx.set_neighbor(0.1, 0)
        ctx.set_timestep(0.002)
        ctx.set_thermostat(600.0, 0.05)

    a, b = run(omdg_lib, make, 1, (20,)), run(omdg_lib, make, 0, (20,))
    ta, tb = check_same(a, b)
    assert ta["launches"] == tb["launches"]
