"""The impact-run modifies on the GPU against the reference running the same
modifies (tests/golden/modifies_eam_al_slab.npz, made by make_golden.py):
an EAM Al 500-atom slab with a free z surface, its top atom launched upward
at 60 A/ps, 30 steps of 2 fs, every atom targeted.

- ForceDamper(0.05) + CoordClamp("xyz"): CoordClamp::Init clamps y and z
  only (its `if(saxis.find('x'))` test), so the launched atom keeps vx alone.
- DynamicTimeStep(maxpath 0.02, max 0.004, update 3): the elapsed time after
  30 steps within 1e-6 relative (the time step follows the fastest atom).
- RangeLimiter(1.0): the escaping atom is deactivated at the same step and
  frozen; the same atoms stay active.
- EnergySource(0.05, start 0.01, width 0.02): the pulse rescales the same
  steps' velocities.

Positions within 1e-6 A, velocities within 1e-4 of their scale, ledger
kinetic 1e-6 and potential 5e-8 relative (the EAM NVE tolerances).
"""
import os

import numpy as np
import pytest

from conftest import GOLD, TABLES

pytestmark = pytest.mark.gpu

EAM_TABLE = os.path.join(TABLES, "eam.aluminum5000")


@pytest.fixture(scope="module")
def slab():
    from objectmd_gb300 import inputs

    x, v, types, (lo, hi), periodic = inputs.read_import(os.path.join(GOLD, "eam_al_slab.dat"))
    return x, v, lo, hi, periodic, np.load(os.path.join(GOLD, "modifies_eam_al_slab.npz"))


def run(omdg, slab, setup):
    from objectmd_gb300 import inputs

    x, v, lo, hi, periodic, d = slab
    with omdg.Context(0) as ctx:
        ctx.set_box(lo, hi, periodic)
        ctx.set_atoms(x, v, masses=[inputs.md_mass("aluminum")], znum=[13.0])
        ctx.add_eam(EAM_TABLE)
        ctx.set_neighbor(0.3, 1)
        ctx.set_timestep(float(d["dt"]))
        setup(ctx)
        ctx.step(int(d["steps"]))
        st = ctx.get_state()
        kin, pot = ctx.ledger_history()
        dt, elapsed = ctx.get_timestep()
        active = ctx.get_active()
    return st, kin, pot, dt, elapsed, active


def check(st, kin, pot, d, name):
    L = d["box_hi"] - d["box_lo"]
    dx = st["x"] - d[name + "_x"]
    dx[:, :2] -= np.round(dx[:, :2] / L[:2]) * L[:2]
    assert np.abs(dx).max() < 1e-6
    assert np.abs(st["v"] - d[name + "_v"]).max() < 1e-4 * np.abs(d[name + "_v"]).max()
    ref = d[name + "_ledger"]  # row 0 before the run, rows 1..30 the steps
    assert len(kin) == int(d["steps"])
    np.testing.assert_allclose(kin, ref[1:1 + len(kin), 1], rtol=1e-6)
    np.testing.assert_allclose(pot, ref[1:1 + len(pot), 2], rtol=5e-8)


def test_force_damper_and_coord_clamp(omdg_lib, slab):
    d = slab[-1]
    st, kin, pot, _, _, _ = run(omdg_lib, slab, lambda c: (c.add_force_damper(-1, 0.05),
                                                           c.add_coord_clamp(-1, "xyz")))
    check(st, kin, pot, d, "damp_clamp")
    assert (st["v"][:, 1:] == 0).all() and (st["v"][:, 0] != 0).any()  # y and z clamped, x free


def test_dynamic_timestep(omdg_lib, slab):
    d = slab[-1]
    st, kin, pot, dt, elapsed, _ = run(omdg_lib, slab, lambda c: c.set_dynamic_timestep(0.02, 0.004, 3))
    check(st, kin, pot, d, "dyndt")
    times = d["dyndt_times"]  # Step TimeStep ElapsedTime at each loop check
    assert times[-1, 0] == int(d["steps"])
    assert abs(elapsed - times[-1, 2]) < 1e-6 * times[-1, 2]
    assert times[0, 1] < 0.002  # the launched atom shortens the step from the start


def test_range_limiter(omdg_lib, slab):
    d = slab[-1]
    st, kin, pot, _, _, active = run(omdg_lib, slab, lambda c: c.add_range_limiter(-1, 1.0))
    check(st, kin, pot, d, "range")
    np.testing.assert_array_equal(active, d["range_active"].astype(bool))
    top = int(d["top"])
    assert not active[top] and active.sum() == len(active) - 1


def test_groups_select_the_atoms_a_modify_acts_on(omdg_lib, slab):
    """A clamp on group 1 holding only the launched atom: it alone loses vy
    and vz; a damper on group 0 (everything else) leaves it undamped."""
    d = slab[-1]
    top = int(d["top"])
    n = len(slab[0])
    member = np.ones(n, dtype=np.uint8)  # group 0
    member[top] = 2  # group 1

    def setup(c):
        c.set_groups(member)
        c.add_force_damper(0, 0.05)
        c.add_coord_clamp(1, "xyz")

    st, _, _, _, _, _ = run(omdg_lib, slab, setup)
    others = np.arange(n) != top
    assert st["v"][top, 1] == 0 and st["v"][top, 2] == 0 and st["v"][top, 0] != 0
    assert (st["v"][others, 1:] != 0).any()


def test_energy_source_pulse(omdg_lib, slab):
    """EnergySource(0.05 eV per atom, start 0.01 ps, width 0.02 ps): its first
    call at Step 5 only arms it, then Steps 6..14 scale the velocities."""
    d = slab[-1]
    st, kin, pot, _, _, _ = run(omdg_lib, slab, lambda c: c.add_energy_source(0.05, 0.01, 0.02))
    check(st, kin, pot, d, "source")
    ref = d["source_ledger"][1:, 1]
    assert ref[6] > ref[5] + 1.0  # the first scaled step
