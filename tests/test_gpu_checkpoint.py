"""Checkpoint/restart on the GPU in the reference's binary format.

- A file the reference wrote (EAM Al 500 after 5 steps) resumes here without
  FirstRun (CONTINUE_MODE: the stored forces drive the first half-kick) and
  reaches Step 10 as the reference's own continuation does: positions within
  1e-6 A, velocities within 1e-4 of their scale, ledger kinetic 1e-6 and
  potential 5e-8 relative (the EAM NVE tolerances: FP32 forces).
- A context saved after 5 steps writes exactly its state (positions and
  velocities bit for bit, Step, elapsed time, ledger, box), and a context
  loaded from that file continues like the original: positions within 1e-8 A
  after 5 more steps (the two differ only in the FP32 summation order of
  their neighbour rows).
"""
import os

import numpy as np
import pytest

from conftest import GOLD, TABLES, load_case

pytestmark = pytest.mark.gpu

EAM_TABLE = os.path.join(TABLES, "eam.aluminum5000")


def reference_file(tmp_path):
    d = np.load(os.path.join(GOLD, "checkpoint_eam_al_500.npz"))
    path = tmp_path / "reference.bin"
    path.write_bytes(d["binary"].tobytes())
    return str(path), d


def eam_setup(ctx, dt):
    ctx.add_eam(EAM_TABLE)
    ctx.set_neighbor(skin=0.3, rebuild_every=1)
    ctx.set_timestep(dt)


def test_resume_from_the_reference_checkpoint(omdg_lib, tmp_path):
    path, d = reference_file(tmp_path)
    dt = float(d["dt"])
    with omdg_lib.Context(0) as ctx:
        conts = ctx.load_simulation(path)
        assert len(conts) == 1 and conts[0].natoms == 500
        eam_setup(ctx, dt)
        ctx.step(5)
        st = ctx.get_state()
        kin, pot = ctx.ledger_history()
        out = str(tmp_path / "after.bin")
        ctx.save_simulation(out, conts)
    v, _, _, _, _ = omdg_lib.checkpoint_read(out)
    assert v.step == 10
    assert abs(v.elapsed_time - 0.02) < 1e-15
    # reference rows: step kinetic potential energy; row 0 is written before
    # the run, row 1 is the loaded Step 5, rows 2.. are Steps 6..10
    ref = d["ledger"]
    assert v.base_potential == omdg_lib.checkpoint_read(path)[0].base_potential
    L = np.array(v.box[6:9])
    dx = st["x"] - d["x10"]
    dx -= np.round(dx / L) * L
    assert np.abs(dx).max() < 1e-6
    assert np.abs(st["v"] - d["v10"]).max() < 1e-4 * np.abs(d["v10"]).max()
    assert len(kin) == 5 and list(ref[2:7, 0]) == [6, 7, 8, 9, 10]
    np.testing.assert_allclose(kin, ref[2:7, 1], rtol=1e-6)
    np.testing.assert_allclose(pot, ref[2:7, 2], rtol=5e-8)


def test_save_load_round_trip_continues(omdg_lib, tmp_path):
    from objectmd_gb300 import inputs

    d = load_case("eam_al_500")
    mass = inputs.md_mass("aluminum")
    path = str(tmp_path / "ctx.bin")
    conts = [omdg_lib.container("Aluminum", len(d["x0"]), id=0, mass=mass, z=13.0, material="aluminum")]
    with omdg_lib.Context(0) as a:
        a.set_box(d["box_lo"], d["box_hi"], (True, True, True))
        a.set_atoms(d["x0"], d["v0"], masses=[mass], znum=[13.0])
        eam_setup(a, 0.002)
        a.step(5)
        st5 = a.get_state()
        led5 = a.ledger()
        a.save_simulation(path, conts)
        v, _, conts2, atoms, _ = omdg_lib.checkpoint_read(path)
        assert v.step == 5 and abs(v.elapsed_time - 0.01) < 1e-15
        assert v.kinetic == led5["kinetic"] and v.potential == led5["potential"]
        assert v.base_potential == led5["base_potential"]
        np.testing.assert_array_equal(np.stack([atoms["x"], atoms["y"], atoms["z"]], 1), st5["x"])
        np.testing.assert_array_equal(np.stack([atoms["vx"], atoms["vy"], atoms["vz"]], 1), st5["v"])
        np.testing.assert_array_equal(np.stack([atoms["fx"], atoms["fy"], atoms["fz"]], 1), st5["f"])
        assert (atoms["nid"] == np.arange(len(atoms))).all() and (atoms["flag"] == 1).all()
        assert conts2[0].name == b"Aluminum" and conts2[0].natoms == len(atoms)
        a.step(5)
        st_a = a.get_state()
        led_a = a.ledger()
    with omdg_lib.Context(0) as b:
        b.load_simulation(path)
        eam_setup(b, 0.002)
        b.step(5)
        st_b = b.get_state()
        led_b = b.ledger()
    assert np.abs(st_a["x"] - st_b["x"]).max() < 1e-8
    assert np.abs(st_a["v"] - st_b["v"]).max() < 1e-6
    assert abs(led_a["potential"] - led_b["potential"]) < 1e-9 * abs(led_a["potential"])
    assert led_a["base_potential"] == led_b["base_potential"]
