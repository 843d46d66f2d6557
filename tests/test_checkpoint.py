"""The reference's binary checkpoint (MDSystem::SaveSimulation / LoadSimulation,
system.cpp:726-827; AtomContainer::Save / Load, container.cpp:554-680), host
side: the codec against a file the reference itself wrote
(tests/golden/checkpoint_eam_al_500.npz, EAM Al 500 saved after 5 steps), and,
where the reference build is present, the reference resuming from a file this
codec wrote.  No GPU needed.
"""
import os

import numpy as np
import pytest

from conftest import GOLD


def reference_file(tmp_path):
    d = np.load(os.path.join(GOLD, "checkpoint_eam_al_500.npz"))
    path = tmp_path / "reference.bin"
    path.write_bytes(d["binary"].tobytes())
    return str(path), d


def test_reader_parses_the_reference_file(omdg_lib, tmp_path):
    path, d = reference_file(tmp_path)
    v, stamp, conts, atoms, rv = omdg_lib.checkpoint_read(path)
    assert v.step == 5 and v.pboundary == 7 and v.write_mode == 0
    assert v.elapsed_time == 0.002 + 0.002 + 0.002 + 0.002 + 0.002  # ElapsedTime += dt per step
    assert v.energy == v.kinetic + v.potential - v.base_potential
    assert list(v.box[6:9]) == [v.box[1] - v.box[0], v.box[3] - v.box[2], v.box[5] - v.box[4]]
    assert list(v.box[9:12]) == [0.5 * b for b in v.box[6:9]]
    assert stamp[:3] in (b"Mon", b"Tue", b"Wed", b"Thu", b"Fri", b"Sat", b"Sun")
    assert rv == []
    assert len(conts) == 1
    c = conts[0]
    assert c.name == b"Aluminum" and c.material == b"aluminum" and c.natoms == 500 and c.z == 13.0
    assert abs(c.mass * 9648.53397731809 - 26.98) < 0.01  # M in simulation units (container.cpp:94)
    assert len(atoms) == 500
    assert (atoms["flag"] == 1).all() and (atoms["tid"] == 0).all()
    assert sorted(atoms["nid"]) == list(range(500))
    assert np.isfinite(atoms["x"]).all() and np.abs(atoms["fx"]).max() > 0


def test_writer_reproduces_the_reference_bytes(omdg_lib, tmp_path):
    path, _ = reference_file(tmp_path)
    v, stamp, conts, atoms, rv = omdg_lib.checkpoint_read(path)
    out = str(tmp_path / "ours.bin")
    omdg_lib.checkpoint_write(out, v, conts, atoms, rv, stamp=stamp.split(b"\0")[0].decode())
    assert open(out, "rb").read() == open(path, "rb").read()


def test_round_trip_with_containers_and_restart_variables(omdg_lib, tmp_path):
    rng = np.random.default_rng(3)
    n0, n1 = 7, 5
    atoms = np.zeros(n0 + n1, dtype=omdg_lib.ATOM_DTYPE)
    for name in ("x", "y", "z", "vx", "vy", "vz", "fx", "fy", "fz", "potential", "virial"):
        atoms[name] = rng.normal(size=n0 + n1)
    atoms["aux"] = rng.normal(size=(n0 + n1, omdg_lib.AUXVAR))
    atoms["tid"] = [0] * n0 + [1] * n1
    atoms["nid"] = np.arange(n0 + n1)
    atoms["gid"] = rng.integers(0, 9, n0 + n1)
    atoms["flag"] = 1
    conts = [omdg_lib.container("target", n0, id=0, mass=0.0029, z=14.0, material="silicon", param="a b"),
             omdg_lib.container("projectile", n1, id=1, mass=0.0041, z=18.0, material="argon")]
    v = omdg_lib.SimVars()
    v.step, v.pboundary, v.kinetic, v.potential, v.base_potential = 42, 3, 1.5, -2.5, -3.0
    v.energy = v.kinetic + v.potential - v.base_potential
    v.elapsed_time, v.begin_time = 0.021, 1234567
    for k in range(12):
        v.box[k] = float(k)
    path = str(tmp_path / "rt.bin")
    rvars = [("e_temp:", "5000"), ("int_Een:", "1.25e-3")]
    omdg_lib.checkpoint_write(path, v, conts, atoms, rvars, stamp="a stamp")
    v2, stamp, conts2, atoms2, rv2 = omdg_lib.checkpoint_read(path)
    assert bytes(v2) == bytes(v)
    assert stamp.split(b"\0")[0] == b"a stamp"
    assert rv2 == rvars
    assert [bytes(c) for c in conts2] == [bytes(c) for c in conts]
    assert atoms2.tobytes() == atoms.tobytes()


def test_malformed_files_are_rejected(omdg_lib, tmp_path):
    path, _ = reference_file(tmp_path)
    data = open(path, "rb").read()
    bad = tmp_path / "bad.bin"
    bad.write_bytes(b"X" + data[1:])  # signature
    with pytest.raises(omdg_lib.OMDGError, match="OMDG_EFILE"):
        omdg_lib.checkpoint_read(str(bad))
    bad.write_bytes(data[:-100])  # truncated atom records
    with pytest.raises(omdg_lib.OMDGError, match="OMDG_EFILE"):
        omdg_lib.checkpoint_read(str(bad))
    with pytest.raises(omdg_lib.OMDGError, match="OMDG_EFILE"):
        omdg_lib.checkpoint_read(str(tmp_path / "missing.bin"))


def test_reference_resumes_from_our_file_exactly(omdg_lib, oracle_lib, tmp_path):
    """The reference's CONTINUE_MODE on a file this codec wrote (new time
    stamp) reaches Step 10 exactly as the reference's own continuation."""
    oc = oracle_lib
    if not os.path.exists(oc.REF_DRIVER):
        pytest.skip("reference build (oracle/_ref) not present")
    import sys

    sys.path.insert(0, os.path.join(GOLD))
    import make_golden

    path, d = reference_file(tmp_path)
    v, stamp, conts, atoms, rv = omdg_lib.checkpoint_read(path)
    ours = str(tmp_path / "ours.bin")
    omdg_lib.checkpoint_write(ours, v, conts, atoms, rv)
    res = oc.run_reference(os.path.join(GOLD, "eam_al_500.dat"), "eam", "aluminum5000", steps=10, dt=0.002,
                           table_dir=make_golden.table_dir(), cont=ours)
    a = res["atoms"]
    np.testing.assert_array_equal(a[:, 2:5], d["x10"])
    np.testing.assert_array_equal(a[:, 5:8], d["v10"])
    np.testing.assert_array_equal(res["ledger"], d["ledger"])
