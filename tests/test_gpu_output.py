"""The output path against the reference's own files
(tests/golden/output_eam_al_500.npz, EAM Al 500, 6 steps of 2 fs):

- DumpAtoms of a state loaded from the reference's checkpoint (positions,
  velocities, id, nid: FP64 values taken over exactly) equals the reference's
  DumpAtoms of that state line for line; the reference writes its storage
  order, so lines are compared as a set.
- DumpAtoms (velocity, force, potential, id, nid) and SysMonitor's md.out
  after 6 steps run here: the same header and number formats; values within
  the EAM NVE tolerances (positions 1e-5 A, the 5-decimal print; velocities
  1e-4 of their scale; forces 1e-4 eV/A; energies 1e-6 relative).
"""
import os
import re

import numpy as np
import pytest

from conftest import GOLD, TABLES, load_case

pytestmark = pytest.mark.gpu

EAM_TABLE = os.path.join(TABLES, "eam.aluminum5000")
INFO = ["$ PeriodicBoundary 7"]  # the Import header line the reference keeps


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(GOLD, "output_eam_al_500.npz"))


def text(a):
    return a.tobytes().decode()


def split(doc):
    lines = doc.splitlines()
    head = [l for l in lines if l.startswith("#")]
    body = [l for l in lines if not l.startswith("#")]
    return head, body


def test_dump_of_a_loaded_state_equals_the_reference(omdg_lib, golden, tmp_path):
    ck = tmp_path / "final.bin"
    ck.write_bytes(golden["checkpoint"].tobytes())
    out = str(tmp_path / "dump.dat")
    with omdg_lib.Context(0) as ctx:
        ctx.load_simulation(str(ck))
        ctx.dump_atoms(out, ("velocity", "tid", "nid"), posprec=5, valprec=5, material="aluminum", info=INFO)
    mine = open(out).read()
    ref = text(golden["dump_state"])
    h1, b1 = split(mine)
    h2, b2 = split(ref)
    assert h1 == h2
    assert sorted(b1) == sorted(b2)


def fields(line):
    return [float(t) for t in line.split()]


def test_dump_and_monitor_after_steps(omdg_lib, golden, tmp_path):
    from objectmd_gb300 import inputs

    d = load_case("eam_al_500")
    dump, md = str(tmp_path / "dump.dat"), str(tmp_path / "md.out")
    with omdg_lib.Context(0) as ctx:
        ctx.set_box(d["box_lo"], d["box_hi"], (True, True, True))
        ctx.set_atoms(d["x0"], d["v0"], masses=[inputs.md_mass("aluminum")], znum=[13.0])
        ctx.add_eam(EAM_TABLE)
        ctx.set_neighbor(0.3, 1)
        ctx.set_timestep(float(golden["dt"]))
        ctx.step(int(golden["steps"]))
        ctx.monitor_append(md, every=2, header=True)
        ctx.dump_atoms(dump, ("velocity", "force", "potential", "tid", "nid"), material="aluminum", info=INFO)
    h1, b1 = split(open(dump).read())
    h2, b2 = split(text(golden["dump_full"]))
    assert h1 == h2
    # the reference's number formats: x y z fixed with 5 decimals, then
    # scientific with 5 (velocity, force, potential), then the integer ids
    fixed, sci, integer = re.compile(r"^-?\d+\.\d{5}$"), re.compile(r"^-?\d\.\d{5}e[+-]\d{2}$"), re.compile(r"^\d+$")
    pattern = [fixed] * 3 + [sci] * 7 + [integer] * 2
    assert len(b1) == len(b2)
    ref = {int(fields(l)[-1]): l for l in b2}
    for l in b1:
        nid = int(fields(l)[-1])
        r = ref[nid]
        for tok, rtok, pat in zip(l.split(), r.split(), pattern):
            assert pat.match(tok) and pat.match(rtok), (tok, rtok)
        assert len(l.split()) == len(r.split()) == len(pattern)
        a, b = np.array(fields(l)), np.array(fields(r))
        assert np.abs(a[0:3] - b[0:3]).max() <= 1.1e-5
        assert np.abs(a[3:6] - b[3:6]).max() <= 1e-4 * max(1.0, np.abs(b[3:6]).max())
        assert np.abs(a[6:9] - b[6:9]).max() <= 1e-4
        assert abs(a[9] - b[9]) <= 1e-5 * abs(b[9]) + 5e-5  # pot printed with 6 significant digits
        assert a[10:] .tolist() == b[10:].tolist()
    m1 = open(md).read().splitlines()
    m2 = text(golden["monitor"]).splitlines()
    assert m1[0] == m2[0] and len(m1) == len(m2)
    energy = re.compile(r"^-?\d\.\d{10}E[+-]\d{2}$")
    for l1, l2 in zip(m1[1:], m2[1:]):
        t1, t2 = l1.split(), l2.split()
        assert t1[:3] == t2[:3]  # Step, ElapsedTime, TimeStep: the same strings
        assert all(energy.match(t) for t in t1[3:] + t2[3:])
        ek, ep, e = (float(t) for t in t1[3:])
        rek, rep, re_ = (float(t) for t in t2[3:])
        assert abs(ek - rek) <= 1e-6 * abs(rek)
        # Ep = P - P0 and E differ by the potential's 5e-8 relative tolerance (|P| ~ 1670 eV)
        assert abs(ep - rep) <= 2e-4 and abs(e - re_) <= 2e-4


def test_thermo_dump_of_a_loaded_state(omdg_lib, tmp_path):
    """ThermoDetector's data file (tests/golden/thermo_eam_al_2048.npz: the
    reference's intensive detector on periodic EAM Al 2048 after 6 steps,
    with the checkpoint of that state): loaded here, forces evaluated, the
    same file.  Headers equal line for line except the pressure value (it
    carries the FP32 per-atom virials: 1e-5 relative).  Per atom, keyed by
    the printed position: the density as printed for every atom; the
    temperature as printed and the local pressure within 1e-5 relative +
    1e-4 GPa for the atoms farther than two detector cutoffs from every
    periodic face.  (Nearer a face the reference sums neighbours' kinetic
    energies about the centre-of-mass velocities of their ghost copies,
    taken over the ghosts' neighbours inside the ghost shell only; here an
    image neighbour uses its owner's full neighbourhood.  An FP64
    restatement of this detector agrees with the reference to 5e-16 there.)"""
    g = np.load(os.path.join(GOLD, "thermo_eam_al_2048.npz"))
    ck = tmp_path / "final.bin"
    ck.write_bytes(g["checkpoint"].tobytes())
    out = str(tmp_path / "thermo.001")
    ercut = 5.558  # the EAM cutoff: the detector's default
    with omdg_lib.Context(0) as ctx:
        ctx.load_simulation(str(ck))
        ctx.add_eam(EAM_TABLE)
        ctx.set_neighbor(0.3, 1)
        ctx.set_thermo_detector(True)
        ctx.compute_forces()
        summ = ctx.dump_thermo(out, mode=0, material="aluminum", info=INFO)
    h1, b1 = split(open(out).read())
    h2, b2 = split(text(g["thermo_dump"]))
    assert len(h1) == len(h2) and len(b1) == len(b2)
    for l1, l2 in zip(h1, h2):
        if l1.startswith("#$ Pressure"):
            p1, p2 = float(l1.split()[2]), float(l2.split()[2])
            assert abs(p1 - p2) <= 1e-5 * abs(p2) + 1e-5, (l1, l2)
            assert abs(summ["pressure"] - p2) <= 1e-5 * abs(p2) + 1e-5
        else:
            assert l1 == l2
    t_sys = float([l for l in h2 if l.startswith("#$ Temperature")][0].split()[2])
    assert abs(summ["temperature"] - t_sys) <= 1e-5 * t_sys
    box = [float(t) for t in [l for l in h2 if l.startswith("#$ Box")][0].split()[2:]]
    lo, hi = np.array(box[:3]), np.array(box[3:])
    ref = {tuple(l.split()[:3]): fields(l) for l in b2}
    deep = 0
    for l in b1:
        key = tuple(l.split()[:3])
        assert key in ref, key
        x, (t, p, n) = np.array(fields(l)[:3]), fields(l)[3:]
        rt, rp, rn = ref[key][3:]
        # printed with 6 significant digits: equal, or one unit of the last
        # digit apart where an FP64 value sits on a rounding boundary
        assert abs(n - rn) <= 1.01e-5 * abs(rn)
        if ((x - lo) > 2 * ercut).all() and ((hi - x) > 2 * ercut).all():
            deep += 1
            assert abs(t - rt) <= 1.01e-5 * abs(rt), (key, t, rt)
            assert abs(p - rp) <= 1e-5 * abs(rp) + 1e-4, (key, p, rp)
    assert deep >= 50
    assert summ["avg_temperature"] > 0 and summ["avg_density"] > 0


def test_monitor_with_thermo_detector_slots(omdg_lib, tmp_path):
    """SysMonitor with a ThermoDetector registered (tests/golden/
    thermo_eam_al_2048.npz: the reference's md.out on a free EAM Al cluster
    of 864 atoms, 6 steps of 2 fs, every 2): the same label line with
    temp: avtemp: pres: avpres:, those four printed as %0.3E and within 2e-3
    relative + 2e-3 (GPa) of the reference's: system temperature about the
    centre-of-mass velocity, average local temperature, system pressure over
    the atoms' bounding box and average local pressure (FP32 virials)."""
    from objectmd_gb300 import inputs

    g = np.load(os.path.join(GOLD, "thermo_eam_al_2048.npz"))
    md = str(tmp_path / "md.out")
    with omdg_lib.Context(0) as ctx:
        ctx.set_box(g["cluster_lo"], g["cluster_hi"], (False, False, False))
        ctx.set_atoms(g["cluster_x"], g["cluster_v"], masses=[inputs.md_mass("aluminum")], znum=[13.0])
        ctx.add_eam(EAM_TABLE)
        ctx.set_neighbor(0.3, 1)
        ctx.set_timestep(0.002)
        ctx.set_thermo_detector(True)
        ctx.step(6)
        ctx.monitor_append(md, every=2, header=True)
    m1 = open(md).read().splitlines()
    m2 = text(g["monitor"]).splitlines()
    assert m1[0] == m2[0] and len(m1) == len(m2)
    slot = re.compile(r"^-?\d\.\d{3}E[+-]\d{2}$")
    for l1, l2 in zip(m1[1:], m2[1:]):
        t1, t2 = l1.split(), l2.split()
        assert len(t1) == len(t2) == 10
        assert t1[:3] == t2[:3]
        assert all(slot.match(t) for t in t1[6:])
        for a, b in zip(t1[6:], t2[6:]):
            assert abs(float(a) - float(b)) <= 2e-3 * abs(float(b)) + 2e-3, (l1, l2)
