"""Tabulated pair potential (TForcePair) and the Berendsen thermostat on the GPU,
against the reference's own outputs (tests/golden).

FP64 mode (the plain-FP64 Lennard-Jones configuration): forces within 1e-10
eV/A and the trajectory within 1e-9 A of the reference.  FP32 mode: the
norm-wise relative force error <= 1e-5.
"""
import os

import numpy as np
import pytest

from conftest import TABLES, load_case, nbr_set

pytestmark = pytest.mark.gpu

LJ = os.path.join(TABLES, "pair.lj.argon")


def lj_context(omdg, d, fp64, rebuild_every=1):
    from objectmd_gb300 import inputs

    ctx = omdg.Context(0)
    ctx.set_box(d["box_lo"], d["box_hi"])
    ctx.set_atoms(d["x0"], d["v0"], masses=[inputs.md_mass("argon")], znum=[18.0])
    ctx.add_pair_table(LJ, fp64=fp64)
    ctx.set_neighbor(0.3, rebuild_every)
    return ctx


@pytest.mark.parametrize("fp64", [True, False])
def test_lj_static_matches_reference(omdg_lib, fp64):
    d = load_case("lj_ar_500")
    with lj_context(omdg_lib, d, fp64) as ctx:
        ctx.compute_forces()
        st = ctx.get_state()
        mine = nbr_set(*ctx.neighbors())
    if fp64:
        assert np.abs(st["f"] - d["f"]).max() < 1e-10
        assert np.abs(st["pot"] - d["pot"]).max() < 1e-12
    else:
        rel = np.linalg.norm(st["f"] - d["f"]) / np.linalg.norm(d["f"])
        assert rel <= 1e-5, rel
    assert mine == set(map(tuple, d["nbr"].tolist()))


def test_lj_fp64_nve_trajectory_matches_reference(omdg_lib):
    """50 steps, dt 1 fs, FP64 end to end (plain LJ configuration)."""
    d = load_case("lj_ar_nve")
    with lj_context(omdg_lib, d, True) as ctx:
        ctx.set_timestep(float(d["dt"]))
        ctx.step(int(d["steps"]))
        st = ctx.get_state()
        kin, pot = ctx.ledger_history()
    L = d["box_hi"] - d["box_lo"]
    dx = st["x"] - d["x"]
    dx -= np.round(dx / L) * L
    assert np.abs(dx).max() < 1e-9
    np.testing.assert_allclose(kin, d["ledger"][1:1 + len(kin), 1], rtol=1e-9)
    np.testing.assert_allclose(pot, d["ledger"][1:1 + len(pot), 2], rtol=1e-9)


def run_thermostat(omdg_lib, d, count_ghosts):
    from objectmd_gb300 import inputs

    ctx = omdg_lib.Context(0)
    ctx.set_box(d["box_lo"], d["box_hi"])
    ctx.set_atoms(d["x0"], d["v0"], masses=[inputs.md_mass("aluminum")], znum=[13.0])
    ctx.add_eam(os.path.join(TABLES, "eam.aluminum5000"))
    ctx.set_neighbor(0.3, 1)
    ctx.set_timestep(float(d["dt"]))
    ctx.set_thermostat(float(d["tcontrol"][0]), float(d["tcontrol"][1]))
    ctx.set_compat("thermostat_counts_ghosts", count_ghosts)
    ctx.step(int(d["steps"]))
    kin, pot = ctx.ledger_history()
    st = ctx.get_state()
    ctx.close()
    return kin, st


def test_berendsen_thermostat_matches_reference(omdg_lib):
    """TempController(300 K, 0.05 ps) on EAM Al starting at 600 K, 20 steps, with
    the reference's temperature divisor (owners plus ghost images)."""
    d = load_case("eam_al_tc")
    kin, st = run_thermostat(omdg_lib, d, True)
    np.testing.assert_allclose(kin, d["ledger"][1:1 + len(kin), 1], rtol=1e-6)
    assert np.abs(st["v"] - d["v"]).max() < 1e-4 * np.abs(d["v"]).max()


def test_berendsen_thermostat_default_counts_owners(omdg_lib, oracle_lib):
    """Default divisor: the box's own atoms; against an FP64 oracle replay."""
    from conftest import TABLES as T
    from objectmd_gb300 import inputs

    oc = oracle_lib
    d = load_case("eam_al_tc")
    kin, st = run_thermostat(omdg_lib, d, False)
    tab = os.path.join(T, "eam.aluminum5000")
    phi, ed, em = (oc.Table.from_file(tab, s) for s in ("PAIR", "EDENS", "EMBED"))
    box = oc.make_box(d["box_lo"], d["box_hi"], (1, 1, 1))
    x = oc.wrap(box, d["x0"])
    v = d["v0"].copy()
    n = len(x)
    mass = np.full(n, inputs.md_mass("aluminum"))
    f = np.zeros((n, 3))
    dt, (tset, tau) = float(d["dt"]), d["tcontrol"]
    ref = []
    for step in range(int(d["steps"])):
        oc.vv_kick_drift(x, v, f, mass, dt)
        x = oc.wrap(box, x)
        f = oc.eam(box, x, oc.neighbors(box, x, phi.max_range() + 0.3), phi, ed, em)[0]
        oc.vv_kick(v, f, mass, dt)
        k = oc.kinetic(v, mass)
        ref.append(k)
        if step:
            v *= oc.berendsen_factor(dt, tau, tset, (2.0 / 3.0) / 8.61734279e-05 * k / n)
    np.testing.assert_allclose(kin, ref, rtol=1e-6)
