"""The impact run's Ar-Si interaction and the replica (ensemble) mode.

- The reference's own Ar-Si table (tables/pair.ar-si.zbl, TForcePair between
  projectile and target as in test/si-impact/main.cpp:70-71) with
  Stillinger-Weber Si, against the reference's runs
  (tests/golden/impact_ar_si_slab.npz): an Ar atom 0.6-3.1 A above a Si slab
  (periodic x/y, free z), and an 83 eV Ar collision over 80 steps of 0.5 fs.
  The fixture comes from the reference build whose SW triplets take third
  atoms of the kernel's types only (the reference takes any neighbour there,
  sw.cpp:265-268, which puts the Ar projectile into Si three-body terms).
- The analytic ZBL kernel (omdg_add_zbl: the universal ZBL of sw.cpp:118-146
  with a switch to zero) against the oracle's restatement.
- Replica mode: two slabs of the impact ensemble (Tersoff Si + the Ar-Si
  table) stepped together for 50 steps, each against the oracle stepping that
  slab alone.

Static tolerances as elsewhere: norm-wise relative force error <= 1e-5,
components within 1e-5 max|f| + 1e-6 eV/A, per-atom energies within
2e-6 eV + 1e-6 relative (the Ar atom holds up to 123 eV at 0.6 A).
"""
import os

import numpy as np
import pytest

from conftest import GOLD, TABLES

pytestmark = pytest.mark.gpu

SW_FILE = os.path.join(TABLES, "sw.silicon")
TERSOFF_FILE = os.path.join(TABLES, "tersoff.silicon27")
ARSI = os.path.join(TABLES, "pair.ar-si.zbl")

SW_PARAM = dict(eps=2.1683, A=7.049556277, B=0.6022245584, p=4, q=0, sigma=2.0951, a=1.80, lam=21.0, gamma=1.2,
                icos0=-3.0, usezbl=1, sx0=1.2107, sx1=1.8456, sa0=335.0594, sa1=-492.3905, sa2=244.5280,
                sa3=-41.2347, z1=14, z2=14)
TERSOFF_PARAM = dict(A=3264.7, B=95.373, lambda1=3.2394, lambda2=1.3258, lambda3=1.3258, beta=0.33675, n=22.956,
                     c=4.8381, d=2.0417, h=0.0, R=2.7, D=0.15)


def gold():
    return dict(np.load(os.path.join(GOLD, "impact_ar_si_slab.npz")))


def check(f, fref, e, eref):
    rel = np.linalg.norm(f - fref) / np.linalg.norm(fref)
    assert rel <= 1e-5, rel
    err = np.abs(f - fref).max()
    assert err <= 1e-5 * np.abs(fref).max() + 1e-6, err
    eerr = np.abs(e - eref) / (2e-6 + 1e-6 * np.abs(eref))
    assert eerr.max() <= 1.0, (np.abs(e - eref).max(), int(eerr.argmax()))


def slab_ctx(omdg, x, v, types, lo, hi, si="sw", arsi="table"):
    from objectmd_gb300 import inputs

    ctx = omdg.Context(0)
    ctx.set_box(lo, hi, (True, True, False))
    ctx.set_atoms(x, v, types=types, masses=[inputs.md_mass("silicon"), inputs.md_mass("argon")], znum=[14.0, 18.0])
    if si == "sw":
        ctx.add_sw(SW_FILE, 0, 0)
    else:
        ctx.add_tersoff(TERSOFF_FILE, 0, 0)
    if arsi == "table":
        ctx.add_pair_table(ARSI, ta=1, tb=0)
    else:
        ctx.add_zbl(1, 0, 3.0, 0.5)
    ctx.set_neighbor(0.3, 1)
    return ctx


def test_ar_si_table_static_vs_reference(omdg_lib):
    d = gold()
    for k, h in enumerate(d["heights"]):
        with slab_ctx(omdg_lib, d["static_x0"][k], d["static_v0"], d["types"], d["box_lo"], d["box_hi"]) as ctx:
            ctx.compute_forces()
            st = ctx.get_state()
        check(st["f"], d["static_f"][k], st["pot"], d["static_pot"][k])
        far = np.abs(st["f"][-1] - d["static_f"][k][-1]).max()
        assert far <= 1e-5 * np.abs(d["static_f"][k][-1]).max() + 1e-6, (h, far)


def test_ar_si_table_keeps_the_reference_cut_radius(omdg_lib):
    """The table's knots reach 5.1 A (its CutRadius, tpair.h:59), but it is
    zero from 3.2 A on: the list radius stops where its tail becomes
    negligible, and the full range stays available as a compatibility key."""
    d = gold()
    with slab_ctx(omdg_lib, d["static_x0"][0], d["static_v0"], d["types"], d["box_lo"], d["box_hi"]) as ctx:
        assert abs(ctx.max_cut_radius() - 5.1) < 1e-9
        ctx.compute_forces()
        f_trim = ctx.get_state()["f"]
        n_trim = len(ctx.neighbors()[1])
        ctx.set_compat("pair_table_full_range", 1)
        ctx.compute_forces()
        f_full = ctx.get_state()["f"]
        n_full = len(ctx.neighbors()[1])
    assert n_full > 1.5 * n_trim  # Rv 5.4 A instead of SW's 3.771 + 0.3
    assert np.abs(f_full - f_trim).max() <= 1e-6 * np.abs(f_full).max()


def test_ar_si_collision_trajectory_vs_reference(omdg_lib):
    """83 eV Ar into the slab, 80 steps of 0.5 fs, the reference's first-step
    rule: FP32 forces on FP64 integration against the reference's FP64 run
    (measured on a GB300: positions 6.7e-7 A, velocities 3.3e-5 A/ps, kinetic
    energy 1.1e-7 and potential 1.9e-8 relative)."""
    d = gold()
    with slab_ctx(omdg_lib, d["nve_x0"], d["nve_v0"], d["types"], d["nve_lo"], d["nve_hi"]) as ctx:
        ctx.set_timestep(float(d["dt"]))
        ctx.set_first_step_mode(True)
        ctx.step(int(d["steps"]))
        st = ctx.get_state()
        kin, pot = ctx.ledger_history()
    L = d["nve_hi"] - d["nve_lo"]
    dx = st["x"] - d["nve_x"]
    dx[:, :2] -= np.round(dx[:, :2] / L[:2]) * L[:2]
    dxm, dvm = np.abs(dx).max(), np.abs(st["v"] - d["nve_v"]).max()
    kref, pref = d["nve_ledger"][1:1 + len(kin), 1], d["nve_ledger"][1:1 + len(pot), 2]
    krel = np.abs(kin - kref).max() / np.abs(kref).max()
    prel = np.abs(pot - pref).max() / np.abs(pref).max()
    print("Ar-Si collision, 80 steps: |dx| %.2e A |dv| %.2e A/ps kinetic %.2e potential %.2e" % (dxm, dvm, krel, prel))
    assert dxm < 1e-5, dxm
    assert dvm < 1e-3, dvm
    assert krel < 1e-6, krel
    assert prel < 1e-7, prel


def test_analytic_zbl_vs_oracle(omdg_lib, oracle_lib):
    oc = oracle_lib
    d = gold()
    types = d["types"]
    si = types == 0
    for k in (0, 2, 5, 8):
        x = d["static_x0"][k]
        with slab_ctx(omdg_lib, x, d["static_v0"], types, d["box_lo"], d["box_hi"], arsi="zbl") as ctx:
            ctx.compute_forces()
            st = ctx.get_state()
        box = oc.make_box(d["box_lo"], d["box_hi"], (1, 1, 0))
        fsi, esi, _ = oc.sw(box, x[si], oc.neighbors(box, x[si], 2.0951 * 1.8 + 0.3), oc.SWParam(**SW_PARAM))
        f = np.zeros_like(x)
        e = np.zeros(len(x))
        f[si], e[si] = fsi, esi
        oc.zbl(box, x, types, 1, 0, 18.0, 14.0, 3.0, 0.5, oc.neighbors(box, x, 3.3), f, e)
        check(st["f"], f, st["pot"], e)


def oracle_replica_run(oc, x, v, types, lo, hi, masses, dt, steps):
    """Velocity Verlet (integrator.cpp:225-259, forces kept at the first
    step) of one slab: Tersoff on the Si atoms, the Ar-Si table between Ar
    and Si, periodic x/y wrapped each step."""
    box = oc.make_box(lo, hi, (1, 1, 0))
    phi = oc.Table.from_file(ARSI)
    tp = oc.TersoffParam(**TERSOFF_PARAM)
    m = np.where(types == 0, masses[0], masses[1]).astype(np.float64)
    si = types == 0

    def forces(x):
        f = np.zeros_like(x)
        e = np.zeros(len(x))
        vir = np.zeros(len(x))
        fs, es, _ = oc.tersoff(box, x[si], oc.neighbors(box, x[si], 2.85 + 0.3), tp)
        f[si], e[si] = fs, es
        oc.pair_table_typed(box, x, types, 1, 0, oc.neighbors(box, x, phi.max_range() + 0.3), phi, f, e, vir)
        return f

    x, v = x.copy(), v.copy()
    f = forces(x)
    for _ in range(steps):
        v += 0.5 * dt * f / m[:, None]
        x += dt * v
        x = oc.wrap(box, x)
        f = forces(x)
        v += 0.5 * dt * f / m[:, None]
    return x, v


def test_replica_mode_vs_oracle(omdg_lib, oracle_lib):
    """Two slabs of the impact ensemble in one context (replica mode: one
    atom array, per-replica grids and periodic lengths), Tersoff + the Ar-Si
    table, 50 steps of 0.5 fs; each slab against the oracle stepping it alone."""
    from objectmd_gb300 import inputs

    oc = oracle_lib
    e = inputs.impact_ensemble(nrep=2, nmin=1200, nmax=2500, seed=17, emin=50.0, emax=60.0, height=2.0)
    n = e["natoms"]
    dt, steps = 0.0005, 50
    ctx = omdg_lib.Context(0)
    ctx.set_replicas(n, e["lo"], e["hi"], (1, 1, 0))
    ctx.set_atoms(e["x"], e["v"], types=e["types"], masses=e["masses"], znum=e["znum"])
    ctx.add_tersoff(TERSOFF_FILE, 0, 0)
    ctx.add_pair_table(ARSI, ta=1, tb=0)
    ctx.set_neighbor(0.5, 0)
    ctx.set_timestep(dt)
    ctx.set_first_step_mode(False)
    ctx.step(steps)
    st = ctx.get_state()
    ctx.close()
    off = np.concatenate([[0], np.cumsum(n)])
    for r in range(2):
        sl = slice(off[r], off[r + 1])
        xr, vr = oracle_replica_run(oc, e["x"][sl], e["v"][sl], e["types"][sl], e["lo"][r], e["hi"][r], e["masses"],
                                    dt, steps)
        L = e["hi"][r] - e["lo"][r]
        dx = st["x"][sl] - xr
        dx[:, :2] -= np.round(dx[:, :2] / L[:2]) * L[:2]
        dxm = np.abs(dx).max()
        dvm = np.abs(st["v"][sl] - vr).max()
        # measured on a GB300: |dx| 1.2e-7 A, |dv| 8.8e-6 A/ps
        print("replica %d (%d atoms): |dx| %.2e A |dv| %.2e A/ps" % (r, n[r], dxm, dvm))
        assert dxm < 2e-6, dxm
        assert dvm < 2e-4, dvm
