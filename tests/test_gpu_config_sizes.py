"""Parity at the configured problem sizes, not only on small boxes.

- EAM Al FCC 40^3 = 256,000 atoms (a = 4.05 A, Gaussian 0.05 A, 300 K,
  5000-knot table, skin 0.3 A) against the FP64 oracle: every force and
  per-atom energy, and the full neighbour set (13.7M entries) exactly.
- Si diamond 40^3 = 512,000 atoms (a = 5.431 A, Gaussian 0.03 A, 1000 K)
  for Stillinger-Weber (cutoff 3.771 A) and Tersoff (R = 2.7, D = 0.15 A)
  against the FP64 oracle: every force and energy, the full neighbour sets.
- Lennard-Jones argon FCC 10^3 = 4,000 atoms (a = 5.26 A, 100 K, 2.5 sigma
  table, skin 0.3 A) in FP64, 1000 NVE steps of 1 fs, against the reference's
  own run (tests/golden/lj_ar_4000.npz): final positions, velocities, forces
  and the energy ledger of every step.

Force tolerances are those of the small-box tests: norm-wise relative error
<= 1e-5 and every component within 1e-5 max|f| + 1e-6 eV/A; per-atom energies
within 2e-6 eV (3e-6 for SW, the extreme of 512,000 atoms; 5e-6 for Tersoff,
whose f_R - b f_A cancels).
"""
import os

import numpy as np
import pytest

from conftest import TABLES, load_case

pytestmark = pytest.mark.gpu

EAM_TABLE = os.path.join(TABLES, "eam.aluminum5000")
SW_FILE = os.path.join(TABLES, "sw.silicon")
TERSOFF_FILE = os.path.join(TABLES, "tersoff.silicon27")
LJ = os.path.join(TABLES, "pair.lj.argon")


def check(f, fref, e, eref, etol):
    rel = np.linalg.norm(f - fref) / np.linalg.norm(fref)
    assert rel <= 1e-5, rel
    err = np.abs(f - fref).max()
    assert err <= 1e-5 * np.abs(fref).max() + 1e-6, err
    eerr = np.abs(e - eref).max()
    assert eerr <= etol, eerr


def sorted_tuples(off, j, code, n):
    """Every (i, j, image) entry of a list as one sorted int64 key."""
    i = np.repeat(np.arange(n, dtype=np.int64), np.diff(off))
    return np.sort((i * n + np.asarray(j, dtype=np.int64)) * 27 + np.asarray(code, dtype=np.int64))


def run_static(omdg, x, v, lo, hi, mass, z, add):
    ctx = omdg.Context(0)
    ctx.set_box(lo, hi)
    ctx.set_atoms(x, v, masses=[mass], znum=[z])
    add(ctx)
    ctx.set_neighbor(0.3, 1)
    ctx.compute_forces()
    st = ctx.get_state()
    nb = ctx.neighbors()
    ctx.close()
    return st, nb


def test_eam_al_256k_vs_oracle(omdg_lib, oracle_lib):
    from objectmd_gb300 import inputs

    oc = oracle_lib
    x, v, (lo, hi) = inputs.eam_aluminium(ncell=40, a=4.05, sigma=0.05, temp=300.0, seed_pos=2, seed_vel=3)
    assert len(x) == 256000
    phi, ed, em = (oc.Table.from_file(EAM_TABLE, s) for s in ("PAIR", "EDENS", "EMBED"))
    box = oc.make_box(lo, hi, (1, 1, 1))
    nb = oc.neighbors(box, x, phi.max_range() + 0.3)
    fref, eref, _, _ = oc.eam(box, x, nb, phi, ed, em)
    st, mine = run_static(omdg_lib, x, v, lo, hi, inputs.md_mass("aluminum"), 13.0, lambda c: c.add_eam(EAM_TABLE))
    check(st["f"], fref, st["pot"], eref, 2e-6)
    n = len(x)
    assert np.array_equal(sorted_tuples(*mine, n), sorted_tuples(*nb, n))


SW_PARAM = dict(eps=2.1683, A=7.049556277, B=0.6022245584, p=4, q=0, sigma=2.0951, a=1.80, lam=21.0, gamma=1.2,
                icos0=-3.0, usezbl=1, sx0=1.2107, sx1=1.8456, sa0=335.0594, sa1=-492.3905, sa2=244.5280,
                sa3=-41.2347, z1=14, z2=14)
TERSOFF_PARAM = dict(A=3264.7, B=95.373, lambda1=3.2394, lambda2=1.3258, lambda3=1.3258, beta=0.33675, n=22.956,
                     c=4.8381, d=2.0417, h=0.0, R=2.7, D=0.15)


@pytest.mark.parametrize("kind", ["sw", "tersoff"])
def test_si_512k_vs_oracle(omdg_lib, oracle_lib, kind):
    from objectmd_gb300 import inputs

    oc = oracle_lib
    x, v, (lo, hi) = inputs.diamond_silicon(ncell=40, a=5.431, sigma=0.03, temp=1000.0, seed_pos=4, seed_vel=5)
    assert len(x) == 512000
    box = oc.make_box(lo, hi, (1, 1, 1))
    if kind == "sw":
        nb = oc.neighbors(box, x, 2.0951 * 1.8 + 0.3)
        fref, eref, _ = oc.sw(box, x, nb, oc.SWParam(**SW_PARAM))
        # the largest of 512,000 FP32 per-atom sums (measured 2.09e-6 eV on a
        # GB300; 1.5e-6 on 4,096 atoms)
        add, etol = (lambda c: c.add_sw(SW_FILE)), 3e-6
    else:
        nb = oc.neighbors(box, x, 2.85 + 0.3)
        fref, eref, _ = oc.tersoff(box, x, nb, oc.TersoffParam(**TERSOFF_PARAM))
        add, etol = (lambda c: c.add_tersoff(TERSOFF_FILE)), 5e-6
    st, mine = run_static(omdg_lib, x, v, lo, hi, inputs.md_mass("silicon"), 14.0, add)
    check(st["f"], fref, st["pot"], eref, etol)
    n = len(x)
    assert np.array_equal(sorted_tuples(*mine, n), sorted_tuples(*nb, n))


def test_lj_ar_4000_fp64_1000_steps_vs_reference(omdg_lib):
    """FP64 end to end, the reference's first-step rule, list rebuilt every
    step (the reference's default refresh), 1000 steps of 1 fs.  Both runs are
    FP64; the pair kernel keeps the reference's per-pair arithmetic, so the
    trajectories stay together to rounding (measured on a GB300: positions
    4e-14 A, velocities 5e-13 A/ps, forces 3e-14 eV/A, energies 7e-15
    relative after 1000 steps).  The bounds leave room for the chaotic growth
    of a summation-order difference."""
    from objectmd_gb300 import inputs

    d = load_case("lj_ar_4000")
    ctx = omdg_lib.Context(0)
    ctx.set_box(d["box_lo"], d["box_hi"])
    ctx.set_atoms(d["x0"], d["v0"], masses=[inputs.md_mass("argon")], znum=[18.0])
    ctx.add_pair_table(LJ, fp64=True)
    ctx.set_neighbor(0.3, 1)
    ctx.set_timestep(float(d["dt"]))
    ctx.set_first_step_mode(True)
    ctx.step(int(d["steps"]))
    st = ctx.get_state()
    kin, pot = ctx.ledger_history()
    ctx.close()
    L = d["box_hi"] - d["box_lo"]
    dx = st["x"] - d["x"]
    dx -= np.round(dx / L) * L
    dxm = np.abs(dx).max()
    dvm = np.abs(st["v"] - d["v"]).max()
    dfm = np.abs(st["f"] - d["f"]).max()
    kref, pref = d["ledger"][1:1 + len(kin), 1], d["ledger"][1:1 + len(pot), 2]
    krel = np.abs(kin - kref).max() / np.abs(kref).max()
    prel = np.abs(pot - pref).max() / np.abs(pref).max()
    print("LJ 4000 x 1000 steps: |dx| %.2e A |dv| %.2e A/ps |df| %.2e eV/A kinetic %.2e potential %.2e" %
          (dxm, dvm, dfm, krel, prel))
    assert dxm < 1e-10, dxm
    assert dvm < 1e-9, dvm
    assert dfm < 1e-10, dfm
    assert krel < 1e-12, krel
    assert prel < 1e-12, prel
