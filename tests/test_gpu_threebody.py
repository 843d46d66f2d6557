"""Stillinger-Weber and Tersoff on the GPU.

SW is checked against the reference's own SW with every triplet evaluated
(the sw.cpp:261 guard removed, tests/golden), Tersoff against the FP64 C
oracle (the reference's tersoff.h does not compile).  Tolerance as for EAM:
norm-wise relative force error <= 1e-5, components within
1e-5 * max|f| + 1e-6 eV/A, per-atom energies within 2e-6 eV.
"""
import os

import numpy as np
import pytest

from conftest import TABLES, load_case, nbr_set

pytestmark = pytest.mark.gpu

SW_FILE = os.path.join(TABLES, "sw.silicon")
TERSOFF_FILE = os.path.join(TABLES, "tersoff.silicon27")


def check(f, fref, e=None, eref=None, etol=2e-6):
    rel = np.linalg.norm(f - fref) / np.linalg.norm(fref)
    assert rel <= 1e-5, rel
    assert np.abs(f - fref).max() <= 1e-5 * np.abs(fref).max() + 1e-6
    if e is not None:
        err = np.abs(e - eref)
        assert err.max() <= etol, (err.max(), int(err.argmax()), float(eref[err.argmax()]))


def si_context(omdg, x, v, lo, hi, kind):
    from objectmd_gb300 import inputs

    ctx = omdg.Context(0)
    ctx.set_box(lo, hi)
    ctx.set_atoms(x, v, masses=[inputs.md_mass("silicon")], znum=[14.0])
    if kind == "sw":
        ctx.add_sw(SW_FILE)
    else:
        ctx.add_tersoff(TERSOFF_FILE)
    ctx.set_neighbor(0.3, 1)
    return ctx


@pytest.mark.parametrize("case", ["sw_si_216", "sw_si_1000"])
def test_sw_matches_reference_every_triplet(omdg_lib, case):
    d = load_case(case)
    with si_context(omdg_lib, d["x0"], d["v0"], d["box_lo"], d["box_hi"], "sw") as ctx:
        ctx.compute_forces()
        st = ctx.get_state()
        mine = nbr_set(*ctx.neighbors())
    check(st["f"], d["f"], st["pot"], d["pot"])
    assert mine == set(map(tuple, d["nbr"].tolist()))


def test_sw_large_vs_oracle(omdg_lib, oracle_lib):
    from objectmd_gb300 import inputs

    oc = oracle_lib
    x, v, (lo, hi) = inputs.diamond_silicon(ncell=8, a=5.431, sigma=0.03, temp=1000.0, seed_pos=41, seed_vel=42)
    box = oc.make_box(lo, hi, (1, 1, 1))
    p = oc.SWParam(eps=2.1683, A=7.049556277, B=0.6022245584, p=4, q=0, sigma=2.0951, a=1.80, lam=21.0, gamma=1.2,
                   icos0=-3.0, usezbl=1, sx0=1.2107, sx1=1.8456, sa0=335.0594, sa1=-492.3905, sa2=244.5280,
                   sa3=-41.2347, z1=14, z2=14)
    fref, eref, _ = oc.sw(box, x, oc.neighbors(box, x, 2.0951 * 1.8 + 0.3), p)
    with si_context(omdg_lib, x, v, lo, hi, "sw") as ctx:
        ctx.compute_forces()
        st = ctx.get_state()
    check(st["f"], fref, st["pot"], eref)


@pytest.mark.parametrize("ncell,sigma,temp", [(3, 0.06, 1000.0), (8, 0.03, 1000.0)])
def test_tersoff_vs_oracle(omdg_lib, oracle_lib, ncell, sigma, temp):
    from objectmd_gb300 import inputs

    oc = oracle_lib
    x, v, (lo, hi) = inputs.diamond_silicon(ncell=ncell, a=5.431, sigma=sigma, temp=temp, seed_pos=8, seed_vel=9)
    box = oc.make_box(lo, hi, (1, 1, 1))
    p = oc.TersoffParam(A=3264.7, B=95.373, lambda1=3.2394, lambda2=1.3258, lambda3=1.3258, beta=0.33675, n=22.956,
                        c=4.8381, d=2.0417, h=0.0, R=2.7, D=0.15)
    nb = oc.neighbors(box, x, 2.85 + 0.3)
    fref, eref, _ = oc.tersoff(box, x, nb, p)
    with si_context(omdg_lib, x, v, lo, hi, "tersoff") as ctx:
        ctx.compute_forces()
        st = ctx.get_state()
        assert nbr_set(*ctx.neighbors()) == nbr_set(*nb)
    # bond energies cancel (f_R - b f_A): FP32 exp/pow leave ~1e-6 relative per atom
    check(st["f"], fref, st["pot"], eref, etol=5e-6)


def interstitial_silicon(ncell, seed):
    """Diamond Si with three atoms planted on tetrahedral interstitial sites
    ((1/2, 1/2, 1/2) of a cubic cell, relative to its first site): each has 4 neighbours at sqrt(3)/4 a
    and 6 at a/2, inside both cutoffs, and its 4 nearest hosts gain a fifth."""
    from objectmd_gb300 import inputs

    a = 5.431
    x, v, (lo, hi) = inputs.diamond_silicon(ncell=ncell, a=a, sigma=0.03, temp=1000.0, seed_pos=seed,
                                            seed_vel=seed + 1)
    cells = np.array([[1, 1, 1], [ncell // 2, 2, ncell - 2], [ncell - 2, ncell // 2, 3]], dtype=np.float64)
    extra = np.array(lo)[None, :] + (cells + 0.5) * a + a / 8  # lattice sites are offset by a/8
    rng = np.random.default_rng(seed + 2)
    x = np.vstack([x, extra + rng.normal(0.0, 0.03, extra.shape)])
    v = np.vstack([v, np.zeros_like(extra)])
    return x, v, lo, hi


@pytest.mark.parametrize("kind", ["sw", "tersoff"])
def test_dense_centres_take_the_wide_kernel(omdg_lib, oracle_lib, kind):
    """Centres with more in-cutoff neighbours than the register path holds go
    to k_sw_wide / k_tersoff_wide; their forces must still match the oracle,
    and the queue count shows that the dense pass ran."""
    oc = oracle_lib
    x, v, lo, hi = interstitial_silicon(6, 61)
    box = oc.make_box(lo, hi, (1, 1, 1))
    if kind == "sw":
        p = oc.SWParam(eps=2.1683, A=7.049556277, B=0.6022245584, p=4, q=0, sigma=2.0951, a=1.80, lam=21.0,
                       gamma=1.2, icos0=-3.0, usezbl=1, sx0=1.2107, sx1=1.8456, sa0=335.0594, sa1=-492.3905,
                       sa2=244.5280, sa3=-41.2347, z1=14, z2=14)
        fref, eref, _ = oc.sw(box, x, oc.neighbors(box, x, 2.0951 * 1.8 + 0.3), p)
        # an interstitial's energy sums ~45 three-body terms of up to ~10 eV in
        # FP32 (measured on a GB300: 5.8e-6 eV); lattice atoms stay below 3e-7
        etol = 2e-5
    else:
        p = oc.TersoffParam(A=3264.7, B=95.373, lambda1=3.2394, lambda2=1.3258, lambda3=1.3258, beta=0.33675,
                            n=22.956, c=4.8381, d=2.0417, h=0.0, R=2.7, D=0.15)
        fref, eref, _ = oc.tersoff(box, x, oc.neighbors(box, x, 2.85 + 0.3), p)
        etol = 5e-6
    with si_context(omdg_lib, x, v, lo, hi, kind) as ctx:
        ctx.compute_forces()
        st = ctx.get_state()
        wide = ctx.wide_centres()
    assert wide >= 3, wide
    check(st["f"], fref, st["pot"], eref, etol=etol)


def test_tersoff_nve_conserves_energy(omdg_lib):
    from objectmd_gb300 import inputs

    x, v, (lo, hi) = inputs.diamond_silicon(ncell=4, a=5.431, sigma=0.03, temp=1000.0, seed_pos=4, seed_vel=5)
    with si_context(omdg_lib, x, v, lo, hi, "tersoff") as ctx:
        ctx.set_neighbor(0.3, 0)
        ctx.set_timestep(0.001)
        ctx.set_first_step_mode(False)
        ctx.step(1)
        e0 = ctx.ledger()["energy"]
        ctx.step(500)
        e1 = ctx.ledger()["energy"]
    assert abs(e1 - e0) / len(x) < 2e-4  # eV/atom over 0.5 ps at 1000 K


@pytest.mark.parametrize("kind,bound", [("sw", 3e-4), ("tersoff", 3e-4)])
def test_nve_drift_over_10k_steps(omdg_lib, kind, bound):
    """10^4 NVE steps of 4096 Si atoms at 1000 K, dt 1 fs, displacement-triggered
    rebuilds: the run stays finite (SW pairs at r == rc in FP32 would give
    0 * inf) and the energy drift stays below `bound` eV/atom (measured on a
    GB300: SW 7.5e-5, Tersoff 6.4e-5)."""
    from objectmd_gb300 import inputs

    x, v, (lo, hi) = inputs.diamond_silicon(ncell=8, a=5.431, sigma=0.03, temp=1000.0, seed_pos=4, seed_vel=5)
    with si_context(omdg_lib, x, v, lo, hi, kind) as ctx:
        ctx.set_neighbor(0.3, 0)
        ctx.set_timestep(0.001)
        ctx.set_first_step_mode(False)
        ctx.step(1)
        e0 = ctx.ledger()["energy"]
        ctx.step(10000)
        e1 = ctx.ledger()["energy"]
    assert np.isfinite(e1)
    assert abs(e1 - e0) / len(x) < bound
