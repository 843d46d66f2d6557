"""The CPU oracle against the reference's own outputs (tests/golden, made by
tests/golden/make_golden.py from the reference's code).  No GPU needed."""
import os

import numpy as np
import pytest

from conftest import GOLD, TABLES, load_case, nbr_set

EAM_TABLE = os.path.join(TABLES, "eam.aluminum5000")


def eam_tables(oc):
    return tuple(oc.Table.from_file(EAM_TABLE, s) for s in ("PAIR", "EDENS", "EMBED"))


@pytest.mark.parametrize("sec", ["PAIR", "EMBED"])
def test_table_reader_matches_reference(oracle_lib, sec):
    """treader.cpp:37-64 + :193-229 restated, against the reference TableReader itself."""
    g = np.load(os.path.join(GOLD, "table_%s.npz" % sec.lower()))
    t = oracle_lib.Table.from_file(EAM_TABLE, sec)
    got = np.array([t.read(r) for r in g["r"]])
    np.testing.assert_array_equal(got[:, 0], g["val"])
    np.testing.assert_array_equal(got[:, 1], g["dval"])


def test_table_out_of_range_is_an_error(oracle_lib):
    t = oracle_lib.Table.from_file(EAM_TABLE, "PAIR")
    with pytest.raises(ValueError):
        t.read(t.max_range() + 2.5 * t.spec["dr"])


@pytest.mark.parametrize("case", ["eam_al_500", "eam_al_4000"])
def test_eam_oracle_matches_reference(oracle_lib, case):
    oc = oracle_lib
    d = load_case(case)
    phi, ed, em = eam_tables(oc)
    box = oc.make_box(d["box_lo"], d["box_hi"], (1, 1, 1))
    x = oc.wrap(box, d["x0"])
    nb = oc.neighbors(box, x, phi.max_range() + 0.3)
    f, e, vir, rho = oc.eam(box, x, nb, phi, ed, em)
    assert np.abs(f - d["f"]).max() < 1e-12
    assert np.abs(e - d["pot"]).max() < 1e-12
    assert np.abs(vir - d["vir"]).max() < 1e-10
    assert nbr_set(*nb) == set(map(tuple, d["nbr"].tolist()))


def test_pair_oracle_matches_reference(oracle_lib):
    oc = oracle_lib
    d = load_case("lj_ar_500")
    phi = oc.Table.from_file(os.path.join(TABLES, "pair.lj.argon"), "")
    box = oc.make_box(d["box_lo"], d["box_hi"], (1, 1, 1))
    x = oc.wrap(box, d["x0"])
    nb = oc.neighbors(box, x, phi.max_range() + 0.3)
    f, e, vir = oc.pair_table(box, x, nb, phi)
    assert np.abs(f - d["f"]).max() < 1e-14
    assert np.abs(e - d["pot"]).max() < 1e-14
    assert nbr_set(*nb) == set(map(tuple, d["nbr"].tolist()))


def sw_params(oc):
    return oc.SWParam(eps=2.1683, A=7.049556277, B=0.6022245584, p=4, q=0, sigma=2.0951, a=1.80, lam=21.0,
                      gamma=1.2, icos0=-3.0, usezbl=1, sx0=1.2107, sx1=1.8456, sa0=335.0594, sa1=-492.3905,
                      sa2=244.5280, sa3=-41.2347, z1=14, z2=14)


@pytest.mark.parametrize("case", ["sw_si_216", "sw_si_1000"])
def test_sw_oracle_matches_fixed_reference(oracle_lib, case):
    """Every triplet evaluated: equal to the reference built without the sw.cpp:261 guard."""
    oc = oracle_lib
    d = load_case(case)
    box = oc.make_box(d["box_lo"], d["box_hi"], (1, 1, 1))
    x = oc.wrap(box, d["x0"])
    nb = oc.neighbors(box, x, 2.0951 * 1.8 + 0.3)
    f, e, vir = oc.sw(box, x, nb, sw_params(oc))
    assert np.abs(f - d["f"]).max() < 1e-11
    assert np.abs(e - d["pot"]).max() < 1e-12
    assert nbr_set(*nb) == set(map(tuple, d["nbr"].tolist()))


@pytest.mark.parametrize("case", ["sw_si_dimer", "sw_si_trimer", "sw_si_tetra", "sw_si_1x1x1"])
def test_sw_oracle_matches_reference_on_its_own_clusters(oracle_lib, case):
    """The reference's own silicon test clusters (test/check-verlet-list),
    free boundaries: forces, per-atom energies and the full neighbour tuples
    equal the reference built with every triplet evaluated."""
    oc = oracle_lib
    d = load_case(case)
    box = oc.make_box(d["box_lo"], d["box_hi"], (0, 0, 0))
    x = d["x0"]
    nb = oc.neighbors(box, x, 2.0951 * 1.8 + 0.3)
    f, e, vir = oc.sw(box, x, nb, sw_params(oc))
    assert np.abs(f - d["f"]).max() < 1e-11
    assert np.abs(e - d["pot"]).max() < 1e-12
    assert nbr_set(*nb) == set(map(tuple, d["nbr"].tolist()))


def test_sw_reference_guard_drops_triplets(oracle_lib):
    """The unmodified reference (sw.cpp:261) differs from the full triplet sum,
    already on its own three-atom test cluster."""
    d = load_case("sw_si_216")
    assert np.abs(d["f_asis"] - d["f"]).max() > 1e-3
    d = load_case("sw_si_trimer")
    assert np.abs(d["f_asis"] - d["f"]).max() > 1.0


def test_sw_forces_are_energy_gradients(oracle_lib):
    """Finite-difference check of the oracle's SW (away from the ZBL/spline core)."""
    oc = oracle_lib
    d = load_case("sw_si_216")
    box = oc.make_box(d["box_lo"], d["box_hi"], (1, 1, 1))
    x = oc.wrap(box, d["x0"])
    rv = 2.0951 * 1.8 + 0.3
    p = sw_params(oc)
    f, e, _ = oc.sw(box, x, oc.neighbors(box, x, rv), p)
    h = 1e-5
    for atom in (0, 17, 101):
        for q in range(3):
            xp = x.copy()
            xp[atom, q] += h
            xm = x.copy()
            xm[atom, q] -= h
            ep = oc.sw(box, xp, oc.neighbors(box, xp, rv), p)[1].sum()
            em = oc.sw(box, xm, oc.neighbors(box, xm, rv), p)[1].sum()
            assert abs(-(ep - em) / (2 * h) - f[atom, q]) < 2e-6


def test_tersoff_forces_are_energy_gradients(oracle_lib):
    """Tersoff has no running reference (tersoff.h does not compile); its oracle is
    pinned by energy-force consistency and the diamond cohesive energy."""
    oc = oracle_lib
    from objectmd_gb300 import inputs

    p = oc.TersoffParam(A=3264.7, B=95.373, lambda1=3.2394, lambda2=1.3258, lambda3=1.3258, beta=0.33675, n=22.956,
                        c=4.8381, d=2.0417, h=0.0, R=2.7, D=0.15)
    x, v, (lo, hi) = inputs.diamond_silicon(ncell=3, a=5.431, sigma=0.06, temp=1000.0, seed_pos=8, seed_vel=9)
    box = oc.make_box(lo, hi, (1, 1, 1))
    rv = 2.85 + 0.3
    f, e, _ = oc.tersoff(box, x, oc.neighbors(box, x, rv), p)
    h = 1e-5
    for atom in (0, 33, 150):
        for q in range(3):
            xp = x.copy()
            xp[atom, q] += h
            xm = x.copy()
            xm[atom, q] -= h
            ep = oc.tersoff(box, xp, oc.neighbors(box, xp, rv), p)[1].sum()
            em = oc.tersoff(box, xm, oc.neighbors(box, xm, rv), p)[1].sum()
            assert abs(-(ep - em) / (2 * h) - f[atom, q]) < 2e-6
    # perfect diamond at a = 5.431: Tersoff (1988) Si cohesive energy 4.63 eV/atom
    x0, lo, hi = inputs.diamond(3, 5.431)
    box = oc.make_box(lo, hi, (1, 1, 1))
    e0 = oc.tersoff(box, x0, oc.neighbors(box, x0, rv), p)[1]
    assert abs(e0.mean() + 4.63) < 0.01


def test_velocity_verlet_oracle_matches_reference_trajectory(oracle_lib):
    """20 NVE steps with the reference's first-step rule (forces zeroed after FirstRun)."""
    oc = oracle_lib
    from objectmd_gb300 import inputs

    d = load_case("eam_al_nve")
    phi, ed, em = eam_tables(oc)
    box = oc.make_box(d["box_lo"], d["box_hi"], (1, 1, 1))
    x = oc.wrap(box, d["x0"])
    v = d["v0"].copy()
    n = len(x)
    mass = np.full(n, inputs.md_mass("aluminum"))
    rv = phi.max_range() + 0.3
    f = np.zeros((n, 3))
    dt = float(d["dt"])
    kin = []
    for step in range(int(d["steps"])):
        oc.vv_kick_drift(x, v, f, mass, dt)
        x = oc.wrap(box, x)
        fr, e, vir, rho = oc.eam(box, x, oc.neighbors(box, x, rv), phi, ed, em)
        f = fr
        oc.vv_kick(v, f, mass, dt)
        kin.append(oc.kinetic(v, mass))
    L = d["box_hi"] - d["box_lo"]
    dx = x - d["x"]
    dx -= np.round(dx / L) * L
    assert np.abs(dx).max() < 1e-10
    np.testing.assert_allclose(kin, d["ledger"][1:1 + len(kin), 1], rtol=1e-10)


def test_reference_thermostat_counts_ghost_images(oracle_lib):
    """The reference's TempController divides by owners + periodic ghost images
    (system.h:337 GetTotalAtom = GetNAtom on MDSystemGrid): replaying that rule
    reproduces its kinetic-energy trace exactly."""
    oc = oracle_lib
    from objectmd_gb300 import inputs

    d = load_case("eam_al_tc")
    phi, ed, em = eam_tables(oc)
    box = oc.make_box(d["box_lo"], d["box_hi"], (1, 1, 1))
    lo, hi = d["box_lo"], d["box_hi"]
    x = oc.wrap(box, d["x0"])
    v = d["v0"].copy()
    n = len(x)
    mass = np.full(n, inputs.md_mass("aluminum"))
    rv = phi.max_range() + 0.3
    f = np.zeros((n, 3))
    dt, (tset, tau) = float(d["dt"]), d["tcontrol"]
    kin = []
    for step in range(int(d["steps"])):
        oc.vv_kick_drift(x, v, f, mass, dt)
        x = oc.wrap(box, x)
        f = oc.eam(box, x, oc.neighbors(box, x, rv), phi, ed, em)[0]
        oc.vv_kick(v, f, mass, dt)
        k = oc.kinetic(v, mass)
        kin.append(k)
        ghosts = (np.prod(1 + (x < lo + rv) + (x > hi - rv), axis=1) - 1).sum()
        if step:
            v *= oc.berendsen_factor(dt, tau, tset, (2.0 / 3.0) / 8.61734279e-05 * k / (n + ghosts))
    np.testing.assert_allclose(kin, d["ledger"][1:1 + len(kin), 1], rtol=1e-12)


def test_berendsen_factor(oracle_lib):
    # TempController.h:86: sqrt(1 + dt/tau (T0/T - 1))
    assert abs(oracle_lib.berendsen_factor(0.002, 0.05, 300.0, 600.0) - np.sqrt(1 + 0.04 * (0.5 - 1))) < 1e-15


def test_ttm_oracle_matches_reference(oracle_lib):
    """TTM_Homogen + intensive ThermoDetector on a free EAM Al cluster, 60 steps:
    the restatement (oracle/ttm_oracle.py) replays the reference's electron
    temperature, integrated energies, mean and per-atom local temperatures."""
    oc = oracle_lib
    from objectmd_gb300 import inputs
    from oracle import ttm_oracle as tt

    d = load_case("ttm_al_cluster")
    phi, ed, em = eam_tables(oc)
    tab = os.path.join(TABLES, "ttm.aluminum")
    G = oc.Table.from_file(tab, "ELECTRON_PHONON_COUPLING")
    Ce = oc.Table.from_file(tab, "ELECTRON_HEAT_CAPACITY")
    box = oc.make_box(d["box_lo"], d["box_hi"], (0, 0, 0))
    x = d["x0"].copy()
    v = d["v0"].copy()
    n = len(x)
    mass = np.full(n, inputs.md_mass("aluminum"))
    rv = phi.max_range() + 0.3
    dt = float(d["dt"])
    ttm = tt.TTM(G, Ce, 1.529e-6, 8.43e-10, float(d["atom_volume"]), float(d["te0"]), dt)
    f = np.zeros((n, 3))
    thermo = tt.local_thermo(x, v, mass, phi.max_range())
    kinetic = oc.kinetic(v, mass)
    rows, kin = [], []
    for k in range(int(d["steps"])):
        vmax = np.sqrt((v * v).sum(1).max())
        v = ttm.pre_integration(k * dt, thermo, v, mass, kinetic, vmax)
        oc.vv_kick_drift(x, v, f, mass, dt)
        f = oc.eam(box, x, oc.neighbors(box, x, rv), phi, ed, em)[0]
        oc.vv_kick(v, f, mass, dt)
        kinetic = oc.kinetic(v, mass)
        kin.append(kinetic)
        thermo = tt.local_thermo(x, v, mass, phi.max_range())
        rows.append((k + 1, ttm.te, ttm.int_een, ttm.int_aen, thermo["avg_temp"]))
    rows = np.array(rows)
    ref = d["ttm"]
    np.testing.assert_allclose(rows[:, 1], ref[:, 1], rtol=1e-11)
    np.testing.assert_allclose(rows[:, 2:], ref[:, 2:], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(kin, d["ledger"][1:1 + len(kin), 1], rtol=1e-10)
    np.testing.assert_allclose(thermo["temp"], d["local_temp"], rtol=1e-9)
    np.testing.assert_allclose(thermo["dens"], d["local_dens"], rtol=1e-12)


def test_oracle_sw_and_ar_si_table_match_the_reference_impact_slab(oracle_lib):
    """SW on the Si atoms plus the reference's Ar-Si table between Ar and Si
    (test/si-impact/main.cpp:70-71) equals the reference's own static forces
    and energies for an Ar atom 0.6-3.1 A above a Si slab (periodic x/y, free
    z); the reference build takes SW third atoms of the kernel's types only."""
    oc = oracle_lib
    d = dict(np.load(os.path.join(GOLD, "impact_ar_si_slab.npz")))
    sw = oc.SWParam(eps=2.1683, A=7.049556277, B=0.6022245584, p=4, q=0, sigma=2.0951, a=1.80, lam=21.0, gamma=1.2,
                    icos0=-3.0, usezbl=1, sx0=1.2107, sx1=1.8456, sa0=335.0594, sa1=-492.3905, sa2=244.5280,
                    sa3=-41.2347, z1=14, z2=14)
    phi = oc.Table.from_file(os.path.join(GOLD, "tables", "pair.ar-si.zbl"))
    types = d["types"]
    si = types == 0
    box = oc.make_box(d["box_lo"], d["box_hi"], (1, 1, 0))
    for k in range(len(d["heights"])):
        x = d["static_x0"][k]
        fs, es, _ = oc.sw(box, x[si], oc.neighbors(box, x[si], 2.0951 * 1.8 + 0.3), sw)
        f = np.zeros_like(x)
        e = np.zeros(len(x))
        f[si], e[si] = fs, es
        oc.pair_table_typed(box, x, types, 1, 0, oc.neighbors(box, x, phi.max_range() + 0.3), phi, f, e,
                            np.zeros(len(x)))
        assert np.abs(f - d["static_f"][k]).max() <= 1e-11 * np.abs(d["static_f"][k]).max()
        assert np.abs(e - d["static_pot"][k]).max() <= 1e-12


def test_oracle_matches_the_reference_on_its_own_impact_replica(oracle_lib):
    """The reference's own impact replica (test/si-impact/atom.dat: 10,648 Si
    atoms, periodic x/y, free z, one Ar) with its potentials (SW between Si
    atoms, the Ar-Si table between Ar and Si, test/si-impact/main.cpp:70-71)
    and the Ar atom 0.5-2.0 A above the aim point of its parameter file:
    forces and per-atom energies equal the reference's."""
    oc = oracle_lib
    d = dict(np.load(os.path.join(GOLD, "impact_replica.npz")))
    phi = oc.Table.from_file(os.path.join(GOLD, "tables", "pair.ar-si.zbl"))
    types = d["types"]
    si = types == 0
    box = oc.make_box(d["box_lo"], d["box_hi"], tuple(int(p) for p in d["periodic"]))
    for k in range(len(d["heights"])):
        x = d["x0"].copy()
        x[types == 1] = d["ar"][k]
        xs = oc.wrap(box, x[si])
        fs, es, _ = oc.sw(box, xs, oc.neighbors(box, xs, 2.0951 * 1.8 + 0.3), sw_params(oc))
        f = np.zeros_like(x)
        e = np.zeros(len(x))
        f[si], e[si] = fs, es
        x[si] = xs
        oc.pair_table_typed(box, x, types, 1, 0, oc.neighbors(box, x, phi.max_range() + 0.3), phi, f, e,
                            np.zeros(len(x)))
        assert np.abs(f - d["f"][k]).max() <= 1e-11 * np.abs(d["f"][k]).max()
        assert np.abs(e - d["pot"][k]).max() <= 1e-12
        assert np.abs(d["f"][k][types == 1]).max() > 1.0  # the Ar-Si term acts


def test_oracle_matches_the_reference_with_two_atom_types(oracle_lib):
    """EAM platinum between Pt atoms and the reference's Ar-Pt table between
    an Ar atom and Pt (the combination of test/two_elements/two.cpp), Ar
    1.2-2.8 A above a Pt slab (periodic x/y, free z): forces and per-atom
    energies equal the reference's."""
    oc = oracle_lib
    d = dict(np.load(os.path.join(GOLD, "ar_pt_slab.npz")))
    table = os.path.join(TABLES, "eam.platinum")
    phi, ed, em = (oc.Table.from_file(table, sec) for sec in ("PAIR", "EDENS", "EMBED"))
    zbl = oc.Table.from_file(os.path.join(TABLES, "pair.ar-pt.zbl"))
    types = d["types"]
    pt = types == 0
    box = oc.make_box(d["box_lo"], d["box_hi"], (1, 1, 0))
    for k in range(len(d["heights"])):
        x = d["x0"][k].copy()
        xp = oc.wrap(box, x[pt])
        fp, ep, _, _ = oc.eam(box, xp, oc.neighbors(box, xp, phi.max_range() + 0.3), phi, ed, em)
        f = np.zeros_like(x)
        e = np.zeros(len(x))
        f[pt], e[pt] = fp, ep
        x[pt] = xp
        oc.pair_table_typed(box, x, types, 1, 0, oc.neighbors(box, x, zbl.max_range() + 0.3), zbl, f, e,
                            np.zeros(len(x)))
        assert np.abs(f - d["f"][k]).max() <= 1e-11 * np.abs(d["f"][k]).max()
        assert np.abs(e - d["pot"][k]).max() <= 1e-11
