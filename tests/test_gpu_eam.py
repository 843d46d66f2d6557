"""EAM on the GPU against the reference's own outputs (golden) and the FP64 oracle.

Tolerance (FP32 forces from FP64 positions, Kahan sums): the norm-wise
relative force error ||f - f_ref|| / ||f_ref|| <= 1e-5, every component
within 1e-5 * max|f_ref| + 1e-6 eV/A, per-atom energy within 2e-6 eV and the
total potential within 5e-8 relative (per-atom energies are FP32, whose
rounding near 3.4 eV is 1.2e-7 eV).  Neighbour sets are compared exactly.
"""
import os

import numpy as np
import pytest

from conftest import TABLES, load_case, nbr_set

pytestmark = pytest.mark.gpu

FORCE_REL = 1e-5
EAM_TABLE = os.path.join(TABLES, "eam.aluminum5000")


def make_eam(omdg, d, rebuild_every=1):
    from objectmd_gb300 import inputs

    ctx = omdg.Context(0)
    ctx.set_box(d["box_lo"], d["box_hi"], (True, True, True))
    ctx.set_atoms(d["x0"], d["v0"], masses=[inputs.md_mass("aluminum")], znum=[13.0])
    ctx.add_eam(EAM_TABLE)
    ctx.set_neighbor(skin=0.3, rebuild_every=rebuild_every)
    return ctx


def check_forces(f, fref, pot=None, potref=None):
    rel = np.linalg.norm(f - fref) / np.linalg.norm(fref)
    assert rel <= FORCE_REL, rel
    assert np.abs(f - fref).max() <= FORCE_REL * np.abs(fref).max() + 1e-6
    if pot is not None:
        assert np.abs(pot - potref).max() <= 2e-6
        assert abs(pot.sum() - potref.sum()) <= 5e-8 * abs(potref.sum())


@pytest.mark.parametrize("case", ["eam_al_500", "eam_al_4000"])
def test_eam_static_matches_reference(omdg_lib, case):
    d = load_case(case)
    with make_eam(omdg_lib, d) as ctx:
        ctx.compute_forces()
        st = ctx.get_state()
        check_forces(st["f"], d["f"], st["pot"], d["pot"])
        assert np.abs(st["vir"] - d["vir"]).max() <= 1e-5 * np.abs(d["vir"]).max() + 1e-5
        led = ctx.ledger()
        assert abs(led["potential"] - float(d["summary_potential"][0])) <= 5e-8 * abs(led["potential"])


@pytest.mark.parametrize("case", ["eam_al_500", "eam_al_4000"])
def test_eam_neighbour_set_bit_exact(omdg_lib, case):
    d = load_case(case)
    with make_eam(omdg_lib, d) as ctx:
        ctx.build_neighbors()
        mine = nbr_set(*ctx.neighbors())
    ref = set(map(tuple, d["nbr"].tolist()))
    assert mine == ref


@pytest.mark.parametrize("mode", [0, 1, 4, 8])
def test_build_modes_give_the_reference_set(omdg_lib, mode):
    """Cell-centric, thread-per-atom and lane-group builds all give the reference's set."""
    d = load_case("eam_al_4000")
    with make_eam(omdg_lib, d) as ctx:
        ctx.set_launch("build_lanes", mode)
        ctx.build_neighbors()
        mine = nbr_set(*ctx.neighbors())
    assert mine == set(map(tuple, d["nbr"].tolist()))


@pytest.mark.parametrize("lanes,hshift,stage", [(1, 5, 0), (4, 3, 0), (8, 2, 0), (16, 1, 0), (4, 3, 1), (8, 2, 1)])
def test_eam_lane_shapes_agree(omdg_lib, lanes, hshift, stage):
    """Every lane shape of the gather passes, with the spline knots read
    from global memory or staged in shared memory, against the reference."""
    d = load_case("eam_al_4000")
    with make_eam(omdg_lib, d) as ctx:
        ctx.set_launch("eam_tile", 0)
        ctx.set_launch("eam_lanes", lanes)
        ctx.set_launch("nbr_hshift", hshift)
        ctx.set_launch("eam_stage", stage)
        ctx.compute_forces()
        st = ctx.get_state()
    check_forces(st["f"], d["f"], st["pot"], d["pot"])


@pytest.mark.parametrize("lanes", [4, 8, 16])
@pytest.mark.parametrize("shape", [(2, 2, 2), (3, 1, 2), (4, 4, 4)])
def test_eam_tiles_match_reference(omdg_lib, lanes, shape):
    """The tiled passes (every tile's halo staged in shared memory, rows of
    16-bit slots from the list build) against the reference, and against
    the gather passes on the same list: forces to 1e-6 relative (only pairs
    across a periodic face round their lo parts in another order)."""
    d = load_case("eam_al_4000")
    out = {}
    for tile in (1, 0):
        with make_eam(omdg_lib, d) as ctx:
            ctx.set_launch("eam_tile", tile)
            ctx.set_launch("tile_cap", 5000)  # a 4x4x4 tile's halo is this whole box
            for key, v in zip(("tile_x", "tile_y", "tile_z"), shape):
                ctx.set_launch(key, v)
            ctx.set_launch("eam_lanes", lanes)
            ctx.compute_forces()
            st = ctx.get_state()
            tiles, staged = ctx.tile_counts()
            if tile:
                assert tiles > 1 and staged == tiles
            else:
                assert tiles == 0
            check_forces(st["f"], d["f"], st["pot"], d["pot"])
            out[tile] = st
    a, b = out[1], out[0]
    assert np.linalg.norm(a["f"] - b["f"]) <= 1e-6 * np.linalg.norm(b["f"])
    assert np.abs(a["pot"] - b["pot"]).max() <= 1e-6


def test_eam_tiles_past_capacity_take_the_gather_path(omdg_lib):
    """Tiles whose halo holds more atoms than tile_cap are evaluated by the
    gather passes inside the tiled launch: with a cap below every halo none
    is staged, with one inside the spread of the halo counts some are."""
    d = load_case("eam_al_4000")
    with make_eam(omdg_lib, d) as ctx:
        ctx.set_launch("eam_tile", 1)
        ctx.set_launch("tile_cap", 64)
        ctx.compute_forces()
        st = ctx.get_state()
        tiles, staged = ctx.tile_counts()
        assert tiles > 1 and staged == 0
        check_forces(st["f"], d["f"], st["pot"], d["pot"])
        mixed = None
        for cap in range(900, 1500, 5):
            ctx.set_launch("tile_cap", cap)
            ctx.build_neighbors()
            tiles, staged = ctx.tile_counts()
            if 0 < staged < tiles:
                mixed = cap
                break
        assert mixed is not None
        ctx.compute_forces()
        st = ctx.get_state()
    check_forces(st["f"], d["f"], st["pot"], d["pot"])


def test_eam_tiles_free_surface_slab(omdg_lib, oracle_lib):
    """A slab free in z (no image across it; halo cells past the grid are
    empty) with the tiled passes, against the FP64 oracle."""
    from objectmd_gb300 import inputs

    oc = oracle_lib
    x, v, (lo, hi) = inputs.eam_aluminium(ncell=10, a=4.05, sigma=0.05, temp=300.0, seed_pos=41, seed_vel=42)
    hi = np.array(hi, dtype=np.float64)
    hi[2] += 6.0  # vacuum above the slab
    phi = oc.Table.from_file(EAM_TABLE, "PAIR")
    ed = oc.Table.from_file(EAM_TABLE, "EDENS")
    em = oc.Table.from_file(EAM_TABLE, "EMBED")
    box = oc.make_box(lo, hi, (1, 1, 0))
    nb = oc.neighbors(box, x, phi.max_range() + 0.3)
    fref, eref, _, _ = oc.eam(box, x, nb, phi, ed, em)
    with omdg_lib.Context(0) as ctx:
        ctx.set_box(lo, hi, (True, True, False))
        ctx.set_atoms(x, v, masses=[inputs.md_mass("aluminum")], znum=[13.0])
        ctx.add_eam(EAM_TABLE)
        ctx.set_neighbor(0.3, 1)
        ctx.set_launch("eam_tile", 1)
        ctx.compute_forces()
        st = ctx.get_state()
        tiles, staged = ctx.tile_counts()
    assert tiles > 1 and staged == tiles
    check_forces(st["f"], fref, st["pot"], eref)


def test_eam_large_vs_oracle(omdg_lib, oracle_lib):
    """32,000 atoms: forces against the FP64 C oracle on the same input."""
    from objectmd_gb300 import inputs

    oc = oracle_lib
    x, v, (lo, hi) = inputs.eam_aluminium(ncell=20, a=4.05, sigma=0.05, temp=300.0, seed_pos=31, seed_vel=32)
    phi = oc.Table.from_file(EAM_TABLE, "PAIR")
    ed = oc.Table.from_file(EAM_TABLE, "EDENS")
    em = oc.Table.from_file(EAM_TABLE, "EMBED")
    box = oc.make_box(lo, hi, (1, 1, 1))
    nb = oc.neighbors(box, x, phi.max_range() + 0.3)
    fref, eref, vref, rho = oc.eam(box, x, nb, phi, ed, em)
    ctx = omdg_lib.Context(0)
    ctx.set_box(lo, hi)
    ctx.set_atoms(x, v, masses=[inputs.md_mass("aluminum")], znum=[13.0])
    ctx.add_eam(EAM_TABLE)
    ctx.set_neighbor(0.3, 1)
    ctx.compute_forces()
    st = ctx.get_state()
    check_forces(st["f"], fref, st["pot"], eref)
    mine = nbr_set(*ctx.neighbors())
    ref = nbr_set(*nb)
    assert mine == ref
    ctx.close()


def test_eam_nve_trajectory_matches_reference(omdg_lib):
    """20 steps of velocity Verlet (dt 2 fs) with the reference's first-step rule."""
    d = load_case("eam_al_nve")
    with make_eam(omdg_lib, d, rebuild_every=1) as ctx:
        ctx.set_timestep(float(d["dt"]))
        ctx.set_first_step_mode(True)
        ctx.step(int(d["steps"]))
        st = ctx.get_state()
        kin, pot = ctx.ledger_history()
        led = ctx.ledger()
    L = d["box_hi"] - d["box_lo"]
    dx = st["x"] - d["x"]
    dx -= np.round(dx / L) * L  # the reference wraps owners at every refresh
    assert np.abs(dx).max() < 1e-6
    assert np.abs(st["v"] - d["v"]).max() < 1e-4 * np.abs(d["v"]).max()
    ref = d["ledger"]  # step kinetic potential energy
    assert len(kin) == int(d["steps"])
    np.testing.assert_allclose(kin, ref[1:1 + len(kin), 1], rtol=1e-6)
    np.testing.assert_allclose(pot, ref[1:1 + len(pot), 2], rtol=5e-8)
    assert abs(led["base_potential"] - float(d["summary_base_potential"][0])) < 5e-8 * abs(led["base_potential"])


def test_eam_graph_and_eager_agree(omdg_lib):
    """The captured step graph and the eager launch sequence give identical state."""
    d = load_case("eam_al_nve")
    out = []
    for profiling in (False, True):
        with make_eam(omdg_lib, d, rebuild_every=0) as ctx:
            ctx.set_timestep(0.002)
            ctx.set_profiling(profiling)
            ctx.step(30)
            out.append(ctx.get_state())
    np.testing.assert_array_equal(out[0]["x"], out[1]["x"])
    np.testing.assert_array_equal(out[0]["f"], out[1]["f"])


def test_eam_nve_drift_over_10k_steps(omdg_lib):
    """10^4 NVE steps (20 ps) of 4000 Al atoms at 300 K with displacement-
    triggered rebuilds: energy drift below 5e-4 eV/atom (1.1e-4 measured on a
    GB300)."""
    from objectmd_gb300 import inputs

    x, v, (lo, hi) = inputs.eam_aluminium(ncell=10, temp=300.0)
    with omdg_lib.Context(0) as ctx:
        ctx.set_box(lo, hi)
        ctx.set_atoms(x, v, masses=[inputs.md_mass("aluminum")], znum=[13.0])
        ctx.add_eam(EAM_TABLE)
        ctx.set_neighbor(0.3, 0)
        ctx.set_timestep(0.002)
        ctx.set_first_step_mode(False)
        ctx.step(1)
        e0 = ctx.ledger()["energy"]
        ctx.step(10000)
        e1 = ctx.ledger()["energy"]
    assert np.isfinite(e1)
    assert abs(e1 - e0) / len(x) < 5e-4


def test_position_upload_keeps_or_rebuilds_the_list(omdg_lib):
    """Positions set by the caller keep the list while every atom stays within
    skin/2 of where the list was built, and trigger a rebuild otherwise; the
    forces equal those of a fresh context on the same positions either way."""
    d = load_case("eam_al_500")
    rng = np.random.default_rng(8)
    with make_eam(omdg_lib, d, rebuild_every=0) as ctx:
        ctx.compute_forces()
        r0 = ctx.stats()["rebuilds"]
        for shift, rebuilt in ((0.05, False), (0.4, True)):  # skin/2 = 0.15 A
            x = d["x0"].copy()
            x[7] += rng.normal(size=3) * shift / np.sqrt(3.0) + np.array([shift, 0.0, 0.0])
            ctx.set_positions(x)
            ctx.compute_forces()
            r1 = ctx.stats()["rebuilds"]
            assert (r1 > r0) == rebuilt
            r0 = r1
            f = ctx.get_state()["f"]
            fresh = dict(d)
            fresh["x0"] = x
            with make_eam(omdg_lib, fresh, rebuild_every=0) as ref:
                ref.compute_forces()
                fr = ref.get_state()["f"]
            assert np.abs(f - fr).max() <= 1e-6 * np.abs(fr).max() + 1e-7


def test_pinned_transfers_equal_staged_transfers(omdg_lib):
    """Pinned host arrays are read and written by the device in place,
    pageable ones through a staging copy: the same state comes back bit for
    bit either way, uploads from pinned arrays land exactly, and a pinned
    upload that moves an atom beyond skin/2 triggers the rebuild."""
    torch = pytest.importorskip("torch")
    d = load_case("eam_al_500")
    n = len(d["x0"])
    pin = lambda *shape: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()  # noqa: E731
    with make_eam(omdg_lib, d, rebuild_every=0) as ctx:
        ctx.step(3)
        x, v, f, pot, vir = pin(n, 3), pin(n, 3), pin(n, 3), pin(n), pin(n)
        ctx.get_state_into(x=x, v=v, f=f, pot=pot, vir=vir)
        st = ctx.get_state()  # pageable arrays
        for a, k in ((x, "x"), (v, "v"), (f, "f"), (pot, "pot"), (vir, "vir")):
            np.testing.assert_array_equal(a, st[k])
        rng = np.random.default_rng(5)
        x += rng.normal(size=x.shape) * 0.01
        v *= 1.5
        ctx.set_state(x=x, v=v)
        st = ctx.get_state()
        np.testing.assert_array_equal(st["x"], x)
        np.testing.assert_array_equal(st["v"], v)
        ctx.compute_forces()
        r0 = ctx.stats()["rebuilds"]
        x[11, 0] += 0.4  # skin/2 = 0.15 A
        ctx.set_state(x=x)
        ctx.compute_forces()
        assert ctx.stats()["rebuilds"] > r0
        f_pinned = ctx.get_state()["f"]
        ctx.set_positions(np.array(x))  # the same positions from pageable memory
        ctx.compute_forces()
        np.testing.assert_array_equal(ctx.get_state()["f"], f_pinned)


@pytest.mark.parametrize("rebuild_every", [0, 1])
def test_step_io_equals_upload_step_readback(omdg_lib, rebuild_every):
    """omdg_step_io (upload, steps, read-back in one call) gives bit for bit
    what set_state + step + get_state give: with pinned outputs (written by
    the step graph's download branch while the last step runs; with a list
    rebuild in every step the positions are read after its permutation), with
    pageable outputs, and again after the output arrays change."""
    torch = pytest.importorskip("torch")
    d = load_case("eam_al_500")
    n = len(d["x0"])
    pin = lambda: torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()  # noqa: E731
    rng = np.random.default_rng(3)
    x_in = d["x0"] + rng.normal(size=(n, 3)) * 0.02
    v_in = d["v0"] * 1.2
    with make_eam(omdg_lib, d, rebuild_every=rebuild_every) as a, \
            make_eam(omdg_lib, d, rebuild_every=rebuild_every) as b:
        a.step(2)
        b.step(2)
        for outs in ((pin(), pin(), pin()), (pin(), pin(), pin()), (np.zeros((n, 3)), np.zeros((n, 3)),
                                                                      np.zeros((n, 3)))):
            x, v, f = outs
            a.step_io(3, x_in=x_in, v_in=v_in, x_out=x, v_out=v, f_out=f)
            b.set_state(x=x_in, v=v_in)
            b.step(3)
            st = b.get_state()
            np.testing.assert_array_equal(x, st["x"])
            np.testing.assert_array_equal(v, st["v"])
            np.testing.assert_array_equal(f, st["f"])
            ka, pa = a.ledger_history()
            kb, pb = b.ledger_history()
            np.testing.assert_array_equal(ka, kb)
            np.testing.assert_array_equal(pa, pb)
            x_in, v_in = st["x"], st["v"]


def test_kick_in_the_force_epilogue_is_the_same_step(omdg_lib):
    """The step's second half-kick done by the EAM force kernel's epilogue
    (launch key fuse_kick, for one EAM potential) against the separate kick kernel:
    positions, velocities and forces bit for bit after 30 steps with two
    rebuilds, the ledger to FP32-pair summation order."""
    from objectmd_gb300 import inputs

    x, v, (lo, hi) = inputs.eam_aluminium(ncell=12, a=4.05, sigma=0.05, temp=600.0, seed_pos=71, seed_vel=72)
    out = []
    for fuse in (1, 0):
        with omdg_lib.Context(0) as ctx:
            ctx.set_box(lo, hi)
            ctx.set_atoms(x, v, masses=[inputs.md_mass("aluminum")], znum=[13.0])
            ctx.add_eam(os.path.join(TABLES, "eam.aluminum5000"))
            ctx.set_neighbor(0.1, 0)
            ctx.set_timestep(0.002)
            ctx.set_launch("eam_tile", 0)  # the fused kick rides on the gather passes
            ctx.set_launch("fuse_kick", fuse)
            ctx.step(30)
            kin, pot = ctx.ledger_history()
            out.append((ctx.get_state(), kin, pot, ctx.stats()["rebuilds"]))
    (a, ka, pa, ra), (b, kb, pb, rb) = out
    assert ra == rb and ra >= 2
    for k in ("x", "v", "f", "pot"):
        assert np.array_equal(a[k], b[k]), k
    np.testing.assert_allclose(ka, kb, rtol=1e-6)
    np.testing.assert_allclose(pa, pb, rtol=1e-7)
