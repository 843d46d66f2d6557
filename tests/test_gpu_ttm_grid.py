"""The two-temperature model with the electron temperature on the cells of
the device finite-difference grid (omdg_set_ttm_grid), on the reference's
TTM case (tests/golden/ttm_al_cluster.npz: 864-atom free EAM Al cluster,
electrons at 5000 K, 2 fs steps).

- one periodic cell and no source is the scalar model (TTM_Homogen): the
  face terms vanish and the update is fd_main_loop's term for term; only the
  lattice average differs (the cells sum temperatures as integers of 2^-20 K),
  so Te agrees to 1e-9 and the kinetic energy to 1e-8 over 60 steps;
- a 4 x 4 grid with diffusion: one coupled step's cell vector equals the
  oracle's (oracle/ttm_oracle.grid_pre_integration on oracle/fdtd_oracle.Grid)
  from the device's own detector temperatures, to 1e-12;
- the coupling's errors: ranged strings, steps and assignments on a coupled
  grid; after detaching, host steps continue.
"""
import os

import numpy as np
import pytest

from conftest import TABLES, load_case

pytestmark = pytest.mark.gpu

TTM_TABLE = os.path.join(TABLES, "ttm.aluminum")
G0, C0 = 1.529e-6, 8.43e-10


def cluster_ctx(omdg, d):
    from objectmd_gb300 import inputs

    ctx = omdg.Context(0)
    ctx.set_box(d["box_lo"], d["box_hi"], (False, False, False))
    ctx.set_atoms(d["x0"], d["v0"], masses=[inputs.md_mass("aluminum")], znum=[13.0])
    ctx.add_eam(os.path.join(TABLES, "eam.aluminum5000"))
    ctx.set_neighbor(0.3, 1)
    ctx.set_timestep(float(d["dt"]))
    ctx.set_ttm(TTM_TABLE, float(d["atom_volume"]), float(d["te0"]), 0.0)
    return ctx


def test_one_periodic_cell_is_the_scalar_model(omdg_lib):
    d = load_case("ttm_al_cluster")
    steps = int(d["steps"])
    with cluster_ctx(omdg_lib, d) as ctx:
        te_s, kin_s = [], []
        for _ in range(steps):
            ctx.step(1)
            te_s.append(ctx.ttm_state()["electron_temperature"])
            kin_s.append(ctx.ledger()["kinetic"])
    lo = np.asarray(d["box_lo"]) - 500.0
    with omdg_lib.FDTD(1, 1, 1, "a pppp", "a") as g, cluster_ctx(omdg_lib, d) as ctx:
        g.set_spacestep(5000.0)
        g.set_cell("a %.17g" % float(d["te0"]))
        ctx.set_ttm_grid(g, lo)
        te_g, kin_g = [], []
        for _ in range(steps):
            ctx.step(1)
            te_g.append(g.vector()[0])
            kin_g.append(ctx.ledger()["kinetic"])
        ctx.set_ttm_grid(None)
    assert te_s[-1] < float(d["te0"]) - 100.0  # the electrons cooled
    np.testing.assert_allclose(te_g, te_s, rtol=1e-9)
    np.testing.assert_allclose(kin_g, kin_s, rtol=1e-8)


def test_coupled_grid_step_matches_the_oracle(omdg_lib, oracle_lib):
    from oracle import fdtd_oracle as fo
    from oracle import ttm_oracle as tt

    d = load_case("ttm_al_cluster")
    G = oracle_lib.Table.from_file(TTM_TABLE, "ELECTRON_PHONON_COUPLING")
    Ce = oracle_lib.Table.from_file(TTM_TABLE, "ELECTRON_HEAT_CAPACITY")
    x0 = d["x0"]
    org = x0.min(0) - 0.5
    h = float((x0.max(0) - x0.min(0))[:2].max() + 1.0) / 4.0
    sym, cmap = "a pppp", "a" * 16
    # explicit-step stability: 2 (con/2) dt / (h^2 cap) per face well below 1/4 (cap = C0 Ce(Te) ~ 2e-6 to 7e-6)
    cond = "a 4e-4 @ 1,1,0,2,2,0=1.5e-4"
    dt = float(d["dt"])
    with omdg_lib.FDTD(4, 4, 1, sym, cmap) as g, cluster_ctx(omdg_lib, d) as ctx:
        g.set_spacestep(h)
        g.set_cell("a 2500 @ 0,0,0,0,3,0=8000 @ 3,2,0=-1")
        g.set_conductivity(cond)
        ctx.set_ttm_grid(g, org)
        ctx.step(3)
        rc = ctx.max_cut_radius()
        volcut = 4.0 * np.pi * rc ** 3 / 3.0
        A0 = g.vector()
        x = ctx.get_state()["x"]
        th = ctx.local_thermo()
        ctx.step(1)
        A1 = g.vector()
        ctx.set_ttm_grid(None)
    nneig = np.rint(th["density"] * volcut).astype(int)
    og = fo.Grid(4, 4, 1, sym, cmap)
    og.set_spacestep(h)
    og.set_timestep(dt)
    og.set_conductivity(cond)
    og.A = A0.copy()
    cells = tt.grid_cells(x, org, h, (4, 4, 1))
    assert (cells >= 0).all()
    ta = tt.grid_pre_integration(og, cells, th["temperature"], nneig, G, Ce, G0, C0, first=False)
    assert (ta > 0).sum() >= 8
    np.testing.assert_allclose(A1, og.A, rtol=1e-12)
    assert A0[3 + 2 * 4] >= 0.0  # the negative cell took its lattice temperature at the first step
    assert np.abs(A1 - A0).max() > 1.0


def test_coupling_errors_and_detach(omdg_lib):
    d = load_case("ttm_al_cluster")
    with omdg_lib.FDTD(2, 2, 1, "a pppp", "aaaa") as g, cluster_ctx(omdg_lib, d) as ctx:
        g.set_spacestep(20.0)
        g.set_cell("a 3000")
        g.set_source("a 5:0:10")
        with pytest.raises(omdg_lib.OMDGError) as ei:
            ctx.set_ttm_grid(g, np.asarray(d["box_lo"]))
        assert "time-ranged" in str(ei.value)
        g.set_source("a 0")
        ctx.set_ttm_grid(g, np.asarray(d["box_lo"]))
        with pytest.raises(omdg_lib.OMDGError):
            g.step(1)
        with pytest.raises(omdg_lib.OMDGError):
            g.set_cell("a 1")
        ctx.step(2)
        ctx.set_ttm_grid(None)
        before = g.vector()
        g.step(1)  # host steps again
        assert g.steps_done == 1 and np.isfinite(g.vector()).all() and before.shape == (4,)
