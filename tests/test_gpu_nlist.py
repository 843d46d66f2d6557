"""Neighbour-list builds on geometries that stress the FP32 screens: every
build variant (cell-centric, thread-per-atom, 4- and 8-lane groups) against
the FP64 oracle's neighbour set, exactly, and the forces of all variants
bitwise equal (the variants emit every row in the same order).

  lattice_ties  simple cubic with spacing Rv/2: the axial second neighbours
                sit at Rv up to the last FP64 bit, so the FP64 test decides
  far_atoms     a free-surface slab with atoms far above and below the cell
                grid (clamped into the edge cells: large cell-local
                coordinates widen the screening band)
  small_axes    periodic axes holding one and two cells (every cell with
                every image)
"""
import os

import numpy as np
import pytest

from conftest import TABLES, nbr_set

pytestmark = pytest.mark.gpu

EAM_TABLE = os.path.join(TABLES, "eam.aluminum5000")
SKIN = 0.3
MODES = (0, 1, 4, 8)


def cutoff(oc):
    return oc.Table.from_file(EAM_TABLE, "PAIR").max_range() + SKIN


def lattice_ties(rv):
    a = rv / 2.0
    m = 8
    g = np.arange(m, dtype=np.float64) * a
    x = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    return x, np.zeros(3), np.full(3, m * a), (1, 1, 1)


def far_atoms(rv):
    from objectmd_gb300 import inputs

    x, _, (lo, hi) = inputs.eam_aluminium(ncell=5, a=4.05, sigma=0.05, temp=300.0, seed_pos=5, seed_vel=6)
    keep = x[:, 2] < 3 * 4.05
    x = x[keep]
    hi = np.array(hi, dtype=np.float64)
    hi[2] = 3 * 4.05
    extra = np.array([[5.0, 6.0, 40.0], [5.0, 6.0, 42.5], [9.0, 1.0, -35.0], [1.0, 1.0, 400.0]])
    return np.concatenate([x, extra]), np.asarray(lo, dtype=np.float64), hi, (1, 1, 0)


def small_axes(rv):
    rng = np.random.default_rng(9)
    L = np.array([1.5 * rv, 2.5 * rv, 4.0 * rv])
    n = int(0.05 * np.prod(L))
    return rng.uniform(0.0, 1.0, (n, 3)) * L, np.zeros(3), L, (1, 1, 1)


def context(omdg, x, lo, hi, periodic, mode):
    from objectmd_gb300 import inputs

    ctx = omdg.Context(0)
    ctx.set_box(lo, hi, tuple(bool(p) for p in periodic))
    ctx.set_atoms(x, np.zeros_like(x), masses=[inputs.md_mass("aluminum")], znum=[13.0])
    ctx.add_eam(EAM_TABLE)
    ctx.set_neighbor(SKIN, 1)
    ctx.set_launch("build_lanes", mode)
    return ctx


@pytest.mark.parametrize("geometry", [lattice_ties, far_atoms, small_axes])
def test_build_variants_match_oracle_and_each_other(omdg_lib, oracle_lib, geometry):
    oc = oracle_lib
    rv = cutoff(oc)
    x, lo, hi, periodic = geometry(rv)
    ref = nbr_set(*oc.neighbors(oc.make_box(lo, hi, periodic), x, rv))
    assert ref
    forces = []
    for mode in MODES:
        with context(omdg_lib, x, lo, hi, periodic, mode) as ctx:
            ctx.compute_forces()
            assert nbr_set(*ctx.neighbors()) == ref, mode
            forces.append(ctx.get_state()["f"])
    for mode, f in zip(MODES[1:], forces[1:]):
        assert np.array_equal(f, forces[0]), mode
