"""omdg_count_neighbors_static (the allocation-free entry point) against the
per-atom neighbour counts of the list omdg_build_neighbors builds.

Counts are integers: they must be equal.  Two calls in a row (the second on
positions after 40 MD steps) share the static scratch; a repeated call on the
same input must give the same counts.  Three more boxes exercise the branches
a fully periodic crystal never reaches, against a brute-force count on the
CPU: a free axis with atoms outside [lo, hi) (clamped into the edge cells), a
sparse box whose grid is coarsened to the scratch's cell limit, and a
periodic axis just over 3 rcut (exactly three cells).  This file is collected
last so that it also runs after every other test has used the device.
"""
import ctypes
import os

import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu


def list_counts(off, j, n):
    """Per-atom neighbours of the list: omdg_get_neighbors gives every atom's
    full row (each pair appears in both rows)."""
    rows = np.repeat(np.arange(n), np.diff(off))
    assert np.array_equal(np.bincount(rows, minlength=n), np.bincount(j, minlength=n))
    return np.diff(off)


def static_counts(omdg, x, lo, hi, rcut, periodic=(1, 1, 1)):
    import torch

    xd = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).cuda()
    cnt = torch.full((len(x),), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    lib = omdg.load()
    err = ctypes.create_string_buffer(256)
    rc = lib.omdg_count_neighbors_static(ctypes.c_void_p(xd.data_ptr()), len(x), (ctypes.c_double * 3)(*lo),
                                         (ctypes.c_double * 3)(*hi), (ctypes.c_int * 3)(*periodic), rcut,
                                         ctypes.c_void_p(cnt.data_ptr()), ctypes.c_void_p(stream.cuda_stream), err,
                                         256)
    assert rc == 0, err.value
    stream.synchronize()
    return cnt.cpu().numpy()


def test_static_counts_match_the_verlet_list(omdg_lib):
    from objectmd_gb300 import inputs

    x0, v0, (lo, hi) = inputs.eam_aluminium(ncell=12, temp=600.0)
    skin = 0.3
    with omdg_lib.Context(0) as ctx:
        ctx.set_box(lo, hi)
        ctx.set_atoms(x0, v0, masses=[inputs.md_mass("aluminum")], znum=[13.0])
        ctx.add_eam(os.path.join(TABLES, "eam.aluminum5000"))
        ctx.set_neighbor(skin, 0)
        rcut = ctx.max_cut_radius() + skin
        n = len(x0)

        ctx.build_neighbors()
        x = ctx.get_state()["x"]
        off, j, _ = ctx.neighbors()
        want1 = list_counts(off, j, n)
        got1 = static_counts(omdg_lib, x, lo, hi, rcut)

        ctx.set_timestep(0.002)
        ctx.step(40)
        ctx.build_neighbors()
        x2 = ctx.get_state()["x"]
        off2, j2, _ = ctx.neighbors()
        want2 = list_counts(off2, j2, n)
        got2 = static_counts(omdg_lib, x2, lo, hi, rcut)
        again = static_counts(omdg_lib, x2, lo, hi, rcut)

    assert want1.min() > 0
    np.testing.assert_array_equal(got1, want1)
    np.testing.assert_array_equal(got2, want2)
    np.testing.assert_array_equal(again, got2)
    assert not np.array_equal(want1, want2)  # the second call saw different input


def test_static_limits_are_errors(omdg_lib):
    lo, hi, p = (0.0, 0.0, 0.0), (50.0, 50.0, 50.0), (1, 1, 1)
    with pytest.raises(omdg_lib.OMDGError, match="static scratch limit"):
        omdg_lib.count_neighbors_static(None, omdg_lib.OMDG_STATIC_MAX_ATOMS + 1, lo, hi, p, 5.0, None)
    with pytest.raises(omdg_lib.OMDGError, match="not longer than 3 rcut"):
        omdg_lib.count_neighbors_static(None, 0, lo, hi, p, 20.0, None)


def wrap(x, lo, hi, periodic):
    """Periodic axes wrapped into [lo, hi) as the static path does:
    x - floor((x - lo) / L) L in FP64."""
    x = np.array(x, dtype=np.float64)
    for d in range(3):
        if periodic[d]:
            L = hi[d] - lo[d]
            x[:, d] = x[:, d] - np.floor((x[:, d] - lo[d]) / L) * L
    return x


def brute_counts(x, lo, hi, periodic, rcut):
    """Every (owner or image) neighbour with (dx dx + dy dy) + dz dz <= rcut^2,
    the image of j being x_j + s L with s in {-1, 0, 1} on periodic axes."""
    w = wrap(x, lo, hi, periodic)
    L = np.array(hi, dtype=np.float64) - np.array(lo, dtype=np.float64)
    n = len(w)
    cnt = np.zeros(n, dtype=np.int64)
    rng = [(-1, 0, 1) if periodic[d] else (0,) for d in range(3)]
    for sx in rng[0]:
        for sy in rng[1]:
            for sz in rng[2]:
                s = np.array([sx, sy, sz], dtype=np.float64) * L
                dx = w[:, None, 0] - (w[None, :, 0] + s[0])
                dy = w[:, None, 1] - (w[None, :, 1] + s[1])
                dz = w[:, None, 2] - (w[None, :, 2] + s[2])
                within = ((dx * dx + dy * dy) + dz * dz) <= rcut * rcut
                if sx == 0 and sy == 0 and sz == 0:
                    np.fill_diagonal(within, False)
                cnt += within.sum(axis=1)
    return cnt


def test_static_free_axis_with_atoms_outside_the_box(omdg_lib):
    rng = np.random.default_rng(11)
    lo, hi, per, rcut = (0.0, 0.0, 0.0), (12.0, 12.0, 12.0), (1, 1, 0), 3.0
    n = 1500
    x = np.column_stack([rng.uniform(-1.0, 13.0, n), rng.uniform(0.0, 12.0, n), rng.uniform(-4.0, 16.0, n)])
    assert (x[:, 2] < lo[2]).sum() > 50 and (x[:, 2] >= hi[2]).sum() > 50
    want = brute_counts(x, lo, hi, per, rcut)
    got = static_counts(omdg_lib, x, lo, hi, rcut, per)
    again = static_counts(omdg_lib, x, lo, hi, rcut, per)
    assert want.max() > 20
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(again, got)


def test_static_sparse_box_coarsened_grid(omdg_lib):
    """50 rcut per axis gives 125,000 cells, above the 32,768-cell scratch, so
    the grid is coarsened (wider cells stay correct)."""
    spatial = pytest.importorskip("scipy.spatial")
    rng = np.random.default_rng(12)
    L, rcut, n = 100.0, 2.0, 40000
    assert (L / rcut) ** 3 > omdg_lib.OMDG_STATIC_MAX_CELLS
    lo, hi, per = (0.0, 0.0, 0.0), (L, L, L), (1, 1, 1)
    x = rng.uniform(0.0, L, (n, 3))
    x[:100] += rng.choice([-L, L], (100, 3))  # some atoms outside: wrapped on the fly
    w = wrap(x, lo, hi, per)
    tree = spatial.cKDTree(w, boxsize=L)
    want = tree.query_ball_point(w, rcut, return_length=True) - 1
    got = static_counts(omdg_lib, x, lo, hi, rcut, per)
    assert want.sum() > n
    np.testing.assert_array_equal(got, want)


def test_static_periodic_axis_just_over_three_cutoffs(omdg_lib):
    rng = np.random.default_rng(13)
    rcut = 2.5
    lo, hi, per = (0.0, 0.0, 0.0), (3 * rcut * (1 + 1e-9), 13.0, 11.0), (1, 1, 1)
    n = 900
    x = rng.uniform(0.0, 1.0, (n, 3)) * np.array(hi)
    want = brute_counts(x, lo, hi, per, rcut)
    got = static_counts(omdg_lib, x, lo, hi, rcut, per)
    np.testing.assert_array_equal(got, want)
    with pytest.raises(omdg_lib.OMDGError, match="not longer than 3 rcut"):
        omdg_lib.count_neighbors_static(None, 0, lo, (3 * rcut, 13.0, 11.0), per, rcut, None)
