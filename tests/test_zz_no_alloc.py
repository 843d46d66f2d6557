"""omdg_count_neighbors_static (the allocation-free entry point) against the
per-atom neighbour counts of the list omdg_build_neighbors builds.

Counts are integers: they must be equal.  Two calls in a row (the second on
positions after 40 MD steps) share the static scratch; a repeated call on the
same input must give the same counts.  This file is collected last so that it
also runs after every other test has used the device.
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


def static_counts(omdg, x, lo, hi, rcut):
    import torch

    xd = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).cuda()
    cnt = torch.full((len(x),), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    lib = omdg.load()
    err = ctypes.create_string_buffer(256)
    rc = lib.omdg_count_neighbors_static(ctypes.c_void_p(xd.data_ptr()), len(x), (ctypes.c_double * 3)(*lo),
                                         (ctypes.c_double * 3)(*hi), (ctypes.c_int * 3)(1, 1, 1), rcut,
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
    with pytest.raises(omdg_lib.OMDGError, match="shorter than 3 rcut"):
        omdg_lib.count_neighbors_static(None, 0, lo, hi, p, 20.0, None)
