"""Failure detection, with faults made on the host (no GPU fault, trap or hang).

Each error path returns its OMDG_E* code and the reference's own error text
(the texts of die() in gadget.cpp:149-159 and treader.cpp:199-218), and the
context stays usable: after the bad input is replaced, the same call gives
the same result as a context that never saw it.

- overlapping atoms (r = 1e-4 A, under OMD_PROXIMITY) -> OMDG_EOVERLAP with
  CalcSqrDistance's message naming both atoms and their positions;
- a NaN coordinate -> OMDG_ENONFINITE;
- a pair closer than a pair table's first knot -> OMDG_ERANGE "low limit";
- an electron density beyond the EMBED table (compressed lattice) ->
  OMDG_ERANGE "high limit exeeded in EMBED@...";
- a table file with fewer values than NumberOfData -> OMDG_EFILE;
- bounded waits made to run out: an mbarrier nothing arrives at (in a CTA
  holding TMEM like the tensor-core kernels) and a grid barrier whose count
  the grid cannot reach -> ERR_TIMEOUT in the returned status, device usable.
"""
import os
import re

import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu

EAM_TABLE = os.path.join(TABLES, "eam.aluminum5000")
LJ = os.path.join(TABLES, "pair.lj.argon")
ERR_TIMEOUT = 32


def eam_ctx(omdg, x, v, lo, hi):
    from objectmd_gb300 import inputs

    ctx = omdg.Context(0)
    ctx.set_box(lo, hi)
    ctx.set_atoms(x, v, masses=[inputs.md_mass("aluminum")], znum=[13.0])
    ctx.add_eam(EAM_TABLE)
    ctx.set_neighbor(0.3, 1)
    return ctx


def small_al():
    from objectmd_gb300 import inputs

    return inputs.eam_aluminium(ncell=6, a=4.05, sigma=0.05, temp=300.0, seed_pos=91, seed_vel=92)


def forces(omdg, x, v, lo, hi):
    with eam_ctx(omdg, x, v, lo, hi) as ctx:
        ctx.compute_forces()
        return ctx.get_state()["f"]


def test_overlap_is_reported_with_the_reference_text(omdg_lib):
    x, v, (lo, hi) = small_al()
    good = forces(omdg_lib, x, v, lo, hi)
    bad = x.copy()
    bad[17] = bad[5] + np.array([1e-4, 0.0, 0.0])
    with eam_ctx(omdg_lib, bad, v, lo, hi) as ctx:
        with pytest.raises(omdg_lib.OMDGError) as ei:
            ctx.compute_forces()
        assert ei.value.code == omdg_lib.OMDG_EOVERLAP
        msg = str(ei.value)
        m = re.search(r"CalcSqrDistance: overlapping atoms: r=1\.0E-04 between atom nid=(\d+) and nid=(\d+) "
                      r"\(([-0-9.E+]+),([-0-9.E+]+),([-0-9.E+]+)\) -- \(([-0-9.E+]+),([-0-9.E+]+),([-0-9.E+]+)\)",
                      msg)
        assert m, msg
        assert {int(m.group(1)), int(m.group(2))} == {5, 17}
        a = int(m.group(1))
        np.testing.assert_allclose([float(m.group(k)) for k in (3, 4, 5)], bad[a], rtol=1e-5)
        ctx.set_positions(x)  # the same context recovers
        ctx.compute_forces()
        np.testing.assert_allclose(ctx.get_state()["f"], good, rtol=0, atol=1e-6)


def test_nonfinite_position_is_reported(omdg_lib):
    x, v, (lo, hi) = small_al()
    good = forces(omdg_lib, x, v, lo, hi)
    bad = x.copy()
    bad[3, 0] = np.nan
    with eam_ctx(omdg_lib, bad, v, lo, hi) as ctx:
        with pytest.raises(omdg_lib.OMDGError) as ei:
            ctx.compute_forces()
        assert ei.value.code == omdg_lib.OMDG_ENONFINITE
        ctx.set_positions(x)
        ctx.compute_forces()
        np.testing.assert_allclose(ctx.get_state()["f"], good, rtol=0, atol=1e-6)


def test_pair_closer_than_the_first_knot(omdg_lib):
    """The LJ table starts at 2.0 A; two argon atoms 1.5 A apart."""
    from objectmd_gb300 import inputs

    lo, hi = np.zeros(3), np.full(3, 30.0)
    x = np.array([[10.0, 10.0, 10.0], [11.5, 10.0, 10.0], [20.0, 20.0, 20.0]])
    ctx = omdg_lib.Context(0)
    ctx.set_box(lo, hi)
    ctx.set_atoms(x, np.zeros_like(x), masses=[inputs.md_mass("argon")], znum=[18.0])
    ctx.add_pair_table(LJ)
    ctx.set_neighbor(0.3, 1)
    with pytest.raises(omdg_lib.OMDGError) as ei:
        ctx.compute_forces()
    assert ei.value.code == omdg_lib.OMDG_ERANGE
    msg = str(ei.value)
    assert re.search(r"low limit exeeded in @.*pair\.lj\.argon \(read\) index=-\d+ r=1\.50000E\+00 delta=\S+ "
                     r"low_limit=2\.00000E\+00 hi_limit=8\.51250E\+00", msg), msg
    x[1, 0] = 14.0
    ctx.set_positions(x)
    ctx.compute_forces()
    assert np.isfinite(ctx.get_state()["f"]).all()
    ctx.close()


def test_density_beyond_the_embedding_table(omdg_lib):
    """Aluminium squeezed to a = 2.6 A: the electron density passes the
    EMBED table's last knot."""
    from objectmd_gb300 import inputs

    x, v, (lo, hi) = inputs.eam_aluminium(ncell=5, a=2.6, sigma=0.0, temp=0.0, seed_pos=1, seed_vel=1)
    with eam_ctx(omdg_lib, x, v, lo, hi) as ctx:
        with pytest.raises(omdg_lib.OMDGError) as ei:
            ctx.compute_forces()
    assert ei.value.code == omdg_lib.OMDG_ERANGE
    msg = str(ei.value)
    assert re.search(r"high limit exeeded in EMBED@.*eam\.aluminum5000 \(read\) index=\d+ r=\S+ delta=\S+ "
                     r"low_limit=0\.00000E\+00 hi_limit=1\.90\d+E\+00", msg), msg


def test_truncated_table_file(omdg_lib, tmp_path):
    lines = open(LJ).read().splitlines()
    short = tmp_path / "pair.lj.short"
    short.write_text("\n".join(lines[:200]) + "\n")  # 5000 values announced, under 200 given
    from objectmd_gb300 import inputs

    ctx = omdg_lib.Context(0)
    ctx.set_box(np.zeros(3), np.full(3, 30.0))
    ctx.set_atoms(np.array([[1.0, 1.0, 1.0], [5.0, 5.0, 5.0]]), masses=[inputs.md_mass("argon")], znum=[18.0])
    with pytest.raises(omdg_lib.OMDGError) as ei:
        ctx.add_pair_table(str(short))
    assert ei.value.code == omdg_lib.OMDG_EFILE
    assert "fewer than NumberOfData values" in str(ei.value)
    with pytest.raises(omdg_lib.OMDGError) as ei:
        ctx.add_pair_table(str(tmp_path / "missing.table"))
    assert ei.value.code == omdg_lib.OMDG_EFILE
    ctx.close()


@pytest.mark.parametrize("which,polls", [(0, 1000), (1, 100000)])
def test_bounded_waits_run_out_and_return(omdg_lib, which, polls):
    st = omdg_lib.selftest_wait(which, polls)
    assert st & ERR_TIMEOUT, st
    x, v, (lo, hi) = small_al()  # the device still runs work afterwards
    assert np.isfinite(forces(omdg_lib, x, v, lo, hi)).all()


def test_wait_poll_limit_is_settable(omdg_lib):
    omdg_lib.set_wait_polls(5)
    try:
        assert omdg_lib.selftest_wait(0, 5) & ERR_TIMEOUT
    finally:
        omdg_lib.set_wait_polls(0)
    with pytest.raises(omdg_lib.OMDGError):
        omdg_lib.set_wait_polls(-1)
