"""Replica mode (the batched impact ensemble) against the same replicas run
one by one in single-box contexts: Si slabs, periodic in x and y with a free
surface, Tersoff Si-Si plus ZBL Ar-Si, one Ar atom per replica.

Neighbour sets are compared exactly.  Forces agree to FP32 summation order
(the two paths list neighbours in different orders): components within
1e-5 max|f| + 1e-6 eV/A.  Per-replica energies within 1e-6 relative, and
positions after 50 steps of 0.5 fs through the impact within 1e-5 A.
"""
import os

import numpy as np
import pytest

from conftest import TABLES, nbr_set

pytestmark = pytest.mark.gpu

TERSOFF = os.path.join(TABLES, "tersoff.silicon27")
SKIN = 1.0


@pytest.fixture(scope="module")
def ensemble():
    from objectmd_gb300 import inputs

    return inputs.impact_ensemble(nrep=3, nmin=400, nmax=1500, emin=50.0, emax=200.0, seed=3)


def potentials(ctx):
    ctx.add_tersoff(TERSOFF)
    ctx.add_zbl(1, 0, 3.0, 0.5)
    ctx.set_neighbor(SKIN, 0)
    ctx.set_timestep(0.0005)
    ctx.set_first_step_mode(False)


def batch_context(omdg, e):
    ctx = omdg.Context(0)
    ctx.set_replicas(e["natoms"], e["lo"], e["hi"], (1, 1, 0))
    ctx.set_atoms(e["x"], e["v"], types=e["types"], masses=e["masses"], znum=e["znum"])
    potentials(ctx)
    return ctx


def single_contexts(omdg, e):
    start = np.concatenate([[0], np.cumsum(e["natoms"])])
    out = []
    for r in range(len(e["natoms"])):
        sl = slice(start[r], start[r + 1])
        ctx = omdg.Context(0)
        ctx.set_box(e["lo"][r], e["hi"][r], (True, True, False))
        ctx.set_atoms(e["x"][sl], e["v"][sl], types=e["types"][sl], masses=e["masses"], znum=e["znum"])
        potentials(ctx)
        out.append((sl, ctx))
    return out


def test_replicas_match_single_boxes(omdg_lib, ensemble):
    e = ensemble
    start = np.concatenate([[0], np.cumsum(e["natoms"])])
    with batch_context(omdg_lib, e) as b:
        b.compute_forces()
        st = b.get_state()
        off, j, code = b.neighbors()
        kin_b, pot_b = b.replica_ledger()
        singles = single_contexts(omdg_lib, e)
        try:
            for r, (sl, ctx) in enumerate(singles):
                ctx.compute_forces()
                s1 = ctx.get_state()
                f, f1 = st["f"][sl], s1["f"]
                assert np.abs(f - f1).max() <= 1e-5 * np.abs(f1).max() + 1e-6
                assert np.abs(st["pot"][sl] - s1["pot"]).max() < 1e-5
                # neighbour tuples of the replica, renumbered to replica-local atoms
                o = off[start[r]:start[r + 1] + 1] - off[start[r]]
                jj = j[off[start[r]]:off[start[r + 1]]] - start[r]
                cc = code[off[start[r]]:off[start[r + 1]]]
                assert nbr_set(o, jj, cc) == nbr_set(*ctx.neighbors())
                led = ctx.ledger()
                assert abs(kin_b[r] - led["kinetic"]) <= 1e-6 * abs(led["kinetic"])
                assert abs(pot_b[r] - s1["pot"].sum()) <= 1e-6 * abs(s1["pot"].sum())
        finally:
            for _, ctx in singles:
                ctx.close()


def test_replica_trajectories_match_single_boxes(omdg_lib, ensemble):
    """Also the per-replica rebuilds: a replica is re-listed exactly when it
    would be running alone (one of its own atoms moved past skin/2), so its
    build count equals its single box's."""
    e = ensemble
    nrep = len(e["natoms"])
    with batch_context(omdg_lib, e) as b:
        b.step(50)
        xb = b.get_state()["x"]
        builds = b.replica_builds(nrep)
    alone = []
    for r, (sl, ctx) in enumerate(single_contexts(omdg_lib, e)):
        with ctx:
            ctx.step(50)
            x1 = ctx.get_state()["x"]
            alone.append(ctx.stats()["rebuilds"])
        L = np.asarray(e["hi"][r]) - np.asarray(e["lo"][r])
        dx = xb[sl] - x1
        dx[:, :2] -= np.round(dx[:, :2] / L[:2]) * L[:2]
        assert np.abs(dx).max() < 1e-5, r
    assert list(builds) == alone
    assert len(set(alone)) > 1  # the replicas rebuild at their own rates


def test_state_upload_between_steps(omdg_lib, ensemble):
    """Positions and velocities written back between steps (a rebuild with the
    step graph already captured) continue the same trajectory."""
    e = ensemble
    with batch_context(omdg_lib, e) as a:
        a.step(20)
        xa = a.get_state()["x"]
    with batch_context(omdg_lib, e) as b:
        b.step(10)
        st = b.get_state()
        for _ in range(2):
            b.set_positions(st["x"])
            b.set_velocities(st["v"])
            b.step(5)
            st = b.get_state()
        xb = st["x"]
    hi, lo = np.asarray(e["hi"]), np.asarray(e["lo"])
    start = np.concatenate([[0], np.cumsum(e["natoms"])])
    for r in range(len(e["natoms"])):
        sl = slice(start[r], start[r + 1])
        L = hi[r] - lo[r]
        dx = xa[sl] - xb[sl]
        dx[:, :2] -= np.round(dx[:, :2] / L[:2]) * L[:2]
        assert np.abs(dx).max() < 1e-5


def test_persistent_tersoff_pass_is_the_same(omdg_lib, ensemble):
    """The Tersoff register pass as one resident grid striding over the
    flattened atoms of every replica gives the same forces bit for bit."""
    e = ensemble
    out = []
    for persistent in (0, 1):
        with batch_context(omdg_lib, e) as b:
            b.set_launch("tb_persistent", persistent)
            b.step(10)
            st = b.get_state()
            out.append((st["x"], st["f"], st["pot"]))
    for a, b_ in zip(*out):
        assert np.array_equal(a, b_)
