"""ThermoDetector and TTM_Homogen on the GPU against the reference's own run
(tests/golden/ttm_al_cluster.npz: 864-atom free EAM Al cluster, electrons
at 5000 K, 60 steps of 2 fs, list rebuilt every step).

The lattice forces are FP32 (Kahan), the detector and the model FP64.  Per
step: electron temperature within 1e-8 relative, integrated energies and
mean local lattice temperature within 1e-5, kinetic energy within 1e-6.
At the end: per-atom local temperatures within 1e-4 relative and local
densities exactly (neighbour counts).
"""
import os

import numpy as np
import pytest

from conftest import TABLES, load_case

pytestmark = pytest.mark.gpu


def test_ttm_matches_reference(omdg_lib):
    from objectmd_gb300 import inputs

    d = load_case("ttm_al_cluster")
    with omdg_lib.Context(0) as ctx:
        ctx.set_box(d["box_lo"], d["box_hi"], (False, False, False))
        ctx.set_atoms(d["x0"], d["v0"], masses=[inputs.md_mass("aluminum")], znum=[13.0])
        ctx.add_eam(os.path.join(TABLES, "eam.aluminum5000"))
        ctx.set_neighbor(0.3, 1)
        ctx.set_timestep(float(d["dt"]))
        ctx.set_ttm(os.path.join(TABLES, "ttm.aluminum"), float(d["atom_volume"]), float(d["te0"]), 0.0)
        rows, kin = [], []
        for k in range(int(d["steps"])):
            ctx.step(1)
            s = ctx.ttm_state()
            rows.append((k + 1, s["electron_temperature"], s["int_een"], s["int_aen"], s["lattice_temperature"]))
            kin.append(ctx.ledger()["kinetic"])
        loc = ctx.local_thermo()
    rows = np.array(rows)
    ref = d["ttm"]
    np.testing.assert_allclose(rows[:, 1], ref[:, 1], rtol=1e-8)
    np.testing.assert_allclose(rows[:, 2:], ref[:, 2:], rtol=1e-5, atol=1e-9)
    np.testing.assert_allclose(kin, d["ledger"][1:1 + len(kin), 1], rtol=1e-6)
    np.testing.assert_allclose(loc["temperature"], d["local_temp"], rtol=1e-4)
    np.testing.assert_array_equal(loc["density"], d["local_dens"])
