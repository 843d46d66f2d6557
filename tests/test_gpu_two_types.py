"""Two atom types with EAM on one of them (the combination of the
reference's test/two_elements/two.cpp): EAM platinum between Pt atoms and
the reference's Ar-Pt table (tables/pair.ar-pt.zbl) between one Ar atom and
Pt, against the reference's static forces and per-atom energies
(tests/golden/ar_pt_slab.npz): the Ar atom 1.2-2.8 A above a Pt slab
(periodic x/y, free z).  With two types the EAM pass runs the general
kernels (k_eam_density, k_eam_force), not the single-type fast passes.

Tolerances: norm-wise relative force error <= 1e-5, components within
1e-5 max|f| + 1e-6 eV/A, per-atom energies within 2e-6 eV + 2e-6 relative
(FP32 splines and compensated sums against the reference's FP64).
"""
import os

import numpy as np
import pytest

from conftest import GOLD, TABLES

pytestmark = pytest.mark.gpu


def test_eam_beside_a_second_atom_type_matches_reference(omdg_lib):
    from objectmd_gb300 import inputs

    d = dict(np.load(os.path.join(GOLD, "ar_pt_slab.npz")))
    for k, h in enumerate(d["heights"]):
        with omdg_lib.Context(0) as ctx:
            ctx.set_box(d["box_lo"], d["box_hi"], (True, True, False))
            ctx.set_atoms(d["x0"][k], None, types=d["types"],
                          masses=[inputs.md_mass("platinum"), inputs.md_mass("argon")], znum=[78.0, 18.0])
            ctx.add_eam(os.path.join(TABLES, "eam.platinum"), 0, 0)
            ctx.add_pair_table(os.path.join(TABLES, "pair.ar-pt.zbl"), ta=1, tb=0)
            ctx.set_neighbor(0.3, 1)
            ctx.compute_forces()
            st = ctx.get_state()
        f, fref = st["f"], d["f"][k]
        rel = np.linalg.norm(f - fref) / np.linalg.norm(fref)
        assert rel <= 1e-5, (h, rel)
        assert np.abs(f - fref).max() <= 1e-5 * np.abs(fref).max() + 1e-6, h
        eref = d["pot"][k]
        eerr = np.abs(st["pot"] - eref) / (2e-6 + 2e-6 * np.abs(eref))
        assert eerr.max() <= 1.0, (h, np.abs(st["pot"] - eref).max())
