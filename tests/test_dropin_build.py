"""The compiled drop-in (objectmd_gb300/dropin/gpu_integrator.h) in the
reference's own example application.

oracle/ref/Makefile compiles test/example/example.cpp unmodified twice where
the Object-MD sources are present: as shipped, and with
oracle/ref/dropin_prelude.h force-included, which makes its
`SetIntegrator(new MDIntegrator)` construct the GPU integrator, linked with
libomdg.so.  Here (a host without a GPU) the swapped program must reach the
library: the reference builds its crystal, registers the EAM kernel, and the
GPU integrator's Init stops at omdg_create with the library's error through
the reference's die().  On a host with a GB300 it runs the 200 steps.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "oracle", "_ref", "example_gpuintegrator")
TABLES = os.path.join(ROOT, "tests", "golden", "tables")


@pytest.mark.skipif(not os.path.exists(BIN), reason="built only where the Object-MD sources are present")
def test_reference_example_runs_through_the_gpu_integrator(tmp_path):
    env = dict(os.environ, OMD_TABLE=TABLES)
    subprocess.run([BIN], cwd=tmp_path, env=env, capture_output=True, timeout=600)
    log = (tmp_path / "run.log").read_text()
    assert "added atoms: name=FCC" in log and "n_atom=1000" in log
    assert "GB300 VERLET INTEGRATOR" in log  # the integrator the application constructed
    if "GPUIntegrator: omdg_create" in log:
        assert "OMDG_ECUDA" in log or "no GB300" in log or "CUDA" in log
    else:
        traj = (tmp_path / "traj.dat").read_text().splitlines()
        assert len(traj) == 200
