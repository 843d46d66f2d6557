"""The device finite-difference heat solver (omdg_fdtd, csrc/fdtd.cu) against
the reference and the oracle, bit for bit.

- the three specs of tests/golden/fdtd_cases.npz (cell vectors printed by the
  reference's own FDTDSolver, src/omd/fdtd.cpp): every step equal;
- a 40 x 32 x 24 slab (30,720 cells) with per-layer symbols, a ranged
  surface source and conductivity and capacity blocks: 20 steps equal to the
  oracle (oracle/fdtd_oracle.py, pinned by the fixtures);
- errors: a '{...}' expression (muParser is not built), a block beyond the
  grid, a map of the wrong length.
"""
import os

import numpy as np
import pytest

from oracle import fdtd_oracle as fo

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "fdtd_cases.npz")


def run_device(omdg, spec):
    """A spec in the driver's format through omdg_fdtd; rows as run_spec."""
    g = None
    dims = symbol = None
    ext = []
    rows = []
    try:
        for line in spec.splitlines():
            parts = line.split(None, 1)
            if not parts:
                continue
            key, rest = parts[0], (parts[1] if len(parts) > 1 else "")
            if key == "dim":
                dims = [int(v) for v in rest.split()]
            elif key == "symbol":
                symbol = rest
            elif key == "map":
                g = omdg.FDTD(dims[0], dims[1], dims[2], symbol, rest.strip())
            elif key == "spacestep":
                g.set_spacestep(float(rest))
            elif key == "timestep":
                g.set_timestep(float(rest))
            elif key == "cell":
                g.set_cell(rest)
            elif key == "conductivity":
                g.set_conductivity(rest)
            elif key == "capacity":
                g.set_capacity(rest)
            elif key == "source":
                g.set_source(rest)
            elif key == "ext":
                i, v = rest.split()
                ext.append((int(i), float(v)))
            elif key == "steps":
                rows.append(g.vector())
                for _ in range(int(rest)):
                    if ext:
                        e = np.zeros(g.dim)
                        for i, v in ext:
                            e[i] = v
                        g.set_ext(e)
                    g.step(1)
                    rows.append(g.vector())
    finally:
        if g is not None:
            g.close()
    return np.array(rows)


@pytest.mark.parametrize("name", ["slab3d", "flat2d_cleared", "edges2d"])
def test_device_equals_the_reference(omdg_lib, name):
    d = np.load(GOLD)
    rows = run_device(omdg_lib, str(d[name + "_spec"]))
    ref = d[name + "_rows"]
    assert rows.shape == ref.shape
    assert np.array_equal(rows, ref), np.abs(rows - ref).max()


def big_slab_spec(nx=40, ny=32, nz=24, steps=20):
    def cell(i, j, k):
        if k == 0:
            return "t"
        if k == nz - 1:
            return "b"
        return "a"

    cmap = "".join(cell(i, j, k) for k in range(nz) for j in range(ny) for i in range(nx))
    return "\n".join([
        "dim %d %d %d" % (nx, ny, nz),
        "symbol a pppp++ t pppp-+ b pppp+-",
        "map " + cmap,
        "spacestep 5.0",
        "timestep 0.2",
        "cell * 300 @ 10,10,0,30,25,3=2000",
        "conductivity a 4.0 t 2.0 b 8.0 @ 0,0,10,%d,%d,12=0.25" % (nx - 1, ny - 1),
        "capacity * 3.0 @ 20,0,5,%d,%d,20=1.5" % (nx - 1, ny - 1),
        "source t 400:0:12 @ 5,5,1=1000:3:8",
        "ext 12345 -50",
        "steps %d" % steps,
    ])


def test_device_equals_the_oracle_on_a_slab(omdg_lib):
    spec = big_slab_spec()
    ref = fo.run_spec(spec)
    rows = run_device(omdg_lib, spec)
    assert np.array_equal(rows, ref), np.abs(rows - ref).max()
    assert np.abs(rows[-1] - rows[0]).max() > 10.0  # the field moved


def test_errors_are_reported(omdg_lib):
    with omdg_lib.FDTD(4, 4, 1, "a pppp", "a" * 16) as g:
        with pytest.raises(omdg_lib.OMDGError) as ei:
            g.set_source("a {2*t}")
        assert ei.value.code == omdg_lib.OMDG_EINVAL and "muParser" in str(ei.value)
        with pytest.raises(omdg_lib.OMDGError) as ei:
            g.set_conductivity("@ 0,0,0,4,4,0=1")
        assert "out of range" in str(ei.value)
    with pytest.raises(omdg_lib.OMDGError) as ei:
        omdg_lib.FDTD(4, 4, 1, "a pppp", "a" * 15)
    assert "map string count" in str(ei.value)
