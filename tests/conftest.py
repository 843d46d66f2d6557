import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLD = os.path.join(ROOT, "tests", "golden")
TABLES = os.path.join(GOLD, "tables")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 and the sm_103a library")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle as oc

    oc.build()
    return oc


@pytest.fixture(scope="session")
def omdg_lib():
    from objectmd_gb300 import build as b

    b.build()
    from objectmd_gb300 import omdg

    return omdg


def load_case(name):
    d = dict(np.load(os.path.join(GOLD, name + ".npz")))
    from objectmd_gb300 import inputs

    x0, v0, types, box, periodic = inputs.read_import(os.path.join(GOLD, name + ".dat"))
    d["x0"], d["v0"], d["types0"], d["periodic"] = x0, v0, types, periodic
    return d


def nbr_set(off, j, code):
    out = set()
    for i in range(len(off) - 1):
        for k in range(off[i], off[i + 1]):
            c = int(code[k])
            out.add((i, int(j[k]), c % 3 - 1, (c // 3) % 3 - 1, c // 9 - 1))
    return out
