"""The shipped surrogate model and the descriptor sets the fitting script
makes keep the default angular layout: term m has zeta 2^((m >> 1) & 3)
and lambda +1 for even m, -1 for odd m.  The MD kernels specialise on that
layout (zeta and lambda as constants of the unrolled term loop) and run
general kernels for any other, so a model that left it would still be
correct but slower.  CPU only: the model file is text."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MODEL = os.path.join(ROOT, "objectmd_gb300", "models", "nn_tersoff_si.nn")

STD_ZETA = np.array([1 << ((m >> 1) & 3) for m in range(16)])
STD_LAM = np.array([-1.0 if m & 1 else 1.0 for m in range(16)])


def read_model(path):
    out = {}
    with open(path) as f:
        for line in f:
            key, *vals = line.split()
            if key in ("zeta", "lambda", "eta_a"):
                out[key] = np.array([float(v) for v in vals])
    return out


def test_shipped_model_has_the_default_angular_layout():
    m = read_model(MODEL)
    assert np.array_equal(m["zeta"], STD_ZETA)
    assert np.array_equal(m["lambda"], STD_LAM)


def test_fitting_descriptor_sets_have_the_default_angular_layout():
    sys.path.insert(0, ROOT)
    from objectmd_gb300 import nn_fit
    from oracle import nn_oracle as nn

    _, (_, _, zeta, lam, _) = nn_fit.switch_descriptors()
    assert np.array_equal(zeta, STD_ZETA) and np.array_equal(lam, STD_LAM)
    p = nn.descriptor_params()
    assert np.array_equal(p["zeta"], STD_ZETA) and np.array_equal(p["lam"], STD_LAM)
