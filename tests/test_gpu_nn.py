"""The neural surrogate on the GPU against the FP64 oracle (oracle/nn_oracle.py).

- descriptors (FP32 kernels) vs the oracle: 2e-5 relative to each
  descriptor's scale;
- the tensor-core network (BF16 operands, FP32 accumulation): against the
  oracle evaluated with the same BF16 rounding points, 95 % of per-atom
  energies within 1e-4 eV (all within 3e-3: an activation at a BF16 rounding
  boundary may round the other way) and forces within 2e-3 norm-wise; within
  BF16 accuracy (1e-2 relative) of the plain FP64 oracle;
- the training gradient (FP32 kernels, energy + force loss, double backward)
  within 1e-3 norm-wise of the oracle's analytic gradient;
- the MD force path (descriptors from the Verlet list) equal to the trainer's
  prediction, and the Tersoff fallback equal to plain Tersoff (to the last
  bits of the force sums) when every atom leaves the training range.
"""
import os

import numpy as np
import pytest

from conftest import TABLES

pytestmark = pytest.mark.gpu

TERSOFF = os.path.join(TABLES, "tersoff.silicon27")
TP = dict(A=3264.7, B=95.373, lambda1=3.2394, lambda2=1.3258, lambda3=1.3258, beta=0.33675, n=22.956, c=4.8381,
          d=2.0417, h=0.0, R=2.7, D=0.15)


@pytest.fixture(scope="module")
def dataset(oracle_lib):
    """Four 64-atom diamond cells with Tersoff energies and forces from the C oracle."""
    from objectmd_gb300 import inputs
    from oracle import nn_oracle as nn

    oc = oracle_lib
    p = nn.descriptor_params()
    confs = []
    for k in range(4):
        x, v, (lo, hi) = inputs.diamond_silicon(ncell=2, a=5.431, sigma=0.08 + 0.03 * k, temp=300.0,
                                                seed_pos=20 + k, seed_vel=30 + k)
        box = oc.make_box(lo, hi, (1, 1, 1))
        f, e, _ = oc.tersoff(box, x, oc.neighbors(box, x, 3.15), oc.TersoffParam(**TP))
        G, jac = nn.descriptors(x, lo, hi, p)
        confs.append(dict(x=x, lo=lo, hi=hi, E=e.sum(), Ea=e, F=f, G=G, jac=jac))
    return confs


def make_network(omdg, confs, seed=3, desc=None):
    from oracle import nn_oracle as nn

    net = omdg.Network(0)
    if desc is not None:
        net.set_descriptors(*desc)
    net.set_dataset([len(c["x"]) for c in confs], np.concatenate([c["x"] for c in confs]),
                    [np.asarray(c["hi"]) - np.asarray(c["lo"]) for c in confs], [c["E"] for c in confs],
                    np.concatenate([c["F"] for c in confs]))
    net.normalize_from_dataset()
    norm = net.normalization()
    w, _ = nn.init_model(seed, norm["mu"], norm["sigma"], -4.6)
    net.set_weights(nn.flatten(w))
    w = nn.unflatten(net.weights())
    return net, w, {"mu": norm["mu"].astype(float), "sigma": norm["sigma"].astype(float)}


def test_descriptors_match_oracle(omdg_lib, dataset):
    net, _, _ = make_network(omdg_lib, dataset)
    G = net.descriptors()
    net.close()
    ref = np.concatenate([c["G"] for c in dataset])
    scale = np.abs(ref).max(0) + 1e-12
    assert (np.abs(G - ref) / scale).max() < 2e-5


def test_tensor_core_network_matches_oracle(omdg_lib, dataset):
    from oracle import nn_oracle as nn

    net, w, norm = make_network(omdg_lib, dataset)
    E, F = net.predict(0, len(dataset))
    net.close()
    Et, Ft, E64, F64 = [], [], [], []
    for c in dataset:
        e, u = nn.forward_backward_tc(w, norm, c["G"])
        Et.append(e)
        Ft.append(nn.forces(c["jac"], u))
        e, u = nn.forward_backward(w, norm, c["G"])
        E64.append(e)
        F64.append(nn.forces(c["jac"], u))
    Et, Ft, E64, F64 = map(np.concatenate, (Et, Ft, E64, F64))
    # same rounding points: agreement to FP32 accumulation order, except where
    # an activation sits at a BF16 rounding boundary and rounds the other way
    # (one BF16 ulp, 2^-8 relative, in one activation)
    assert np.mean(np.abs(E - Et) > 1e-4) < 0.05
    assert np.abs(E - Et).max() < 3e-3
    assert np.linalg.norm(F - Ft) / np.linalg.norm(Ft) < 2e-3
    assert np.abs(E - E64).max() < 1e-2 * np.abs(E64).max()
    assert np.linalg.norm(F - F64) / np.linalg.norm(F64) < 1e-2


@pytest.mark.parametrize("per_atom", [False, True])
def test_training_gradient_matches_oracle(omdg_lib, dataset, per_atom):
    from oracle import nn_oracle as nn

    net, w, norm = make_network(omdg_lib, dataset)
    if per_atom:
        net.set_atom_energies(np.concatenate([c["Ea"] for c in dataset]))
    wE, wF = 1.0, 2.0
    loss, g = net.gradient(0, 3, wE, wF)
    net.close()
    batch = [(c["G"], c["jac"], c["Ea"] if per_atom else c["E"], c["F"]) for c in dataset[:3]]
    L, grad = nn.loss_and_grad(w, norm, batch, wE, wF, per_atom)
    ref = nn.flatten(grad).astype(np.float64)
    assert abs(loss - L) < 1e-4 * abs(L)
    assert np.linalg.norm(g - ref) / np.linalg.norm(ref) < 1e-3


def surrogate_context(omdg, c, model, fallback):
    from objectmd_gb300 import inputs

    ctx = omdg.Context(0)
    ctx.set_box(c["lo"], c["hi"])
    ctx.set_atoms(c["x"], np.zeros_like(c["x"]), masses=[inputs.md_mass("silicon")], znum=[14.0])
    if model:
        ctx.add_nn(model, TERSOFF if fallback else None)
    else:
        ctx.add_tersoff(TERSOFF)
    ctx.set_neighbor(0.3, 1)
    ctx.compute_forces()
    return ctx


def test_md_path_matches_prediction(omdg_lib, dataset, tmp_path):
    net, w, norm = make_network(omdg_lib, dataset)
    model = str(tmp_path / "model.nn")
    net.save(model)
    E, F = net.predict(1, 1)
    net.close()
    with surrogate_context(omdg_lib, dataset[1], model, True) as ctx:
        st = ctx.get_state()
        assert ctx.nn_fallback_atoms() == 0
    assert np.abs(st["pot"] - E).max() < 2e-3
    assert np.linalg.norm(st["f"] - F) / np.linalg.norm(F) < 2e-3


def test_md_path_with_another_angular_layout(omdg_lib, dataset, tmp_path):
    """The MD kernels take zeta and lambda as constants when the angular set
    has the default layout (zeta 1, 2, 4, 8 in pairs, lambda +1 then -1).
    Here lambda comes -1 first and zeta 3 stands in for 4, so the MD path
    runs its general kernels; they too equal the trainer's prediction."""
    from oracle import nn_oracle as nn

    p = nn.descriptor_params()
    zeta = np.where(p["zeta"] == 4, 3, p["zeta"]).astype(np.int32)
    desc = (p["rs"], p["eta_r"], zeta, -np.asarray(p["lam"]), p["eta_a"])
    net, _, _ = make_network(omdg_lib, dataset, desc=desc)
    model = str(tmp_path / "layout.nn")
    net.save(model)
    E, F = net.predict(1, 1)
    net.close()
    with surrogate_context(omdg_lib, dataset[1], model, True) as ctx:
        st = ctx.get_state()
        assert ctx.nn_fallback_atoms() == 0
    assert np.abs(st["pot"] - E).max() < 2e-3
    assert np.linalg.norm(st["f"] - F) / np.linalg.norm(F) < 2e-3


def test_fused_descriptor_network_kernel_is_the_same(omdg_lib, dataset, tmp_path):
    """Descriptors computed inside the tensor-core network kernel (launch key
    nn_fused) against the separate descriptor kernel: the same functions on
    the same rows, so forces, energies and fallback flags agree bit for bit."""
    from objectmd_gb300 import inputs

    net, _, norm = make_network(omdg_lib, dataset)
    model = str(tmp_path / "model.nn")
    net.save(model)
    net.close()
    c = dataset[3]
    out = []
    for fused in (0, 1):
        with omdg_lib.Context(0) as ctx:
            ctx.set_box(c["lo"], c["hi"])
            ctx.set_atoms(c["x"], np.zeros_like(c["x"]), masses=[inputs.md_mass("silicon")], znum=[14.0])
            ctx.add_nn(model, TERSOFF)
            ctx.set_neighbor(0.3, 1)
            ctx.set_launch("nn_fused", fused)
            ctx.compute_forces()
            out.append((ctx.get_state(), ctx.nn_fallback_atoms()))
    (a, na), (b, nb) = out
    assert na == nb
    for k in ("f", "pot", "vir"):
        assert np.array_equal(a[k], b[k]), k


def test_fallback_is_plain_tersoff(omdg_lib, dataset, tmp_path):
    net, w, norm = make_network(omdg_lib, dataset)
    # a training range no atom lies in: every atom falls back
    net.set_normalization(norm["mu"], norm["sigma"], norm["mu"] + 1e9, norm["mu"] + 2e9)
    model = str(tmp_path / "narrow.nn")
    net.save(model)
    net.close()
    c = dataset[2]
    with surrogate_context(omdg_lib, c, model, True) as ctx:
        st = ctx.get_state()
        assert ctx.nn_fallback_atoms() == len(c["x"])
    with surrogate_context(omdg_lib, c, None, False) as ctx:
        ref = ctx.get_state()
    # same Tersoff kernel; the surrogate's longer list (3.5 vs 3.15 A) adds
    # zero-valued slots to the Kahan gather, which can move the last bit
    np.testing.assert_allclose(st["f"], ref["f"], rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(st["pot"], ref["pot"], rtol=1e-6, atol=1e-6)


def test_tersoff_switch_descriptors_and_md_path(omdg_lib, tmp_path):
    """Descriptor cutoff switched over Tersoff's [R - D, R + D] (rin = 2.55,
    rc = 2.85): the trainer's descriptors match the oracle with bonds on both
    sides of rin, the switch round-trips through the model file, and the MD
    force path equals the trainer's prediction."""
    from objectmd_gb300 import inputs
    from oracle import nn_oracle as nn

    p = dict(nn.descriptor_params(), rc=2.85, rin=2.55)
    x, v, (lo, hi) = inputs.diamond_silicon(ncell=2, a=5.431, sigma=0.15, temp=300.0, seed_pos=13, seed_vel=14)
    Gref, _ = nn.descriptors(x, lo, hi, p)
    net = omdg_lib.Network(0)
    net.set_cutoff(2.85, 2.55)
    box = np.asarray(hi) - np.asarray(lo)
    net.set_dataset([len(x)], x, [box], [-4.6 * len(x)], np.zeros_like(x))
    G = net.descriptors()
    scale = np.abs(Gref).max(0) + 1e-12
    assert (np.abs(G - Gref) / scale).max() < 2e-5
    net.normalize_from_dataset()
    norm = net.normalization()
    # the dataset is this one cell: widen its range so that the MD kernels'
    # FP32 rounding cannot put an extreme atom outside it
    pad = 0.01 * (norm["gmax"] - norm["gmin"]) + 1e-6
    net.set_normalization(norm["mu"], norm["sigma"], norm["gmin"] - pad, norm["gmax"] + pad)
    w, _ = nn.init_model(5, norm["mu"], norm["sigma"], -4.6)
    net.set_weights(nn.flatten(w))
    model = str(tmp_path / "switch.nn")
    net.save(model)
    E, F = net.predict(0, 1)
    net.close()
    rin = [ln.split()[1] for ln in open(model) if ln.startswith("rin ")]
    assert len(rin) == 1 and np.float32(rin[0]) == np.float32(2.55)
    c = dict(x=x, lo=lo, hi=hi)
    with surrogate_context(omdg_lib, c, model, True) as ctx:
        st = ctx.get_state()
        assert ctx.nn_fallback_atoms() == 0
    assert np.abs(st["pot"] - E).max() < 2e-3
    assert np.linalg.norm(st["f"] - F) / np.linalg.norm(F) < 2e-3
    with pytest.raises(omdg_lib.OMDGError):
        with omdg_lib.Network(0) as bad:
            bad.set_cutoff(2.5, 2.6)
