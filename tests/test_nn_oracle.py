"""The FP64 neural-surrogate oracle pinned by finite differences (CPU only):
descriptor Jacobian, forces = -dE/dx, and the analytic training gradient
(energy + force loss, including the double backward through the network)."""
import numpy as np
import pytest

from oracle import nn_oracle as nn


@pytest.fixture(scope="module")
def small_system():
    from objectmd_gb300 import inputs

    x, v, (lo, hi) = inputs.diamond_silicon(ncell=2, a=5.431, sigma=0.12, temp=300.0, seed_pos=11, seed_vel=12)
    p = nn.descriptor_params()
    G, jac = nn.descriptors(x, lo, hi, p)
    return x, lo, hi, p, G, jac


def test_descriptor_jacobian_matches_finite_differences(small_system):
    x, lo, hi, p, G, jac = small_system
    h = 1e-6
    for atom in (0, 13):
        for q in range(3):
            xp = x.copy()
            xp[atom, q] += h
            xm = x.copy()
            xm[atom, q] -= h
            dG = (nn.descriptors(xp, lo, hi, p)[0] - nn.descriptors(xm, lo, hi, p)[0]) / (2 * h)
            ana = np.zeros_like(G)
            for i, blocks in enumerate(jac):
                for j, B in blocks.items():
                    if j == atom:
                        ana[i] += B[:, q]
                    if i == atom:
                        ana[i] -= B[:, q]
            assert np.abs(dG - ana).max() < 1e-6 * max(1.0, np.abs(ana).max())


def test_forces_are_energy_gradients(small_system):
    x, lo, hi, p, G, jac = small_system
    w, norm = nn.init_model(3, G.mean(0), G.std(0) + 1e-3, -4.6)
    E, F, _ = nn.predict(w, norm, x, lo, hi, p)
    h = 1e-6
    for atom in (2, 40):
        for q in range(3):
            xp = x.copy()
            xp[atom, q] += h
            xm = x.copy()
            xm[atom, q] -= h
            ep = nn.predict(w, norm, xp, lo, hi, p)[0].sum()
            em = nn.predict(w, norm, xm, lo, hi, p)[0].sum()
            assert abs(-(ep - em) / (2 * h) - F[atom, q]) < 1e-6
    assert np.abs(F.sum(0)).max() < 1e-10  # no net force


@pytest.mark.parametrize("per_atom", [False, True])
def test_training_gradient_matches_finite_differences(small_system, per_atom):
    x, lo, hi, p, G, jac = small_system
    rng = np.random.default_rng(5)
    w, norm = nn.init_model(4, G.mean(0), G.std(0) + 1e-3, -4.6)
    Fref = rng.normal(0, 0.5, (len(x), 3))
    Eref = -4.6 + rng.normal(0, 0.1, len(x)) if per_atom else -4.6 * len(x) + 0.3
    batch = [(G, jac, Eref, Fref)]
    wE, wF = 1.0, 10.0
    L, grad = nn.loss_and_grad(w, norm, batch, wE, wF, per_atom)
    assert abs(L - nn.loss_only(w, norm, batch, wE, wF, per_atom)) < 1e-12
    h = 1e-6
    for name, idx in (("W1", (5, 7)), ("W1", (60, 31)), ("b1", (9,)), ("W2", (3, 50)), ("b2", (17,)),
                      ("w3", (11,)), ("b3", ())):
        wp = {k: np.array(v, dtype=float, copy=True) for k, v in w.items()}
        wm = {k: np.array(v, dtype=float, copy=True) for k, v in w.items()}
        wp[name][idx] += h
        wm[name][idx] -= h
        fd = (nn.loss_only(wp, norm, batch, wE, wF, per_atom) - nn.loss_only(wm, norm, batch, wE, wF, per_atom)) / (2 * h)
        ana = grad[name][idx]
        assert abs(fd - ana) < 1e-6 * max(1.0, abs(ana)), (name, idx, fd, ana)


def test_inner_switch_radius_gives_tersoffs_cutoff_and_its_jacobian():
    """rin = R - D, rc = R + D: f_c equals Tersoff's 1/2 - 1/2 sin(pi/2 (r - R)/D)
    (tersoff.h:183) and the descriptor Jacobian still matches finite
    differences, with bonds on both sides of rin."""
    from objectmd_gb300 import inputs

    R, D = 2.7, 0.15
    r = np.linspace(R - D, R + D, 101)
    np.testing.assert_allclose(nn.fc(r, R + D, R - D), 0.5 - 0.5 * np.sin(0.5 * np.pi * (r - R) / D), atol=1e-15)
    assert nn.fc(2.3, R + D, R - D) == 1.0 and nn.dfc(2.3, R + D, R - D) == 0.0
    x, v, (lo, hi) = inputs.diamond_silicon(ncell=2, a=5.431, sigma=0.15, temp=300.0, seed_pos=13, seed_vel=14)
    p = dict(nn.descriptor_params(), rc=R + D, rin=R - D)
    G, jac = nn.descriptors(x, lo, hi, p)
    L = np.asarray(hi) - np.asarray(lo)
    d = x[:, None] - x[None]
    d -= np.round(d / L) * L
    dist = np.sqrt((d * d).sum(-1))
    inside = (dist > R - D) & (dist < R + D)
    assert inside.sum() >= 4 and ((dist < R - D) & (dist > 0)).sum() > 100
    h = 1e-6
    atoms = sorted({int(np.nonzero(inside)[0][0]), int(np.nonzero(inside)[1][0]), 7})
    for atom in atoms:
        for q in range(3):
            xp = x.copy()
            xp[atom, q] += h
            xm = x.copy()
            xm[atom, q] -= h
            dG = (nn.descriptors(xp, lo, hi, p)[0] - nn.descriptors(xm, lo, hi, p)[0]) / (2 * h)
            ana = np.zeros_like(G)
            for i, blocks in enumerate(jac):
                for j, B in blocks.items():
                    if j == atom:
                        ana[i] += B[:, q]
                    if i == atom:
                        ana[i] -= B[:, q]
            assert np.abs(dG - ana).max() < 1e-6 * max(1.0, np.abs(ana).max())
