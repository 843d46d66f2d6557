"""FP64 restatement of the atom-centred neural surrogate for Tersoff Si.

Test infrastructure (the oracle): tests/ use it to check the GPU descriptor,
network, force and training kernels.  The product never imports it.

The reference has no neural potential; the method restated here is the
Behler-Parrinello atom-centred network (J. Behler, M. Parrinello, PRL 98,
146401 (2007); J. Behler, J. Chem. Phys. 134, 074106 (2011)):

  f_c(r)   = 1                                              r <= rin
           = 0.5 (cos(pi (r - rin) / (rc - rin)) + 1)        rin < r < rc
             (rin = 0 by default; rin = R - D, rc = R + D is Tersoff's own
             switch, tersoff.h:183)
  G2_k(i)  = sum_j exp(-eta_k (r_ij - Rs_k)^2) f_c(r_ij)     (16 radial)
  G5_m(i)  = 2^(1-zeta_m) sum_{j<k} (1 + lambda_m cos theta_jik)^zeta_m
             exp(-eta_m (r_ij^2 + r_ik^2)) f_c(r_ij) f_c(r_ik)  (16 angular)
  E_i      = w3 . tanh(W2 tanh(W1 (G_i - mu)/sigma + b1) + b2) + b3
  F        = -dE/dx through the descriptor Jacobian.

Training loss per batch (energies per atom of each configuration, forces per
component):
  L = wE mean_c ((E_c - E_c^ref) / N_c)^2 + wF mean_(k,a) (F_ka - F_ka^ref)^2
whose force term needs the gradient of u_i . v_i with u_i = dE_i/dG_i (the
"double backward" through the network), derived analytically below.
"""
import numpy as np

RC = 3.2
N_RAD = 16
N_ANG = 16
N_DESC = N_RAD + N_ANG
HIDDEN = 64


def descriptor_params():
    """Radial centres 1.6..3.2 A (eta from the spacing); angular (zeta, lambda, eta)."""
    rs = np.linspace(1.6, RC, N_RAD)
    h = rs[1] - rs[0]
    eta_r = np.full(N_RAD, 1.0 / (2.0 * h * h))
    zeta = np.array([1.0, 2.0, 4.0, 8.0])
    lam = np.array([1.0, -1.0])
    eta_a = np.array([0.0, 0.3])
    ang = np.array([(z, l, e) for e in eta_a for z in zeta for l in lam])
    return {"rs": rs, "eta_r": eta_r, "zeta": ang[:, 0], "lam": ang[:, 1], "eta_a": ang[:, 2], "rc": RC}


def fc(r, rc, rin=0.0):
    t = np.pi * (np.maximum(r, rin) - rin) / (rc - rin)
    return 0.5 * (np.cos(t) + 1.0)


def dfc(r, rc, rin=0.0):
    t = np.pi * (np.maximum(r, rin) - rin) / (rc - rin)
    return -0.5 * np.pi / (rc - rin) * np.sin(t)


def neighbours(x, lo, hi, rc=RC):
    """Minimum-image neighbour lists within rc (box >= 2 rc on every axis)."""
    L = np.asarray(hi) - np.asarray(lo)
    n = len(x)
    out = []
    for i in range(n):
        d = x - x[i]
        d -= np.round(d / L) * L
        r = np.sqrt((d * d).sum(1))
        js = np.nonzero((r < rc) & (np.arange(n) != i))[0]
        out.append([(int(j), d[j]) for j in js])  # d = x_j - x_i (image)
    return out


def descriptors(x, lo, hi, p):
    """G (n x 32) and the Jacobian: jac[i] = list of (j, dG_i/dx_j (32 x 3));
    dG_i/dx_i = -sum of the neighbour blocks (translation invariance)."""
    rc, rin = p["rc"], p.get("rin", 0.0)
    nb = neighbours(x, lo, hi, rc)
    n = len(x)
    G = np.zeros((n, N_DESC))
    jac = []
    for i in range(n):
        blocks = {}
        for j, d in nb[i]:
            blocks.setdefault(j, np.zeros((N_DESC, 3)))
        for j, d in nb[i]:
            r = np.linalg.norm(d)
            e = d / r
            g = np.exp(-p["eta_r"] * (r - p["rs"]) ** 2)
            G[i, :N_RAD] += g * fc(r, rc, rin)
            dg = g * (dfc(r, rc, rin) - 2.0 * p["eta_r"] * (r - p["rs"]) * fc(r, rc, rin))  # dG/dr
            blocks[j][:N_RAD] += np.outer(dg, e)
        m = len(nb[i])
        for a in range(m):
            ja, da = nb[i][a]
            ra = np.linalg.norm(da)
            for b in range(a + 1, m):
                jb, db = nb[i][b]
                rb = np.linalg.norm(db)
                cos = da @ db / (ra * rb)
                z, lam, eta = p["zeta"], p["lam"], p["eta_a"]
                base = 1.0 + lam * cos
                pw = np.where(base > 0, base, 0.0) ** z
                dpw = np.where(base > 0, z * np.where(base > 0, base, 1.0) ** (z - 1.0), 0.0) * lam
                ex = np.exp(-eta * (ra * ra + rb * rb))
                fa, fb = fc(ra, rc, rin), fc(rb, rc, rin)
                pref = 2.0 ** (1.0 - z)
                G[i, N_RAD:] += pref * pw * ex * fa * fb
                # derivatives w.r.t. ra, rb, cos
                d_ra = pref * pw * ex * fb * (dfc(ra, rc, rin) - 2.0 * eta * ra * fa)
                d_rb = pref * pw * ex * fa * (dfc(rb, rc, rin) - 2.0 * eta * rb * fb)
                d_cos = pref * dpw * ex * fa * fb
                ea, eb = da / ra, db / rb
                dcos_da = (eb - cos * ea) / ra  # d cos / d x_ja
                dcos_db = (ea - cos * eb) / rb
                blocks[ja][N_RAD:] += np.outer(d_ra, ea) + np.outer(d_cos, dcos_da)
                blocks[jb][N_RAD:] += np.outer(d_rb, eb) + np.outer(d_cos, dcos_db)
        jac.append(blocks)
    return G, jac


def init_model(seed, mu, sigma, e_mean):
    rng = np.random.default_rng(seed)
    w = {
        "W1": rng.normal(0.0, 1.0 / np.sqrt(N_DESC), (HIDDEN, N_DESC)),
        "b1": np.zeros(HIDDEN),
        "W2": rng.normal(0.0, 1.0 / np.sqrt(HIDDEN), (HIDDEN, HIDDEN)),
        "b2": np.zeros(HIDDEN),
        "w3": rng.normal(0.0, 1.0 / np.sqrt(HIDDEN), HIDDEN),
        "b3": np.array(e_mean),
    }
    return w, {"mu": np.asarray(mu, float), "sigma": np.asarray(sigma, float)}


def forward_backward(w, norm, G):
    """Per-atom energies and u = dE_i/dG_i (G in raw units)."""
    g = (G - norm["mu"]) / norm["sigma"]
    a1 = np.tanh(g @ w["W1"].T + w["b1"])
    a2 = np.tanh(a1 @ w["W2"].T + w["b2"])
    E = a2 @ w["w3"] + w["b3"]
    d2 = w["w3"] * (1.0 - a2 * a2)
    d1 = (d2 @ w["W2"]) * (1.0 - a1 * a1)
    u = (d1 @ w["W1"]) / norm["sigma"]
    return E, u


def forces(jac, u):
    n = len(u)
    F = np.zeros((n, 3))
    for i, blocks in enumerate(jac):
        for j, B in blocks.items():
            t = B.T @ u[i]  # dE_i/dx_j
            F[j] -= t
            F[i] += t  # dG_i/dx_i = -sum_j blocks
    return F


def predict(w, norm, x, lo, hi, p):
    G, jac = descriptors(x, lo, hi, p)
    E, u = forward_backward(w, norm, G)
    return E, forces(jac, u), G


def loss_and_grad(w, norm, batch, wE, wF, per_atom=False):
    """batch: list of (G, jac, E_ref, F_ref) with E_ref the total energy (or,
    per_atom, the per-atom energies: energy term wE mean_i (E_i - E_ref_i)^2).
    Returns L and dL/dw (analytic, including the double backward of the
    force term)."""
    grads = {k: np.zeros_like(v, dtype=float) for k, v in w.items()}
    L = 0.0
    nconf = len(batch)
    ncomp = sum(3 * len(b[0]) for b in batch)
    for G, jac, Eref, Fref in batch:
        n = len(G)
        E, u = forward_backward(w, norm, G)
        F = forces(jac, u)
        if per_atom:
            r = E - Eref
            L += wE * (r * r).sum() / (ncomp / 3)
            e_w = (2.0 * wE * r / (ncomp / 3))[:, None]
        else:
            de = (E.sum() - Eref) / n
            L += wE * de * de / nconf
            e_w = 2.0 * wE * de / (n * nconf)         # dL/dE_i
        res = F - Fref
        L += wF * (res * res).sum() / ncomp
        rho = 2.0 * wF * res / ncomp              # dL/dF_k
        # v_i = dL/du_i = sum_s J_is (rho_i - rho_j)
        v = np.zeros_like(u)
        for i, blocks in enumerate(jac):
            for j, B in blocks.items():
                v[i] += B @ (rho[i] - rho[j])
        g = (G - norm["mu"]) / norm["sigma"]
        vt = v / norm["sigma"]
        z1 = g @ w["W1"].T + w["b1"]
        a1 = np.tanh(z1)
        s1 = 1.0 - a1 * a1
        z2 = a1 @ w["W2"].T + w["b2"]
        a2 = np.tanh(z2)
        s2 = 1.0 - a2 * a2
        dz1 = vt @ w["W1"].T
        da1 = s1 * dz1
        dz2 = da1 @ w["W2"].T
        da2 = s2 * dz2
        d2 = w["w3"] * s2
        r2 = w["w3"] * dz2 * (-2.0 * a2 * s2)
        z2s = e_w * d2 + r2
        d1 = (d2 @ w["W2"]) * s1
        r1 = (r2 @ w["W2"]) * s1 + (d2 @ w["W2"]) * dz1 * (-2.0 * a1 * s1)
        z1s = e_w * d1 + r1
        grads["w3"] += (e_w * a2 + da2).sum(0)
        grads["b3"] += float(np.sum(e_w * np.ones((n, 1)))) if per_atom else e_w * n
        grads["W2"] += z2s.T @ a1 + d2.T @ da1
        grads["b2"] += z2s.sum(0)
        grads["W1"] += z1s.T @ g + d1.T @ vt
        grads["b1"] += z1s.sum(0)
    return L, grads


def loss_only(w, norm, batch, wE, wF, per_atom=False):
    L = 0.0
    nconf = len(batch)
    ncomp = sum(3 * len(b[0]) for b in batch)
    for G, jac, Eref, Fref in batch:
        E, u = forward_backward(w, norm, G)
        F = forces(jac, u)
        if per_atom:
            L += wE * ((E - Eref) ** 2).sum() / (ncomp / 3)
        else:
            de = (E.sum() - Eref) / len(G)
            L += wE * de * de / nconf
        L += wF * ((F - Fref) ** 2).sum() / ncomp
    return L


def bf16(a):
    """Round to BF16 (nearest even) and return as float64."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def forward_backward_tc(w, norm, G):
    """forward_backward with the tensor-core kernel's rounding: the MMA
    operands (normalised input, a1, delta2, delta1 and the weights) in BF16,
    everything else in full precision."""
    isig = (1.0 / np.asarray(norm["sigma"], dtype=np.float32)).astype(np.float32)
    gt = bf16((np.asarray(G, np.float32) - np.asarray(norm["mu"], np.float32)) * isig)
    W1, W2 = bf16(w["W1"]), bf16(w["W2"])
    a1 = np.tanh(gt @ W1.T + w["b1"])
    a2 = np.tanh(bf16(a1) @ W2.T + w["b2"])
    E = a2 @ w["w3"] + w["b3"]
    d2 = bf16(w["w3"] * (1.0 - a2 * a2))
    d1 = bf16((d2 @ W2) * (1.0 - a1 * a1))
    u = (d1 @ W1) * isig
    return E, u


def unflatten(p):
    """The flat FP32 parameter vector of the GPU library as a weight dict."""
    p = np.asarray(p, dtype=np.float64)
    o = 0
    out = {}
    for name, shape in (("W1", (HIDDEN, N_DESC)), ("b1", (HIDDEN,)), ("W2", (HIDDEN, HIDDEN)), ("b2", (HIDDEN,)),
                        ("w3", (HIDDEN,)), ("b3", ())):
        size = int(np.prod(shape)) if shape else 1
        out[name] = p[o:o + size].reshape(shape) if shape else np.array(p[o])
        o += size
    return out


def flatten(w):
    return np.concatenate([np.ravel(w[k]) for k in ("W1", "b1", "W2", "b2", "w3", "b3")]).astype(np.float32)
