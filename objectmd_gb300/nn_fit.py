"""Training set generation and fitting for the neural Tersoff surrogate.

The training set is plain-Tersoff MD run by this library: 512-atom diamond
cells (4^3 cells, a = 5.431 A), each trajectory held at its own temperature,
drawn uniformly from [300, 2500] K, by the Berendsen thermostat.  Every
trajectory is equilibrated, then sampled every 50 fs (50 steps of 1 fs).  The
labels are the Tersoff kernel's per-atom energies (E_i = 1/2 sum_j V_ij) and
forces.  Fitting runs on the
GPU through omdg_nn_train: descriptors, forward and backward passes, the
force-loss double backward and Adam are the library's own kernels.  Defaults:
the descriptors of switch_descriptors() (cutoff switched over Tersoff's own
[R - D, R + D]), 200 epochs, batches of 16 configurations, Adam with the
learning rate decaying from 1e-3 to 1e-5 (cosine), loss = per-atom energy MSE
+ force MSE.

    python -m objectmd_gb300.nn_fit --out objectmd_gb300/models/nn_tersoff_si.nn
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
TERSOFF = os.path.join(ROOT, "tests", "golden", "tables", "tersoff.silicon27")
MODEL = os.path.join(HERE, "models", "nn_tersoff_si.nn")


def generate(nconf=2000, per_traj=50, ncell=4, tmin=300.0, tmax=2500.0, every=50, equil=1000, dt=0.001, seed=7,
             device=0, log=None):
    """Tersoff MD snapshots: per-configuration atom counts, positions, box
    lengths, total energies and forces."""
    from objectmd_gb300 import inputs, omdg

    rng = np.random.default_rng(seed)
    ntraj = (nconf + per_traj - 1) // per_traj
    temps = rng.uniform(tmin, tmax, ntraj)
    natoms, xs, boxes, energies, forces, tlist, eatoms = [], [], [], [], [], [], []
    for k, T in enumerate(temps):
        x, v, (lo, hi) = inputs.diamond_silicon(ncell=ncell, a=5.431, sigma=0.03, temp=float(T),
                                                seed_pos=int(1000 + k), seed_vel=int(2000 + k))
        with omdg.Context(device) as ctx:
            ctx.set_box(lo, hi)
            ctx.set_atoms(x, v, masses=[inputs.md_mass("silicon")], znum=[14.0])
            ctx.add_tersoff(TERSOFF)
            ctx.set_neighbor(0.3, 0)
            ctx.set_timestep(dt)
            ctx.set_first_step_mode(False)
            ctx.set_thermostat(float(T), 0.1)
            ctx.step(equil)
            for s in range(min(per_traj, nconf - len(natoms))):
                ctx.step(every)
                st = ctx.get_state()
                natoms.append(len(x))
                xs.append(st["x"])
                boxes.append(np.asarray(hi) - np.asarray(lo))
                energies.append(float(st["pot"].sum()))
                eatoms.append(st["pot"])
                forces.append(st["f"])
                tlist.append(T)
        if log:
            log("trajectory %d/%d at %.0f K: %d configurations" % (k + 1, ntraj, T, len(natoms)))
    return {"natoms": np.array(natoms), "x": np.concatenate(xs), "box": np.array(boxes),
            "energy": np.array(energies), "forces": np.concatenate(forces), "temperature": np.array(tlist),
            "atom_energy": np.concatenate(eatoms)}


def switch_descriptors(r0=1.9, R=2.7, D=0.15):
    """Descriptor set fitted to Tersoff: the cutoff switched over Tersoff's own
    [R - D, R + D] (tersoff.h:183), 16 radial centres on [r0, R + D] with
    eta = 1 / (2 h^2) (h the spacing), the default angular terms.  Returns
    (cutoff, descriptors) as fit() takes them."""
    rs = np.linspace(r0, R + D, 16)
    h = rs[1] - rs[0]
    eta_r = np.full(16, 1.0 / (2.0 * h * h))
    ang = [(z, l, e) for e in (0.0, 0.3) for z in (1, 2, 4, 8) for l in (1.0, -1.0)]
    zeta = np.array([a[0] for a in ang], dtype=np.int32)
    lam = np.array([a[1] for a in ang])
    eta_a = np.array([a[2] for a in ang])
    return (R + D, R - D), (rs, eta_r, zeta, lam, eta_a)


def init_params(seed, e_mean):
    """Normal initialisation scaled by 1/sqrt(fan-in); the output bias starts
    at the mean per-atom energy."""
    rng = np.random.default_rng(seed)
    w1 = rng.normal(0.0, 1.0 / np.sqrt(32), (64, 32))
    w2 = rng.normal(0.0, 1.0 / np.sqrt(64), (64, 64))
    w3 = rng.normal(0.0, 1.0 / np.sqrt(64), 64) * 0.1
    return np.concatenate([w1.ravel(), np.zeros(64), w2.ravel(), np.zeros(64), w3, [e_mean]]).astype(np.float32)


def fit(data, epochs=200, batch=16, lr=1e-3, wE=1.0, wF=1.0, seed=7, device=0, out=MODEL, log=None, lr_final=1e-5,
        descriptors=None, relative_forces=False, atom_energies=True, cutoff=None):
    from objectmd_gb300 import omdg

    with omdg.Network(device) as net:
        if cutoff is not None:
            net.set_cutoff(*cutoff)
        if descriptors is not None:
            net.set_descriptors(*descriptors)
        net.set_dataset(data["natoms"], data["x"], data["box"], data["energy"], data["forces"])
        net.normalize_from_dataset()
        net.set_force_weighting(relative_forces)
        if atom_energies:
            net.set_atom_energies(data["atom_energy"])
        e_mean = float(np.sum(data["energy"]) / np.sum(data["natoms"]))
        net.set_weights(init_params(seed, e_mean))
        t0 = time.time()
        hist = net.train(epochs, batch, lr, wE, wF, seed, lr_final)
        t1 = time.time()
        if out:
            os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)
            net.save(out)
        if log:
            log("trained %d epochs in %.1f s: loss %.4g -> %.4g" % (epochs, t1 - t0, hist[0], hist[-1]))
        return hist, t1 - t0


def force_rmse(model, x, lo, hi, device=0, fallback=True):
    """Force RMSE (eV/A) of the surrogate against plain Tersoff on one
    configuration, with the number of atoms that fell back."""
    from objectmd_gb300 import inputs, omdg

    out = []
    for use_nn in (True, False):
        with omdg.Context(device) as ctx:
            ctx.set_box(lo, hi)
            ctx.set_atoms(x, np.zeros_like(x), masses=[inputs.md_mass("silicon")], znum=[14.0])
            if use_nn:
                ctx.add_nn(model, TERSOFF if fallback else None)
            else:
                ctx.add_tersoff(TERSOFF)
            ctx.set_neighbor(0.3, 0)
            ctx.compute_forces()
            st = ctx.get_state()
            out.append((st["f"], ctx.nn_fallback_atoms() if use_nn else 0))
    (f_nn, nfb), (f_t, _) = out
    return float(np.sqrt(np.mean((f_nn - f_t) ** 2))), float(np.sqrt(np.mean(f_t ** 2))), nfb


def tersoff_snapshot(ncell=8, temp=1000.0, steps=1000, seed=41, device=0):
    """A diamond cell equilibrated by plain-Tersoff MD at `temp` (Berendsen)."""
    from objectmd_gb300 import inputs, omdg

    x, v, (lo, hi) = inputs.diamond_silicon(ncell=ncell, a=5.431, sigma=0.03, temp=temp, seed_pos=seed,
                                            seed_vel=seed + 1)
    with omdg.Context(device) as ctx:
        ctx.set_box(lo, hi)
        ctx.set_atoms(x, v, masses=[inputs.md_mass("silicon")], znum=[14.0])
        ctx.add_tersoff(TERSOFF)
        ctx.set_neighbor(0.3, 0)
        ctx.set_timestep(0.001)
        ctx.set_thermostat(temp, 0.1)
        ctx.step(steps)
        st = ctx.get_state()
    return st["x"], st["v"], lo, hi


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nconf", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=200)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--lr-final", type=float, default=1e-5)
    ap.add_argument("--wE", type=float, default=1.0)
    ap.add_argument("--wF", type=float, default=1.0)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--out", default=MODEL)
    args = ap.parse_args()
    log = lambda *a: print(*a, file=sys.stderr, flush=True)  # noqa: E731
    t0 = time.time()
    data = generate(nconf=args.nconf, seed=args.seed, log=log)
    log("dataset: %d configurations, %d atoms, %.1f s" % (len(data["natoms"]), data["natoms"].sum(),
                                                         time.time() - t0))
    cutoff, descriptors = switch_descriptors()
    hist, secs = fit(data, args.epochs, args.batch, args.lr, args.wE, args.wF, args.seed, out=args.out, log=log,
                     lr_final=args.lr_final, cutoff=cutoff, descriptors=descriptors)
    x, v, lo, hi = tersoff_snapshot(8, 1000.0)
    rmse, frms, nfb = force_rmse(args.out, x, lo, hi)
    log("force RMSE vs Tersoff at 1000 K (4096 atoms): %.4f eV/A (force RMS %.3f, %d fallback atoms)" %
        (rmse, frms, nfb))
    print({"epochs": args.epochs, "train_seconds": secs, "loss_first": float(hist[0]), "loss_last": float(hist[-1]),
           "rmse_eV_per_A": rmse, "force_rms": frms, "fallback_atoms": nfb})


if __name__ == "__main__":
    main()
