"""Synthetic inputs with the shapes of the benchmark configurations.

Mirrors what the reference's crystal builders produce (FCC.cpp:142-242,
Diamond.h:17-58, Projectile.h:22-49) closely enough for benchmarking, and
writes them in the reference's Import format (container.cpp:290-400) with
``%.17g`` so that the reference CPU path and this library read identical
FP64 coordinates.  Velocities are Maxwell-Boltzmann from a seeded PCG64
stream with the net momentum removed; the reference's own SetTemperature
(container.cpp:683-754) seeds from the process id and is not reproducible,
so both sides are fed the same file instead.

Units are the reference's: Angstrom, ps, eV, mass in amu / 9648.53397731809
(conversion.h:29), k_B = 8.61734279e-5 eV/K (conversion.h:46).
"""
from __future__ import annotations

import math

import numpy as np

NORMAL_AMU = 9.64853397731809e3
MD_BOLTZMANN = 8.61734279e-05

# element: (mass in amu, atomic number) -- the values of the reference's def.* files
ELEMENTS = {
    "aluminum": (26.98154, 13.0),
    "silicon": (28.0855, 14.0),
    "argon": (39.948, 18.0),
    "copper": (63.546, 29.0),
    "platinum": (195.078, 78.0),
}


def md_mass(element: str) -> float:
    """Mass in simulation units (container.cpp:94)."""
    return ELEMENTS[element][0] / NORMAL_AMU


FCC_BASIS = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.0], [0.5, 0.0, 0.5], [0.0, 0.5, 0.5]])
DIAMOND_BASIS = np.concatenate([FCC_BASIS, FCC_BASIS + 0.25])


def lattice(basis: np.ndarray, ncell, a: float, offset: float):
    """Atoms of n[0] x n[1] x n[2] cubic cells, cell-major (z, y, x, basis)."""
    nx, ny, nz = (ncell, ncell, ncell) if np.isscalar(ncell) else ncell
    iz, iy, ix = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    cells = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1).astype(np.float64)
    pos = (cells[:, None, :] + basis[None, :, :] + offset).reshape(-1, 3) * a
    box_hi = np.array([nx, ny, nz], dtype=np.float64) * a
    return pos, np.zeros(3), box_hi


def fcc(ncell, a):
    """FCC crystal; coordinates offset by a/4 so no atom sits on a box face."""
    return lattice(FCC_BASIS, ncell, a, 0.25)


def diamond(ncell, a):
    """Diamond crystal; coordinates offset by a/8."""
    return lattice(DIAMOND_BASIS, ncell, a, 0.125)


def perturb(x, sigma, seed, lo=None, hi=None, periodic=(True, True, True)):
    rng = np.random.default_rng(seed)
    x = x + rng.normal(0.0, sigma, size=x.shape)
    if lo is not None:
        for d in range(3):
            if periodic[d]:
                L = hi[d] - lo[d]
                x[:, d] = lo[d] + np.mod(x[:, d] - lo[d], L)
                x[:, d] = np.where(x[:, d] >= hi[d], x[:, d] - L, x[:, d])
    return x


def maxwell_boltzmann(n, temperature, mass, seed):
    """Velocities (A/ps) at temperature T with zero net momentum.

    ``mass`` is a scalar or per-atom array in simulation units.
    """
    rng = np.random.default_rng(seed)
    m = np.broadcast_to(np.asarray(mass, dtype=np.float64), (n,))
    sig = np.sqrt(MD_BOLTZMANN * temperature / m)
    v = rng.normal(0.0, 1.0, size=(n, 3)) * sig[:, None]
    p = (v * m[:, None]).sum(axis=0) / m.sum()
    return v - p[None, :]


def temperature(v, mass):
    """T = (2/3) KE_per_atom / k_B (unit.h:125)."""
    m = np.broadcast_to(np.asarray(mass, dtype=np.float64), (len(v),))
    ke = 0.5 * float((m[:, None] * v * v).sum())
    return (2.0 / 3.0) / MD_BOLTZMANN * ke / len(v)


def write_import(path, x, v=None, types=None, box=None, periodic=(True, True, True), species=("aluminum",),
                 names=None):
    """Write atoms in the reference Import format.

    Single species: ``#$ Material <element>``.  Several species: one
    ``#$ IDk <name> <element>`` per type and an ``id`` column; atoms must be
    ordered by type so that the reference's enumeration (nid) equals the row
    order (system.cpp:1399-1417, :389-397).
    """
    n = len(x)
    if v is None:
        v = np.zeros_like(x)
    lines = ["# synthetic input (objectmd_gb300.inputs)"]
    multi = len(species) > 1
    if multi:
        if names is None:
            names = ["type%d" % k for k in range(len(species))]
        for k, (nm, el) in enumerate(zip(names, species)):
            lines.append("#$ ID%d %s %s" % (k, nm, el))
        assert types is not None and np.all(np.diff(types) >= 0), "atoms must be ordered by type"
    else:
        lines.append("#$ Material %s" % species[0])
    if box is not None:
        lo, hi = box
        lines.append("#$ Box %.17g %.17g %.17g %.17g %.17g %.17g" % (lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]))
    pb = (1 if periodic[0] else 0) | (2 if periodic[1] else 0) | (4 if periodic[2] else 0)
    lines.append("#$ PeriodicBoundary %d" % pb)
    lines.append("#$ Fields x y z vx vy vz%s --" % (" id" if multi else ""))
    body = []
    if multi:
        for i in range(n):
            body.append("%.17g %.17g %.17g %.17g %.17g %.17g %d" % (x[i, 0], x[i, 1], x[i, 2], v[i, 0], v[i, 1],
                                                                    v[i, 2], types[i]))
    else:
        arr = np.concatenate([x, v], axis=1)
        body = ["%.17g %.17g %.17g %.17g %.17g %.17g" % tuple(r) for r in arr]
    with open(path, "w") as fh:
        fh.write("\n".join(lines + body) + "\n")


def read_import(path):
    """Read back an Import file written by write_import (x, v, types, box, periodic)."""
    lo = hi = None
    pb = 0
    multi = False
    with open(path) as fh:
        head = []
        for line in fh:
            if line.startswith("#"):
                head.append(line)
            else:
                break
    for line in head:
        t = line.split()
        if len(t) > 1 and t[0] == "#$" and t[1] == "Box":
            vals = [float(s) for s in t[2:8]]
            lo, hi = np.array(vals[:3]), np.array(vals[3:])
        if len(t) > 1 and t[0] == "#$" and t[1] == "PeriodicBoundary":
            pb = int(t[2])
        if len(t) > 1 and t[0] == "#$" and t[1] == "Fields":
            multi = "id" in t
    data = np.loadtxt(path, comments="#", ndmin=2)
    x = data[:, 0:3].copy()
    v = data[:, 3:6].copy() if data.shape[1] >= 6 else np.zeros_like(x)
    types = data[:, 6].astype(np.int32) if multi else np.zeros(len(x), dtype=np.int32)
    return x, v, types, (lo, hi), (bool(pb & 1), bool(pb & 2), bool(pb & 4))


# ------------------------------------------------------------------ workloads

def eam_aluminium(ncell=40, a=4.05, sigma=0.05, temp=300.0, seed_pos=2, seed_vel=3):
    """FCC Al, Gaussian displacements and Maxwell-Boltzmann velocities."""
    x, lo, hi = fcc(ncell, a)
    x = perturb(x, sigma, seed_pos, lo, hi)
    v = maxwell_boltzmann(len(x), temp, md_mass("aluminum"), seed_vel)
    return x, v, (lo, hi)


def diamond_silicon(ncell=40, a=5.431, sigma=0.03, temp=1000.0, seed_pos=4, seed_vel=5):
    x, lo, hi = diamond(ncell, a)
    x = perturb(x, sigma, seed_pos, lo, hi)
    v = maxwell_boltzmann(len(x), temp, md_mass("silicon"), seed_vel)
    return x, v, (lo, hi)


def lj_argon(ncell=10, a=5.26, temp=100.0, seed_vel=1):
    x, lo, hi = fcc(ncell, a)
    v = maxwell_boltzmann(len(x), temp, md_mass("argon"), seed_vel)
    return x, v, (lo, hi)


def lj_table_text(sigma=3.405, eps=0.0104, rc=None, r0=2.0, n=5000):
    """An Object-MD PLAIN pair table of the analytic 12-6 Lennard-Jones potential.

    The reference ships no analytic LJ kernel; its TForcePair reads a table
    (tpair.h:38-71).  The table ends at rc (default 2.5 sigma), where the
    reference's strict r < rc cut applies; the potential is not shifted.
    """
    if rc is None:
        rc = 2.5 * sigma
    dr = (rc - r0) / (n - 1)
    r = r0 + dr * np.arange(n)
    sr6 = (sigma / r) ** 6
    phi = 4.0 * eps * (sr6 * sr6 - sr6)
    out = ["# Lennard-Jones 12-6, sigma=%.17g eps=%.17g, not shifted" % (sigma, eps),
           "#$ NumberOfData %d" % n, "#$ Spacing %.17g" % dr, "#$ Offset %.17g" % r0, "#$ Format PLAIN", "#$ --"]
    out += ["%.17g" % p for p in phi]
    return "\n".join(out) + "\n"


def tersoff_param_text(R=2.7, D=0.15):
    """Tersoff Si parameter set (Tersoff, PRB 37, 6991 (1988)) with a chosen cutoff."""
    p = dict(A=3264.7, lambda_1=3.2394, alpha=0.0, c=4.8381, lambda_3=1.3258, B=95.373, lambda_2=1.3258,
             beta=0.33675, d=2.0417, R=R, n=22.956, h=0.0, D=D)
    lines = ["# Tersoff silicon, PRB 37, 6991 (1988); cutoff R=%g D=%g" % (R, D)]
    lines += ["tersoff.%s %.17g" % (k, v) for k, v in p.items()]
    lines.append("tersoff.zbl false")
    return "\n".join(lines) + "\n"


def sw_param_text():
    """Stillinger-Weber silicon (PRB 31, 5262 (1985)) in the reference key names."""
    p = [("sw.epsilon", 2.1683), ("sw.A", 7.049556277), ("sw.B", 0.6022245584), ("sw.p", 4), ("sw.q", 0),
         ("sw.sigma", 2.0951), ("sw.a", 1.80), ("sw.lambda", 21.0), ("sw.gamma", 1.20), ("sw.invers_cos0", -3.0)]
    lines = ["# Stillinger-Weber silicon, PRB 31, 5262 (1985)"] + ["%s %.17g" % kv for kv in p]
    lines += ["zbl yes", "spline.range 1.2107 1.8456", "spline.coeff 335.0594 -492.3905 244.5280 -41.2347"]
    return "\n".join(lines) + "\n"


def projectile(target_xy, z_surface, height, theta_deg, phi_deg, energy_ev, mass):
    """Projectile.h:22-49 semantics: start `height` above the aim point along
    (theta, phi) and move towards it with kinetic energy `energy_ev`."""
    th, ph = math.radians(theta_deg), math.radians(phi_deg)
    u = np.array([math.sin(th) * math.cos(ph), math.sin(th) * math.sin(ph), math.cos(th)])
    start = np.array([target_xy[0], target_xy[1], z_surface]) + height * u
    speed = math.sqrt(2.0 * energy_ev / mass)
    return start, -speed * u


def impact_ensemble(nrep=256, nmin=1000, nmax=16000, temp=300.0, emin=10.0, emax=500.0, theta_max=30.0,
                    a=5.431, sigma=0.03, height=5.0, vacuum=10.0, seed=6):
    """Independent Si diamond slabs of uneven size, each aimed at by one Ar atom.

    Replica r has N_r = round(exp(U[ln nmin, ln nmax])) target atoms arranged
    as an nx x nx x nz cell slab (nx = nz ~ (N_r / 8)^(1/3)), periodic in x
    and y with a free surface on top, Gaussian displacements `sigma` and
    Maxwell-Boltzmann velocities at `temp`.  The Ar atom starts `height` above
    a uniformly drawn aim point on the surface along (theta ~ U[0, theta_max],
    phi ~ U[0, 360)) with E = exp(U[ln emin, ln emax]) eV (Projectile.h:22-49).
    Returns per-replica atom counts, positions, velocities, types (0 Si,
    1 Ar), box lo/hi and the drawn energies and angles.
    """
    rng = np.random.default_rng(seed)
    m_si, m_ar = md_mass("silicon"), md_mass("argon")
    natoms, xs, vs, ts, los, his, meta = [], [], [], [], [], [], []
    for r in range(nrep):
        n_r = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        nx = max(2, int(round((n_r / 8.0) ** (1.0 / 3.0))))
        nz = max(2, int(round(n_r / (8.0 * nx * nx))))
        x, lo, hi = lattice(DIAMOND_BASIS, (nx, nx, nz), a, 0.125)
        x = x + rng.normal(0.0, sigma, size=x.shape)
        for d in range(2):
            x[:, d] = np.mod(x[:, d], hi[d])
        v = maxwell_boltzmann(len(x), temp, m_si, int(rng.integers(1 << 31)))
        z_top = float(x[:, 2].max())
        e = math.exp(rng.uniform(math.log(emin), math.log(emax)))
        th = rng.uniform(0.0, theta_max)
        ph = rng.uniform(0.0, 360.0)
        aim = rng.uniform(0.0, 1.0, 2) * hi[:2]
        p0, pv = projectile(aim, z_top, height, th, ph, e, m_ar)
        p0[:2] = np.mod(p0[:2], hi[:2])
        xs.append(np.vstack([x, p0]))
        vs.append(np.vstack([v, pv]))
        ts.append(np.concatenate([np.zeros(len(x), dtype=np.int32), [1]]).astype(np.int32))
        natoms.append(len(x) + 1)
        los.append([0.0, 0.0, -0.5 * a])
        his.append([hi[0], hi[1], z_top + height + vacuum])
        meta.append((e, th, ph))
    return {"natoms": np.array(natoms), "x": np.concatenate(xs), "v": np.concatenate(vs), "types": np.concatenate(ts),
            "lo": np.array(los), "hi": np.array(his), "energy_theta_phi": np.array(meta),
            "masses": [m_si, m_ar], "znum": [14.0, 18.0]}


def ttm_table_text(g0=1.529e-6, c0=8.43e-10, dT=10.0, n=8001, g_slope=1.0 / 20000.0):
    """Electron-phonon table for TTM_Homogen (TTM_Homogen_SCNA.h:176-180):
    section ELECTRON_PHONON_COUPLING with G(T) = 1 + g_slope T and Constant
    g0 (eV / (ps A^3 K)); section ELECTRON_HEAT_CAPACITY with Ce(T) = T and
    Constant c0 (eV / (A^3 K^2)), so C_e = c0 T.  Knots T = 0, dT, ...
    Defaults: aluminium, G = 2.45e17 W/(m^3 K), gamma = 135 J/(m^3 K^2)."""
    T = np.arange(n) * dT
    out = ["# electron-phonon coupling and electron heat capacity (objectmd_gb300.inputs)"]
    for name, const, vals in (("ELECTRON_PHONON_COUPLING", g0, 1.0 + g_slope * T),
                              ("ELECTRON_HEAT_CAPACITY", c0, T)):
        out += ["#$%s Constant %.17g" % (name, const), "#$%s NumberOfData %d" % (name, n),
                "#$%s Spacing %.17g" % (name, dT), "#$%s Offset 0" % name, "#$%s Format PLAIN" % name,
                "#$%s --" % name]
        out += ["%.17g" % v for v in vals]
    return "\n".join(out) + "\n"


def aluminium_cluster(ncell=6, a=4.05, sigma=0.05, temp=300.0, vacuum=15.0, seed_pos=12, seed_vel=13):
    """A free FCC Al cluster (ncell^3 cells) in a non-periodic box with
    `vacuum` A of space on every side."""
    x, lo, hi = fcc(ncell, a)
    rng = np.random.default_rng(seed_pos)
    x = x + rng.normal(0.0, sigma, size=x.shape)
    v = maxwell_boltzmann(len(x), temp, md_mass("aluminum"), seed_vel)
    return x, v, (np.asarray(lo) - vacuum, np.asarray(hi) + vacuum)
