"""FP64 restatement of the reference's ThermoDetector (intensive mode) and
TTM_Homogen (scaling-corrected homogeneous two-temperature model).

Test infrastructure (the oracle): tests/ use it; the product never imports
it.  Pinned against the reference's own run (tests/golden/ttm_al_cluster.npz,
made by tests/golden/make_golden.py).  Free clusters only: on a periodic
MDSystemGrid the reference computes ghost images' local centre-of-mass
velocities from their incomplete neighbourhoods, which this restatement does
not reproduce.
"""
import numpy as np

MD_BOLTZMANN = 8.61734279e-05  # eV / K (conversion.h:46)
FAC_TEMPERATURE = 2.0 / 3.0 / MD_BOLTZMANN  # Unit::Temperature (unit.h:125)


def pairs_within(x, rcut):
    """All pairs i < j with |x_i - x_j| <= rcut (FP64, as CalcDistance)."""
    d = x[:, None, :] - x[None, :, :]
    r = np.sqrt((d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2])
    i, j = np.nonzero(np.triu(r <= rcut, 1))
    return i, j


def local_thermo(x, v, mass, ercut):
    """ThermoDetector::ExtractTemperature (ThermoDetector.h:176-237).

    v_cm_i = sum m_j v_j / sum m_j over i and its neighbours within ercut;
    T_i = Unit::Temperature(1/2 sum_j m_j |v_j - v_cm_j|^2 / n_i) over the
    same atoms (each one relative to its own local centre of mass);
    density_i = n_i / (4/3 pi ercut^3); averages over atoms with n_i >= 2."""
    n = len(x)
    i, j = pairs_within(x, ercut)
    msum = mass.copy()
    np.add.at(msum, i, mass[j])
    np.add.at(msum, j, mass[i])
    mv = mass[:, None] * v
    psum = mv.copy()
    np.add.at(psum, i, mv[j])
    np.add.at(psum, j, mv[i])
    vcm = psum / msum[:, None]
    c = v - vcm
    ek = mass * (c * c).sum(1)
    sumek = ek.copy()
    np.add.at(sumek, i, ek[j])
    np.add.at(sumek, j, ek[i])
    nn = np.ones(n, dtype=np.int64)
    np.add.at(nn, i, 1)
    np.add.at(nn, j, 1)
    volcut = 4.0 * np.pi * ercut ** 3 / 3.0
    temp = FAC_TEMPERATURE * 0.5 * sumek / nn
    dens = nn / volcut
    sel = nn >= 2
    avg_t = temp[sel].mean() if sel.any() else 0.0
    avg_d = dens[sel].mean() if sel.any() else 0.0
    return {"vcm": vcm, "temp": temp, "dens": dens, "nneig": nn, "avg_temp": avg_t, "avg_dens": avg_d,
            "volcut": volcut}


class TTM:
    """TTM_Homogen (TTM_Homogen_SCNA.h:232-376) without energy source or density
    factors: electron_init_temperature te0, atom volume, tables G and Ce
    (oracle Table objects) with their Constant values g0 and c0."""

    def __init__(self, G, Ce, g0, c0, atom_volume, te0, dt, pulse_offset=0.0):
        self.G, self.Ce, self.g0, self.c0 = G, Ce, g0, c0
        self.vol, self.te, self.dt, self.offset = atom_volume, te0, dt, pulse_offset
        self.first = True
        self.int_een = 0.0
        self.int_aen = 0.0

    def pre_integration(self, elapsed, thermo, v, mass, kinetic, vmax):
        """One PreIntegration (after the first-run detection): the electron
        temperature step and the velocity rescaling about local centres of
        mass; returns the new velocities."""
        if not elapsed > self.offset:
            return v
        ta = thermo["avg_temp"]
        if self.first:
            self.int_een = 0.5 * self.te * self.c0 * self.Ce.read(self.te)[0] * self.vol
            self.int_aen = 2.0 * kinetic / len(v)
            self.first = False
        de = -self.g0 * self.G.read(self.te)[0] * (self.te - ta) * self.dt
        self.int_een += de * self.vol
        self.te += de / (self.c0 * self.Ce.read(self.te)[0])
        coup = self.g0 * self.G.read(self.te)[0]
        small = (vmax * 1e-6) ** 2
        v = v.copy()
        cm, T, nn = thermo["vcm"], thermo["temp"], thermo["nneig"]
        dens, volcut = thermo["dens"], thermo["volcut"]
        s, k = 0.0, 0
        for a in range(len(v)):
            if dens[a] * volcut <= 3.0:
                continue
            dea = coup * (self.te - T[a]) * self.vol * self.dt
            c = v[a] - cm[a]
            c2 = c @ c
            if c2 < small:
                continue
            cmc = cm[a] @ c
            cm2 = cm[a] @ cm[a]
            v2 = v[a] @ v[a]
            rr = cmc * cmc + c2 * (2.0 * dea / mass[a] + v2 - cm2)
            if rr < 0.0:
                continue
            sa = (-cmc + np.sqrt(rr)) / c2
            v[a] = cm[a] + sa * c
            s += dea
            k += 1
        self.int_aen += s / k if k else 0.0
        return v


CELL_SCALE = 1048576.0  # 2^20: the device sums cell temperatures as integers


def grid_cells(x, origin, h, shape, lo=None, L=None, periodic=(False, False, False)):
    """The grid cell index of each position (-1 outside), as the coupled
    step assigns atoms: periodic axes wrapped into the box, a 2D grid
    (nz = 1) spanning every z."""
    nx, ny, nz = shape
    out = np.full(len(x), -1)
    for a, r in enumerate(x):
        c = []
        for d in range(3):
            w = r[d]
            if periodic[d]:
                w -= np.floor((w - lo[d]) / L[d]) * L[d]
            c.append(int(np.floor((w - origin[d]) / h)))
        if nz == 1:
            c[2] = 0
        if 0 <= c[0] < nx and 0 <= c[1] < ny and 0 <= c[2] < nz:
            out[a] = c[2] * nx * ny + c[0] + c[1] * nx
    return out


def grid_pre_integration(grid, cells, temp, nneig, G, Ce, g0, c0, first):
    """The coupled step's electron part on an oracle/fdtd_oracle.Grid:
    lattice temperature per cell (atoms with n_i >= 2, temperatures summed as
    the device does, in units of 2^-20 K), the negative cells set at the
    first active step, E = -g0 G(Te) (Te - Ta) where the cell holds atoms,
    cap = c0 Ce(Te), then one solve.  Returns the per-cell lattice
    temperatures."""
    sums = [0] * grid.dim
    cnt = [0] * grid.dim
    for a in range(len(temp)):
        if nneig[a] < 2 or cells[a] < 0:
            continue
        t = temp[a] if temp[a] > 0.0 else 0.0
        sums[cells[a]] += int(np.rint(t * CELL_SCALE))
        cnt[cells[a]] += 1
    ta = np.array([(float(sums[c]) / CELL_SCALE) / cnt[c] if cnt[c] else 0.0 for c in range(grid.dim)])
    for c in range(grid.dim):
        te = grid.A[c]
        if first and te < 0.0:
            te = ta[c]
        grid.A[c] = te
        grid.E[c] = -g0 * G.read(te)[0] * (te - ta[c]) if cnt[c] else 0.0
        grid.cap[c] = c0 * Ce.read(te)[0]
    grid.solve()
    return ta
