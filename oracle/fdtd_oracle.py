"""FP64 restatement of the reference's finite-difference heat solver
(FDTDSolver, src/omd/fdtd.cpp; include/misc/fdtd.hpp), single rank.

Test infrastructure (the oracle): tests/ use it to check the device solver
(objectmd_gb300/csrc/fdtd.cu).  The product never imports it.  Pinned against
the reference itself: tests/golden/fdtd_cases.npz holds the cell vectors that
oracle/_ref/fdtd_driver (fdtd.cpp compiled from the reference tree by
oracle/ref/Makefile) printed for the specs in tests/golden/make_golden.py.

Solve (fdtd.cpp:605-668), per cell in index order:
    acc = sum over the faces whose flag is set (r, l, b, t, n, f) of
          K (T_nb - T_i),  K = con_nb con_i / (con_nb + con_i)  (skipped if the sum is 0)
    A_i = T_i + (2 acc h2inv + S_i + E_i) dt / cap_i ;  S_i = E_i = 0
A cell whose map character is not a symbol skips the face loop and acc is
its old value.  get_neigcell_index (fdtd.cpp:270-300) clears a symbol's flag
for good the first time a cell of that symbol has that face beyond the grid
and the flag is not periodic.
"""
import numpy as np

INT_MAX = 2147483647
DBL_MAX = np.finfo(np.float64).max


def _flag(c):
    return 1 if c == "+" else (2 if c == "p" else 0)


def _as_double(v):
    """as_double (omdtool.cpp:98-104): the longest leading number, "inf" as DBL_MAX."""
    if v == "inf":
        return DBL_MAX
    if v == "-inf":
        return -DBL_MAX
    best = None
    for k in range(len(v), 0, -1):
        try:
            best = float(v[:k])
            break
        except ValueError:
            continue
    if best is None or v[:1].isspace():
        raise ValueError("conversion error: " + v)
    return best


def _leading_ints(s, n):
    out = []
    for tok in s.split():
        if len(out) == n:
            break
        try:
            out.append(int(tok))
        except ValueError:
            break
    return out


class Grid:
    def __init__(self, nx, ny, nz, symbol, cmap):
        self.nx, self.ny = nx, ny
        self.nz = 1 if nz <= 2 else nz
        self.dim = self.nx * self.ny * self.nz
        self.bound = []  # [sym, l, r, t, b, n, f]
        toks = symbol.split()
        for a in range(0, len(toks) - 1, 2):
            tok, sb = toks[a], toks[a + 1]
            if len(sb) < 4:
                raise ValueError("invalid map symbol entry")
            for ch in tok:
                nf = (_flag(sb[4]), _flag(sb[5])) if (self.nz > 1 and len(sb) == 6) else (0, 0)
                self.bound.append([ch, _flag(sb[0]), _flag(sb[1]), _flag(sb[2]), _flag(sb[3]), nf[0], nf[1]])
        if len(cmap) != self.dim:
            raise ValueError("map string count inconsistent")
        syms = [b[0] for b in self.bound]
        self.map = np.array([syms.index(c) if c in syms else -1 for c in cmap])
        self.A = np.zeros(self.dim)
        self.S = np.zeros(self.dim)
        self.E = np.zeros(self.dim)
        self.con = np.ones(self.dim)
        self.cap = np.ones(self.dim)
        self.step = 0
        self.timestep = 1.0
        self.h2inv = 1.0
        self.str_src = self.str_con = self.str_cap = ""

    def index(self, i, j, k):
        return k * self.nx * self.ny + i + j * self.nx

    def set_timestep(self, dt):
        self.timestep = dt

    def set_spacestep(self, h):
        self.h2inv = 1.0 / (h * h)

    # AssignArray(ptr, str) (fdtd.cpp:528-592); returns the kept tokens
    def assign(self, a, s):
        if not s:
            return s
        toks = s.split()
        kept = ""
        for p in range(0, len(toks) - 1, 2):
            tok, val = toks[p], toks[p + 1]
            isequ = "{" in val
            parts = val.replace(":", " ").replace("{", "").replace("}", "").split()
            val = parts[0] if parts else ""
            ints = _leading_ints(" ".join(parts[1:]), 2)
            if ints:
                t0 = ints[0]
                t1 = ints[1] if len(ints) > 1 else t0
            else:
                t0, t1 = -INT_MAX, INT_MAX
            if not (t0 <= self.step <= t1):
                continue
            if t0 != t1:
                kept += (tok + " {" + val + ":%d:%d} " if isequ else tok + " " + val + ":%d:%d ") % (t0, t1)
            if isequ:
                raise ValueError("expressions need muParser")
            if tok[0] == "@":
                q = val.find("=")
                cs = val if q < 0 else val[:q]
                v = val if q < 0 else val[q + 1:]
                c = _leading_ints(cs.replace(",", " "), 6)
                if len(c) < 3:
                    raise ValueError("wrong coordinate")
                if len(c) == 6:
                    ix, iy, iz, jx, jy, jz = c
                    if self.nz == 1:
                        iz = jz = 0
                    cells = [(i, j, k) for i in range(ix, jx + 1) for j in range(iy, jy + 1) for k in range(iz, jz + 1)]
                else:
                    cells = [tuple(c[:3])]
                for i, j, k in cells:
                    idx = self.index(i, j, k)
                    if idx >= self.dim or idx < 0:
                        raise ValueError("AssignArray out of range")
                    a[idx] = _as_double(v)
            else:
                for ch in tok:
                    for i in range(self.nx):
                        for j in range(self.ny):
                            for k in range(self.nz):
                                idx = self.index(i, j, k)
                                m = self.map[idx]
                                sym = "." if m < 0 else self.bound[m][0]
                                if ch == "*" or sym == ch:
                                    a[idx] = _as_double(val)
        return kept

    def set_cell(self, s):
        self.assign(self.A, s)

    def set_source(self, s):
        self.str_src = s
        self.assign(self.S, s)

    def set_conductivity(self, s):
        self.str_con = s
        self.assign(self.con, s)

    def set_capacity(self, s):
        self.str_cap = s
        self.assign(self.cap, s)

    def _neighbours(self, idx):
        """get_neigcell_index (fdtd.cpp:270-300), flags cleared in place."""
        xy = self.nx * self.ny
        k, a = divmod(idx, xy)
        j, i = divmod(a, self.nx)
        cc = self.bound[self.map[idx]]
        l, r, t, b, n, f = i - 1, i + 1, j - 1, j + 1, k - 1, k + 1
        if l < 0:
            if cc[1] == 2:
                l = self.nx - 1
            else:
                cc[1] = 0
        if r >= self.nx:
            if cc[2] == 2:
                r = 0
            else:
                cc[2] = 0
        if t < 0:
            if cc[3] == 2:
                t = self.ny - 1
            else:
                cc[3] = 0
        if b >= self.ny:
            if cc[4] == 2:
                b = 0
            else:
                cc[4] = 0
        if self.nz != 1:
            if n < 0:
                if cc[5] == 2:
                    n = self.nz - 1
                else:
                    cc[5] = 0
            if f >= self.nz:
                if cc[6] == 2:
                    f = 0
                else:
                    cc[6] = 0
        else:
            n = f = 0
        out = [self.index(l, j, k), self.index(r, j, k), self.index(i, t, k), self.index(i, b, k)]
        if self.nz != 1:
            out += [self.index(i, j, n), self.index(i, j, f)]
        return cc, out

    def solve(self):
        T = self.A.copy()
        A = self.A
        for idx in range(self.dim):
            if self.map[idx] < 0:
                continue
            cc, nb = self._neighbours(idx)
            l, r, t, b = nb[:4]
            acc = 0.0
            order = [(cc[2], r), (cc[1], l), (cc[4], b), (cc[3], t)]
            if self.nz != 1:
                order += [(cc[5], nb[4]), (cc[6], nb[5])]
            for fl, o in order:
                if fl:
                    K = self.con[o] + self.con[idx]
                    if K != 0.0:
                        K = self.con[o] * self.con[idx] / K
                        acc += K * (T[o] - T[idx])
            A[idx] = acc
        self.A = T + (2.0 * A * self.h2inv + self.S + self.E) * self.timestep / self.cap
        self.S[:] = 0.0
        self.E[:] = 0.0

    def run_step(self):
        """One loop of Step (fdtd.cpp:671-689) on one rank."""
        self.str_src = self.assign(self.S, self.str_src)
        self.str_con = self.assign(self.con, self.str_con)
        self.str_cap = self.assign(self.cap, self.str_cap)
        self.solve()
        self.step += 1


def run_spec(spec):
    """Run a spec in the driver's format (oracle/ref/fdtd_driver.cpp); the
    cell vector before the steps and after each, as rows."""
    g = None
    dims = symbol = None
    ext = []
    rows = []
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
            g = Grid(dims[0], dims[1], dims[2], symbol, rest.strip())
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
            rows.append(g.A.copy())
            for _ in range(int(rest)):
                for i, v in ext:
                    g.E[i] = v
                g.run_step()
                rows.append(g.A.copy())
    return np.array(rows)
