"""CPU FP64 oracle for the Object-MD force path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may import this module, and only as
the checker.  The product library never loads it.

This wraps ``liboracle.so`` (``oracle/omd_oracle.c``, a restatement of the
reference's hot path in C) and runs ``oracle/_ref/ref_driver`` (the reference's
own code, built from its sources by ``oracle/ref/Makefile``) when it exists.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_DRIVER = os.path.join(REF_DIR, "ref_driver")
REF_DRIVER_SWFIX = os.path.join(REF_DIR, "ref_driver_swfix")


def build(force: bool = False) -> str:
    """Compile the C restatement (gcc, FP64, no FMA contraction)."""
    src = os.path.join(HERE, "omd_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        os.makedirs(BUILD, exist_ok=True)
        tmp = LIB_PATH + ".tmp%d" % os.getpid()
        # OpenMP: the per-atom loops run in threads for the timed CPU baseline
        # (OMP_NUM_THREADS); every atom's sums are its own, so results do not change
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-o", tmp, src,
                               "-lm"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_reference(ref_root: str) -> bool:
    """Compile the reference sources found under ``ref_root`` (the Object-MD
    source tree) into oracle/_ref; False where that tree is absent."""
    if not ref_root or not os.path.isdir(ref_root):
        return False
    subprocess.check_call(["make", "-s", "-C", os.path.join(HERE, "ref"), "REF=" + ref_root, "-j8"])
    return os.path.exists(REF_DRIVER)


class _Table(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int),
        ("dr", ctypes.c_double),
        ("off", ctypes.c_double),
        ("rmult", ctypes.c_int),
        ("allow_lo", ctypes.c_int),
        ("allow_hi", ctypes.c_int),
        ("out_lo", ctypes.c_double),
        ("out_hi", ctypes.c_double),
        ("a", ctypes.POINTER(ctypes.c_double)),
        ("b", ctypes.POINTER(ctypes.c_double)),
        ("c", ctypes.POINTER(ctypes.c_double)),
        ("d", ctypes.POINTER(ctypes.c_double)),
    ]


class _Box(ctypes.Structure):
    _fields_ = [("lo", ctypes.c_double * 3), ("hi", ctypes.c_double * 3), ("periodic", ctypes.c_int * 3)]


class SWParam(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("eps", "A", "B", "p", "q", "sigma", "a", "lam", "gamma", "icos0")] + [
        ("usezbl", ctypes.c_int)
    ] + [(k, ctypes.c_double) for k in ("sx0", "sx1", "sa0", "sa1", "sa2", "sa3", "z1", "z2")]


class TersoffParam(ctypes.Structure):
    _fields_ = [
        (k, ctypes.c_double)
        for k in ("A", "B", "lambda1", "lambda2", "lambda3", "beta", "n", "c", "d", "h", "R", "D")
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        P = ctypes.POINTER
        d, i = ctypes.c_double, ctypes.c_int
        _lib.oc_table_coef.argtypes = [P(_Table)]
        _lib.oc_table_read.argtypes = [P(_Table), d, P(d), P(d)]
        _lib.oc_table_read.restype = i
        _lib.oc_neighbors.argtypes = [P(_Box), i, P(d), d, P(i), P(i), P(i), ctypes.c_long]
        _lib.oc_neighbors.restype = ctypes.c_long
        nb = [P(_Box), i, P(d), P(i), P(i), P(i)]
        _lib.oc_eam.argtypes = nb + [P(_Table), P(_Table), P(_Table), P(d), P(d), P(d), P(d)]
        _lib.oc_pair_table.argtypes = nb + [P(_Table), P(d), P(d), P(d)]
        _lib.oc_pair_table_typed.argtypes = [P(_Box), i, P(d), P(i), i, i, P(i), P(i), P(i), P(_Table), P(d), P(d),
                                             P(d)]
        _lib.oc_sw.argtypes = nb + [P(SWParam), P(d), P(d), P(d)]
        _lib.oc_tersoff.argtypes = nb + [P(TersoffParam), P(d), P(d), P(d)]
        _lib.oc_zbl.argtypes = [P(_Box), i, P(d), P(i), i, i, d, d, d, d, P(i), P(i), P(i), P(d), P(d), P(d)]
        for fn in ("oc_eam", "oc_pair_table", "oc_pair_table_typed", "oc_sw", "oc_tersoff", "oc_zbl"):
            getattr(_lib, fn).restype = i
        _lib.oc_vv_kick_drift.argtypes = [i, P(d), P(d), P(d), P(d), d]
        _lib.oc_vv_kick.argtypes = [i, P(d), P(d), P(d), d]
        _lib.oc_kinetic.argtypes = [i, P(d), P(d)]
        _lib.oc_kinetic.restype = d
        _lib.oc_wrap.argtypes = [P(_Box), i, P(d)]
        _lib.oc_berendsen_factor.argtypes = [d, d, d, d]
        _lib.oc_berendsen_factor.restype = d
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


# --------------------------------------------------------------------- tables

def parse_table(path: str, name: str = "") -> dict:
    """Read one ``#$NAME``-tagged section of an Object-MD table file.

    Follows TableReader::open_omd (treader.cpp:83-136) and read_pseudo
    (param.cpp:106-136): every token after ``#$<name>`` on its lines goes into
    one flat list up to the line ``#$<name> --``; a key's value is the token
    after its first occurrence (param.cpp:165-171, 218-223).  Keys:
    NumberOfData, Spacing, Offset (default 0), Format (PLAIN|RMULT),
    OutOfRangeLower/Upper; the values follow the ``--`` line.
    """
    tag = "#$" + name
    spar = []
    values = []
    with open(path) as fh:
        lines = fh.read().split("\n")
    start = None
    for k, line in enumerate(lines):
        tok = line.split()
        if len(tok) >= 2 and tok[0] == tag:
            if tok[1] == "--":
                start = k + 1
                break
            spar.extend(tok[1:])

    def value(key, default=None):
        for i, t in enumerate(spar):
            if t == key:
                return spar[i + 1] if i + 1 < len(spar) else default
        return default

    if start is None:
        raise ValueError("can not find table %s@%s" % (name, path))
    n = int(value("NumberOfData"))
    toks = " ".join(lines[start:]).split()
    values = np.array([float(t) for t in toks[:n]], dtype=np.float64)
    if len(values) != n:
        raise ValueError("short table %s@%s" % (name, path))
    fmt = value("Format", "PLAIN")
    return {
        "n": n,
        "dr": float(value("Spacing")),
        "off": float(value("Offset", "0")),
        "rmult": 1 if fmt == "RMULT" else 0,
        "allow_lo": "OutOfRangeLower" in spar,
        "allow_hi": "OutOfRangeUpper" in spar,
        "out_lo": float(value("OutOfRangeLower", "0")),
        "out_hi": float(value("OutOfRangeUpper", "0")),
        "values": values,
    }


class Table:
    """Spline table with the reference's coefficients (oracle side)."""

    def __init__(self, spec: dict):
        self.spec = spec
        n = spec["n"]
        self.a = np.zeros(n)
        self.b = np.zeros(n)
        self.c = np.zeros(n)
        self.d = np.array(spec["values"], dtype=np.float64)
        self.t = _Table(n, spec["dr"], spec["off"], spec["rmult"], int(spec["allow_lo"]), int(spec["allow_hi"]),
                        spec["out_lo"], spec["out_hi"], _dp(self.a), _dp(self.b), _dp(self.c), _dp(self.d))
        lib().oc_table_coef(ctypes.byref(self.t))

    @classmethod
    def from_file(cls, path, name=""):
        return cls(parse_table(path, name))

    def max_range(self):
        return self.spec["off"] + (self.spec["n"] - 1) * self.spec["dr"]

    def read(self, r):
        v = ctypes.c_double()
        dv = ctypes.c_double()
        if lib().oc_table_read(ctypes.byref(self.t), float(r), ctypes.byref(v), ctypes.byref(dv)):
            raise ValueError("table read out of range r=%r" % r)
        return v.value, dv.value


# ------------------------------------------------------------------ geometry

def make_box(lo, hi, periodic):
    b = _Box()
    for d in range(3):
        b.lo[d] = lo[d]
        b.hi[d] = hi[d]
        b.periodic[d] = int(periodic[d])
    return b


def wrap(box, x):
    x = np.ascontiguousarray(x, dtype=np.float64).copy()
    lib().oc_wrap(ctypes.byref(box), len(x), _dp(x))
    return x


def neighbors(box, x, rv, cap_per_atom=512, buffers=None):
    """Canonical neighbour tuples as CSR (offsets, j, code).  buffers: a
    reused (offsets, j, code) triple of int32 arrays; the result then views
    them (for timing loops)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    n = len(x)
    if buffers is None:
        cap = max(1, n * cap_per_atom)
        off = np.zeros(n + 1, dtype=np.int32)
        j = np.zeros(cap, dtype=np.int32)
        c = np.zeros(cap, dtype=np.int32)
    else:
        off, j, c = buffers
        cap = len(j)
    cnt = lib().oc_neighbors(ctypes.byref(box), n, _dp(x), float(rv), _ip(off), _ip(j), _ip(c), cap)
    if cnt < 0:
        raise RuntimeError("oc_neighbors failed (%d)" % cnt)
    if buffers is not None:
        return off, j[:cnt], c[:cnt]
    return off, j[:cnt].copy(), c[:cnt].copy()


def _forces(fn, box, x, nb, *params):
    x = np.ascontiguousarray(x, dtype=np.float64)
    n = len(x)
    off, j, c = nb
    f = np.zeros((n, 3))
    e = np.zeros(n)
    vir = np.zeros(n)
    extra = []
    args = [ctypes.byref(box), n, _dp(x), _ip(off), _ip(j), _ip(c)] + list(params) + [_dp(f), _dp(e), _dp(vir)]
    if fn == "oc_eam":
        rho = np.zeros(n)
        args.append(_dp(rho))
        extra = [rho]
    rc = getattr(lib(), fn)(*args)
    if rc:
        raise RuntimeError("%s failed (%d)" % (fn, rc))
    return (f, e, vir, *extra)


def eam(box, x, nb, phi: Table, edens: Table, embed: Table):
    return _forces("oc_eam", box, x, nb, ctypes.byref(phi.t), ctypes.byref(edens.t), ctypes.byref(embed.t))


def pair_table(box, x, nb, phi: Table):
    return _forces("oc_pair_table", box, x, nb, ctypes.byref(phi.t))


def pair_table_typed(box, x, types, ta, tb, nb, phi: Table, f, e, vir):
    x = np.ascontiguousarray(x, dtype=np.float64)
    types = np.ascontiguousarray(types, dtype=np.int32)
    off, j, c = nb
    rc = lib().oc_pair_table_typed(ctypes.byref(box), len(x), _dp(x), _ip(types), ta, tb, _ip(off), _ip(j), _ip(c),
                                   ctypes.byref(phi.t), _dp(f), _dp(e), _dp(vir))
    if rc:
        raise RuntimeError("oc_pair_table_typed failed")


def zbl(box, x, types, ta, tb, z1, z2, rc, width, nb, f=None, e=None, vir=None):
    """Universal ZBL (sw.cpp:118-146) on (ta, tb) pairs with omdg_add_zbl's
    switch over [rc - width, rc]; adds to f, e, vir (new arrays if None)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    types = np.ascontiguousarray(types, dtype=np.int32)
    n = len(x)
    f = np.zeros((n, 3)) if f is None else f
    e = np.zeros(n) if e is None else e
    vir = np.zeros(n) if vir is None else vir
    off, j, c = nb
    lib().oc_zbl(ctypes.byref(box), n, _dp(x), _ip(types), ta, tb, z1, z2, rc, width, _ip(off), _ip(j), _ip(c),
                 _dp(f), _dp(e), _dp(vir))
    return f, e, vir


def sw(box, x, nb, p: SWParam):
    return _forces("oc_sw", box, x, nb, ctypes.byref(p))


def tersoff(box, x, nb, p: TersoffParam):
    return _forces("oc_tersoff", box, x, nb, ctypes.byref(p))


def vv_kick_drift(x, v, f, mass, dt):
    lib().oc_vv_kick_drift(len(x), _dp(x), _dp(v), _dp(f), _dp(mass), float(dt))


def vv_kick(v, f, mass, dt):
    lib().oc_vv_kick(len(v), _dp(v), _dp(f), _dp(mass), float(dt))


def kinetic(v, mass):
    v = np.ascontiguousarray(v, dtype=np.float64)
    mass = np.ascontiguousarray(mass, dtype=np.float64)
    return lib().oc_kinetic(len(v), _dp(v), _dp(mass))


def berendsen_factor(dt, tau, tset, tnow):
    return lib().oc_berendsen_factor(dt, tau, tset, tnow)


# ------------------------------------------------------- reference executable

def run_reference(import_file, kind, table, steps=0, dt=0.001, skin=0.3, refresh=0, dump_nbr=False,
                  pair2=None, tcontrol=None, table_dir=None, swfix=False, time_only=False, timeout=3600, ttm=None,
                  save=None, cont=None, damp=None, clamp=None, dyndt=None, range_border=None, dump=None,
                  monitor=None, source=None, thermodump=False):
    """Run the reference's own code (oracle/_ref/ref_driver) on an Import file.

    Returns a dict with 'atoms' (nid, tid, x, v, f, potential, virial sorted
    by nid), optional 'nbr' tuples, 'ledger' rows and the summary values.
    save: write the reference's binary checkpoint there after the run;
    cont: resume from that checkpoint (steps is then the Step to stop at).
    damp (factor), clamp (axes), dyndt (maxpath, max, update), range_border:
    the impact-run modifies on every atom; the result then also holds 'times'
    (Step, TimeStep, ElapsedTime per step) and 'active' (nid, flag bit).
    thermodump: an intensive ThermoDetector whose data file of the final
    state is returned as 'thermo_dump' (bytes) with 'thermo' (nid T_i n_i).
    """
    exe = REF_DRIVER_SWFIX if swfix else REF_DRIVER
    if not os.path.exists(exe):
        raise FileNotFoundError(exe)
    out = tempfile.mkdtemp(prefix="omdref_")
    args = [exe, out, "import", os.path.abspath(import_file), "kind", kind, "table", table, "steps", str(steps),
            "dt", repr(dt), "skin", repr(skin), "refresh", str(refresh), "dump_nbr", "1" if dump_nbr else "0",
            "time_only", "1" if time_only else "0"]
    if pair2:
        args += ["pair2", pair2]
    if tcontrol:
        args += ["tcontrol", repr(tcontrol[0]), repr(tcontrol[1])]
    if damp is not None:
        args += ["damp", repr(float(damp))]
    if clamp is not None:
        args += ["clamp", clamp]
    if dyndt is not None:
        args += ["dyndt", repr(float(dyndt[0])), repr(float(dyndt[1])), str(int(dyndt[2]))]
    if range_border is not None:
        args += ["range", repr(float(range_border))]
    if source is not None:  # (energy per atom, start, width): EnergySource pulse
        args += ["source", repr(float(source[0])), repr(float(source[1])), repr(float(source[2]))]
    if dump:  # (file, write mode): DumpAtoms after the run
        args += ["dump", os.path.abspath(dump[0]), str(int(dump[1]))]
    if monitor:  # (file, every): SysMonitor
        args += ["monitor", os.path.abspath(monitor[0]), str(int(monitor[1]))]
    if thermodump:  # ThermoDetector's data file after the run: <out>/thermo.001
        args += ["thermodump", "thermo"]
    if save:
        args += ["save", os.path.abspath(save)]
    if cont:
        args += ["continue", os.path.abspath(cont)]
    if ttm:  # (electron-phonon table file, atom volume, initial electron temperature)
        args += ["ttm", os.path.abspath(ttm[0]), repr(float(ttm[1])), repr(float(ttm[2]))]
    env = dict(os.environ)
    if table_dir:
        env["OMD_TABLE"] = table_dir
    proc = subprocess.run(args, cwd=out, env=env, capture_output=True, text=True, timeout=timeout)
    if proc.returncode != 0:
        raise RuntimeError("reference run failed (%d): %s %s" % (proc.returncode, proc.stdout[-2000:],
                                                                 proc.stderr[-2000:]))
    res = {"dir": out, "stdout": proc.stdout}
    summ = {}
    sp = os.path.join(out, "summary.txt")
    if os.path.exists(sp):
        for line in open(sp):
            t = line.split()
            summ[t[0]] = [float(v) for v in t[1:]]
    res["summary"] = summ
    if time_only:
        return res
    a = np.loadtxt(os.path.join(out, "atoms.txt"), ndmin=2)
    res["atoms"] = a
    if dump_nbr:
        res["nbr"] = np.loadtxt(os.path.join(out, "nbr.txt"), dtype=np.int64, ndmin=2)
    lp = os.path.join(out, "ledger.txt")
    if os.path.exists(lp):
        res["ledger"] = np.loadtxt(lp, ndmin=2)
    for name in ("ttm", "thermo", "times", "active"):
        fp = os.path.join(out, name + ".txt")
        if os.path.exists(fp):
            res[name] = np.loadtxt(fp, ndmin=2)
    tp = os.path.join(out, "thermo.001")
    if os.path.exists(tp):
        res["thermo_dump"] = open(tp, "rb").read()
    return res
