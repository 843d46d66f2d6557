"""ctypes binding of libomdg's C ABI (include/omdg.h).

This is the thin host layer the Python tests, the benchmark and the plugin
mirror (objectmd_gb300.plugin) call.  It loads the in-tree
``objectmd_gb300/_build/libomdg.so`` and fails loudly when it is missing:
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libomdg.so")

OMDG_OK = 0
OMDG_STATIC_MAX_ATOMS = 131072  # include/omdg.h
OMDG_STATIC_MAX_CELLS = 32768
ERRORS = {
    -1: "OMDG_EINVAL",
    -2: "OMDG_ECUDA",
    -3: "OMDG_ERANGE",
    -4: "OMDG_EOVERLAP",
    -5: "OMDG_ENOMEM",
    -6: "OMDG_ESTATE",
    -7: "OMDG_EFILE",
    -8: "OMDG_ENONFINITE",
}

OMDG_EINVAL, OMDG_ECUDA, OMDG_ERANGE, OMDG_EOVERLAP = -1, -2, -3, -4
OMDG_ENOMEM, OMDG_ESTATE, OMDG_EFILE, OMDG_ENONFINITE = -5, -6, -7, -8

# every symbol include/omdg.h declares, with its ctypes signature
_P = ctypes.POINTER
_d, _i, _l, _vp, _cp = ctypes.c_double, ctypes.c_int, ctypes.c_long, ctypes.c_void_p, ctypes.c_char_p
_f = ctypes.c_float


# ---- the reference's binary checkpoint (include/omdg.h, checkpoints)
AUXVAR = 16
FLAG_ACTIVE = 1


class SimVars(ctypes.Structure):
    """MDSystem::SaveVariables (system.cpp:656-668)."""
    _fields_ = [("begin_time", ctypes.c_longlong), ("step", _i), ("pboundary", _i), ("energy", _d),
                ("kinetic", _d), ("virial", _d), ("potential", _d), ("base_potential", _d),
                ("elapsed_time", _d), ("box", _d * 12), ("write_mode", _i)]


class ContainerDesc(ctypes.Structure):
    """A container's saved header (container.cpp:566-581)."""
    _fields_ = [("name", ctypes.c_char * 256), ("material", ctypes.c_char * 256),
                ("filename", ctypes.c_char * 256), ("param", ctypes.c_char * 1024), ("id", _i), ("mass", _d),
                ("z", _d), ("value", _d), ("posprec", _i), ("valprec", _i), ("write_mode", _i), ("natoms", _i)]


# Atom (base.h:114-125): 232 bytes
ATOM_DTYPE = np.dtype([("tid", "<i4"), ("gid", "<i4"), ("nid", "<i4"), ("flag", "<i4"), ("x", "<f8"),
                       ("y", "<f8"), ("z", "<f8"), ("vx", "<f8"), ("vy", "<f8"), ("vz", "<f8"), ("fx", "<f8"),
                       ("fy", "<f8"), ("fz", "<f8"), ("potential", "<f8"), ("virial", "<f8"),
                       ("aux", "<f8", (AUXVAR,))])
assert ATOM_DTYPE.itemsize == 232


def container(name, natoms, id=0, mass=1.0, z=0.0, material="", filename="", param="", value=0.0, posprec=0,
              valprec=0, write_mode=0):
    d = ContainerDesc()
    d.name = name.encode()
    d.material = material.encode()
    d.filename = filename.encode()
    d.param = param.encode()
    d.id, d.mass, d.z, d.value = int(id), float(mass), float(z), float(value)
    d.posprec, d.valprec, d.write_mode, d.natoms = int(posprec), int(valprec), int(write_mode), int(natoms)
    return d


def _strings(items):
    arr = (_cp * max(1, len(items)))(*[x.encode() for x in items])
    return arr
SIGNATURES = {
    "omdg_create": [_P(_vp), _i],
    "omdg_destroy": [_vp],
    "omdg_last_error": [_vp],
    "omdg_get_stream": [_vp, _P(_vp)],
    "omdg_set_box": [_vp, _P(_d), _P(_d), _P(_i)],
    "omdg_set_atoms": [_vp, _i, _P(_d), _P(_d), _P(_i), _i, _P(_d), _P(_d)],
    "omdg_num_atoms": [_vp, _P(_i)],
    "omdg_get_state": [_vp, _P(_d), _P(_d), _P(_d), _P(_d), _P(_d)],
    "omdg_set_positions": [_vp, _P(_d)],
    "omdg_set_velocities": [_vp, _P(_d)],
    "omdg_set_state": [_vp, _P(_d), _P(_d)],
    "omdg_step_io": [_vp, _P(_d), _P(_d), _i, _P(_d), _P(_d), _P(_d)],
    "omdg_add_eam": [_vp, _i, _i, _cp],
    "omdg_add_pair_table": [_vp, _i, _i, _cp, _i],
    "omdg_add_sw": [_vp, _i, _i, _cp],
    "omdg_add_tersoff": [_vp, _i, _i, _cp],
    "omdg_add_zbl": [_vp, _i, _i, _d, _d],
    "omdg_max_cut_radius": [_vp, _P(_d)],
    "omdg_set_neighbor": [_vp, _d, _i],
    "omdg_build_neighbors": [_vp],
    "omdg_get_neighbors": [_vp, _P(_i), _P(_i), _P(_i), _l, _P(_l)],
    "omdg_compute_forces": [_vp],
    "omdg_set_timestep": [_vp, _d],
    "omdg_step": [_vp, _i],
    "omdg_step_async": [_vp, _i],
    "omdg_sync": [_vp],
    "omdg_set_first_step_mode": [_vp, _i],
    "omdg_ledger": [_vp, _P(_d), _P(_d), _P(_d), _P(_d)],
    "omdg_ledger_history": [_vp, _P(_d), _P(_d), _i, _P(_i)],
    "omdg_set_thermostat": [_vp, _d, _d],
    "omdg_set_compat": [_vp, _cp, _i],
    "omdg_stats": [_vp, _P(_l), _P(_l)],
    "omdg_wide_centres": [_vp, _P(_i)],
    "omdg_tile_counts": [_vp, _P(_i), _P(_i)],
    "omdg_set_wait_polls": [_i],
    "omdg_selftest_wait": [_i, _i, _P(ctypes.c_uint)],
    "omdg_set_launch": [_vp, _cp, _i],
    "omdg_get_launch": [_vp, _cp, _P(_i)],
    "omdg_autotune": [_vp, _i, _P(_d)],
    "omdg_set_profiling": [_vp, _i],
    "omdg_kernel_times": [_vp, _cp, _i, _P(_d), _P(_l), _i, _P(_i)],
    "omdg_count_neighbors_static": [_vp, _i, _P(_d), _P(_d), _P(_i), _d, _vp, _vp, _cp, _i],
    "omdg_set_replicas": [_vp, _i, _P(_i), _P(_d), _P(_d), _P(_i)],
    "omdg_replica_ledger": [_vp, _i, _P(_d), _P(_d)],
    "omdg_set_thermo_detector": [_vp, _i, _d],
    "omdg_local_thermo": [_vp, _P(_d), _P(_d), _P(_d)],
    "omdg_set_ttm": [_vp, _cp, _d, _d, _d],
    "omdg_set_ttm_grid": [_vp, _vp, _P(_d)],
    "omdg_replica_builds": [_vp, _P(_i), _i],
    "omdg_ttm_state": [_vp, _P(_d), _P(_d), _P(_d), _P(_d)],
    "omdg_add_nn": [_vp, _i, _i, _cp, _cp],
    "omdg_nn_fallback_atoms": [_vp, _P(_l)],
    "omdg_fdtd_create": [_P(_vp), _i, _i, _i, _i, _cp, _cp],
    "omdg_fdtd_destroy": [_vp],
    "omdg_fdtd_last_error": [_vp],
    "omdg_fdtd_set_timestep": [_vp, _d],
    "omdg_fdtd_set_spacestep": [_vp, _d],
    "omdg_fdtd_assign": [_vp, _i, _cp],
    "omdg_fdtd_step": [_vp, _i],
    "omdg_fdtd_get": [_vp, _i, _P(_d), _l],
    "omdg_fdtd_set_ext": [_vp, _P(_d), _l],
    "omdg_fdtd_info": [_vp, _P(_i), _P(_i), _P(_i), _P(_i)],
    "omdg_nn_create": [_P(_vp), _i],
    "omdg_nn_destroy": [_vp],
    "omdg_nn_last_error": [_vp],
    "omdg_nn_set_descriptors": [_vp, _P(_f), _P(_f), _P(_i), _P(_f), _P(_f)],
    "omdg_nn_set_cutoff": [_vp, _f, _f],
    "omdg_nn_set_dataset": [_vp, _i, _P(_i), _P(_d), _P(_d), _P(_d), _P(_d)],
    "omdg_nn_set_force_weighting": [_vp, _i],
    "omdg_nn_set_atom_energies": [_vp, _P(_d)],
    "omdg_nn_descriptors": [_vp, _P(_f), _l],
    "omdg_nn_normalize_from_dataset": [_vp],
    "omdg_nn_set_normalization": [_vp, _P(_f), _P(_f), _P(_f), _P(_f)],
    "omdg_nn_get_normalization": [_vp, _P(_f), _P(_f), _P(_f), _P(_f)],
    "omdg_nn_set_weights": [_vp, _P(_f), _l],
    "omdg_nn_get_weights": [_vp, _P(_f), _l],
    "omdg_nn_gradient": [_vp, _i, _i, _d, _d, _P(_d), _P(_f)],
    "omdg_nn_train": [_vp, _i, _i, _d, _d, _d, _d, ctypes.c_uint, _P(_d)],
    "omdg_nn_predict": [_vp, _i, _i, _i, _P(_d), _P(_d)],
    "omdg_nn_save": [_vp, _cp],
    "omdg_nn_load": [_vp, _cp],
    "omdg_set_groups": [_vp, _P(ctypes.c_ubyte)],
    "omdg_set_active": [_vp, _P(_i)],
    "omdg_get_active": [_vp, _P(_i)],
    "omdg_add_force_damper": [_vp, _i, _d],
    "omdg_add_coord_clamp": [_vp, _i, _cp],
    "omdg_add_range_limiter": [_vp, _i, _d],
    "omdg_set_dynamic_timestep": [_vp, _d, _d, _i],
    "omdg_get_timestep": [_vp, _P(_d), _P(_d)],
    "omdg_add_energy_source": [_vp, _d, _d, _d],
    "omdg_dump_atoms": [_vp, _cp, _i, _i, _i, _cp, _i, _P(_cp), _P(_i)],
    "omdg_dump_thermo": [_vp, _cp, _i, _i, _i, _cp, _i, _P(_cp), _cp, _P(_d)],
    "omdg_monitor_append": [_vp, _cp, _i, _i],
    "omdg_checkpoint_write": [_cp, _cp, _P(SimVars), _i, _P(_cp), _P(_cp), _i, _P(ContainerDesc), _vp, _cp, _i],
    "omdg_checkpoint_info": [_cp, _P(_i), _P(_i), _P(_i), _cp, _i],
    "omdg_checkpoint_read": [_cp, _P(SimVars), _cp, _i, _P(ContainerDesc), _i, _vp, _cp, _i, _cp, _i],
    "omdg_save_simulation": [_vp, _cp, _i, _P(ContainerDesc), _P(_i), _P(_i), _P(_d), _i, _P(_cp), _P(_cp)],
    "omdg_load_simulation": [_vp, _cp, _i, _P(ContainerDesc), _P(_i)],
}
STRING_RESULT = ("omdg_last_error", "omdg_nn_last_error", "omdg_fdtd_last_error")


class OMDGError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (ERRORS.get(code, str(code)), msg))
        self.code = code


_lib = None


def load(path: str = LIB_PATH):
    """Load libomdg.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError("libomdg.so not built (%s); run objectmd_gb300/build.py" % path)
    lib = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _cp if name in STRING_RESULT else _i
    _lib = lib
    return lib


def set_wait_polls(polls):
    """omdg_set_wait_polls: poll limit of the tensor-core kernels' waits (0: default)."""
    rc = load().omdg_set_wait_polls(int(polls))
    if rc != OMDG_OK:
        raise OMDGError(rc, "omdg_set_wait_polls(%d)" % polls)


def selftest_wait(which, polls):
    """omdg_selftest_wait: the status word after making a bounded wait run
    out (which 0: mbarrier in a TMEM-holding CTA, 1: grid barrier)."""
    st = ctypes.c_uint(0)
    rc = load().omdg_selftest_wait(int(which), int(polls), ctypes.byref(st))
    if rc != OMDG_OK:
        raise OMDGError(rc, "omdg_selftest_wait")
    return st.value


def count_neighbors_static(x_ptr, n, lo, hi, periodic, rcut, count_ptr, stream=None):
    """omdg_count_neighbors_static: per-atom neighbour counts for n*3 FP64
    positions at device address x_ptr into n ints at device address
    count_ptr, queued on `stream` (a cudaStream_t address; None = default
    stream).  Allocates no device memory; see include/omdg.h for the limits."""
    lib = load()
    lo3 = (_d * 3)(*[float(v) for v in lo])
    hi3 = (_d * 3)(*[float(v) for v in hi])
    per3 = (_i * 3)(*[1 if p else 0 for p in periodic])
    err = ctypes.create_string_buffer(256)
    rc = lib.omdg_count_neighbors_static(x_ptr, int(n), lo3, hi3, per3, float(rcut), count_ptr, stream, err, 256)
    if rc != OMDG_OK:
        raise OMDGError(rc, err.value.decode())


def checkpoint_write(path, vars, containers, atoms, restart_vars=(), stamp=None):
    """omdg_checkpoint_write (host only): vars a SimVars, containers a list of
    ContainerDesc, atoms an ATOM_DTYPE array (the containers' atoms back to
    back), restart_vars (label, value) string pairs."""
    lib = load()
    atoms = np.ascontiguousarray(atoms, dtype=ATOM_DTYPE)
    conts = (ContainerDesc * len(containers))(*containers)
    labels = _strings([l for l, _ in restart_vars])
    values = _strings([v for _, v in restart_vars])
    err = ctypes.create_string_buffer(256)
    rc = lib.omdg_checkpoint_write(path.encode(), None if stamp is None else stamp.encode(), ctypes.byref(vars),
                                   len(restart_vars), labels, values, len(containers), conts,
                                   atoms.ctypes.data_as(_vp), err, 256)
    if rc != OMDG_OK:
        raise OMDGError(rc, err.value.decode())


def checkpoint_read(path):
    """omdg_checkpoint_read (host only) -> (SimVars, stamp bytes, [ContainerDesc],
    ATOM_DTYPE array, [(label, value)])."""
    lib = load()
    err = ctypes.create_string_buffer(256)
    nc, na, nv = _i(), _i(), _i()
    rc = lib.omdg_checkpoint_info(path.encode(), ctypes.byref(nc), ctypes.byref(na), ctypes.byref(nv), err, 256)
    if rc != OMDG_OK:
        raise OMDGError(rc, err.value.decode())
    vars = SimVars()
    stamp = ctypes.create_string_buffer(32)
    conts = (ContainerDesc * max(1, nc.value))()
    atoms = np.zeros(na.value, dtype=ATOM_DTYPE)
    vlen = 1 << 20
    vbuf = ctypes.create_string_buffer(vlen)
    rc = lib.omdg_checkpoint_read(path.encode(), ctypes.byref(vars), stamp, nc.value, conts, na.value,
                                  atoms.ctypes.data_as(_vp), vbuf, vlen, err, 256)
    if rc != OMDG_OK:
        raise OMDGError(rc, err.value.decode())
    parts = vbuf.raw.split(b"\0")
    rv = [(parts[2 * k].decode(), parts[2 * k + 1].decode()) for k in range(nv.value)]
    return vars, stamp.raw, list(conts)[:nc.value], atoms, rv


NN_PARAMS = 6337  # W1[64x32] b1[64] W2[64x64] b2[64] w3[64] b3
NN_DESC = 32


def _fp(a):
    return None if a is None else a.ctypes.data_as(_P(_f))


class FDTD:
    """The finite-difference heat solver on one GPU (omdg_fdtd), with the
    reference's FDTDSolver interface: SetTimestep, SetSpacestep, SetCell,
    SetSource, SetConductivity, SetCapacity, Step, GetVector, GetExtVector."""

    CELL, SOURCE, CONDUCTIVITY, CAPACITY, EXT = range(5)

    def __init__(self, nx, ny, nz, symbol, map, device=0):
        self.lib = load()
        self.h = _vp()
        rc = self.lib.omdg_fdtd_create(ctypes.byref(self.h), int(device), int(nx), int(ny), int(nz),
                                       symbol.encode(), map.encode())
        if rc != OMDG_OK:
            msg = (self.lib.omdg_fdtd_last_error(self.h) or b"").decode() if self.h else "omdg_fdtd_create failed"
            self.close()
            raise OMDGError(rc, msg)
        a, b, c = _i(), _i(), _i()
        self._check(self.lib.omdg_fdtd_info(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), None))
        self.shape = (a.value, b.value, c.value)
        self.dim = a.value * b.value * c.value

    def _check(self, rc):
        if rc != OMDG_OK:
            raise OMDGError(rc, (self.lib.omdg_fdtd_last_error(self.h) or b"").decode())

    def close(self):
        if self.h:
            self.lib.omdg_fdtd_destroy(self.h)
            self.h = _vp()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_timestep(self, dt):
        self._check(self.lib.omdg_fdtd_set_timestep(self.h, float(dt)))

    def set_spacestep(self, h):
        self._check(self.lib.omdg_fdtd_set_spacestep(self.h, float(h)))

    def set_cell(self, s):
        self._check(self.lib.omdg_fdtd_assign(self.h, self.CELL, s.encode()))

    def set_source(self, s):
        self._check(self.lib.omdg_fdtd_assign(self.h, self.SOURCE, s.encode()))

    def set_conductivity(self, s):
        self._check(self.lib.omdg_fdtd_assign(self.h, self.CONDUCTIVITY, s.encode()))

    def set_capacity(self, s):
        self._check(self.lib.omdg_fdtd_assign(self.h, self.CAPACITY, s.encode()))

    def step(self, n=1):
        self._check(self.lib.omdg_fdtd_step(self.h, int(n)))

    def get(self, which=0):
        out = np.zeros(self.dim)
        self._check(self.lib.omdg_fdtd_get(self.h, int(which), _dp(out), self.dim))
        return out

    def vector(self):
        return self.get(self.CELL)

    def set_ext(self, e):
        e = np.ascontiguousarray(e, dtype=np.float64).ravel()
        self._check(self.lib.omdg_fdtd_set_ext(self.h, _dp(e), e.size))

    @property
    def steps_done(self):
        st = _i()
        self._check(self.lib.omdg_fdtd_info(self.h, None, None, None, ctypes.byref(st)))
        return st.value


class Network:
    """The neural surrogate's trainer on one GPU (omdg_nn)."""

    def __init__(self, device=0):
        self.lib = load()
        self.h = _vp()
        rc = self.lib.omdg_nn_create(ctypes.byref(self.h), int(device))
        if rc != OMDG_OK:
            raise OMDGError(rc, "omdg_nn_create failed (no usable GPU?)")
        self.natoms = 0

    def _check(self, rc):
        if rc != OMDG_OK:
            raise OMDGError(rc, (self.lib.omdg_nn_last_error(self.h) or b"").decode())

    def close(self):
        if self.h:
            self.lib.omdg_nn_destroy(self.h)
            self.h = _vp()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_descriptors(self, rs, eta_r, zeta, lam, eta_a):
        f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)  # noqa: E731
        rs, eta_r, lam, eta_a = f32(rs), f32(eta_r), f32(lam), f32(eta_a)
        zeta = np.ascontiguousarray(zeta, dtype=np.int32)
        self._check(self.lib.omdg_nn_set_descriptors(self.h, _fp(rs), _fp(eta_r), _ip(zeta), _fp(lam), _fp(eta_a)))

    def set_cutoff(self, rc, rin=0.0):
        """omdg_nn_set_cutoff: descriptor cutoff rc, switch starting at rin."""
        self._check(self.lib.omdg_nn_set_cutoff(self.h, rc, rin))

    def set_dataset(self, natoms, x, box_len, energy, forces):
        natoms = np.ascontiguousarray(natoms, dtype=np.int32)
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        box_len = np.ascontiguousarray(box_len, dtype=np.float64).reshape(-1, 3)
        energy = np.ascontiguousarray(energy, dtype=np.float64)
        forces = np.ascontiguousarray(forces, dtype=np.float64).reshape(-1, 3)
        self._check(self.lib.omdg_nn_set_dataset(self.h, len(natoms), _ip(natoms), _dp(x), _dp(box_len),
                                                 _dp(energy), _dp(forces)))
        self.natoms = int(natoms.sum())
        self.conf_start = np.concatenate([[0], np.cumsum(natoms)])

    def set_force_weighting(self, relative):
        self._check(self.lib.omdg_nn_set_force_weighting(self.h, 1 if relative else 0))

    def set_atom_energies(self, e_atom):
        e = None if e_atom is None else np.ascontiguousarray(e_atom, dtype=np.float64)
        self._check(self.lib.omdg_nn_set_atom_energies(self.h, _dp(e)))

    def descriptors(self):
        G = np.zeros((self.natoms, NN_DESC), dtype=np.float32)
        self._check(self.lib.omdg_nn_descriptors(self.h, _fp(G), G.size))
        return G

    def normalize_from_dataset(self):
        self._check(self.lib.omdg_nn_normalize_from_dataset(self.h))

    def set_normalization(self, mu, sigma, gmin=None, gmax=None):
        arr = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float32)  # noqa: E731
        mu, sigma, gmin, gmax = arr(mu), arr(sigma), arr(gmin), arr(gmax)
        self._check(self.lib.omdg_nn_set_normalization(self.h, _fp(mu), _fp(sigma), _fp(gmin), _fp(gmax)))

    def normalization(self):
        out = [np.zeros(NN_DESC, dtype=np.float32) for _ in range(4)]
        self._check(self.lib.omdg_nn_get_normalization(self.h, *[_fp(a) for a in out]))
        return dict(zip(("mu", "sigma", "gmin", "gmax"), out))

    def set_weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        self._check(self.lib.omdg_nn_set_weights(self.h, _fp(w), w.size))

    def weights(self):
        w = np.zeros(NN_PARAMS, dtype=np.float32)
        self._check(self.lib.omdg_nn_get_weights(self.h, _fp(w), w.size))
        return w

    def gradient(self, conf0, nconf, wE, wF):
        loss = _d()
        g = np.zeros(NN_PARAMS, dtype=np.float32)
        self._check(self.lib.omdg_nn_gradient(self.h, int(conf0), int(nconf), float(wE), float(wF),
                                              ctypes.byref(loss), _fp(g)))
        return loss.value, g

    def train(self, epochs, batch_confs, lr, wE, wF, seed=7, lr_final=None):
        hist = np.zeros(int(epochs))
        lr_final = lr if lr_final is None else lr_final
        self._check(self.lib.omdg_nn_train(self.h, int(epochs), int(batch_confs), float(lr), float(lr_final),
                                           float(wE), float(wF), int(seed), _dp(hist)))
        return hist

    def predict(self, conf0, nconf, fp32=False):
        n = int(self.conf_start[conf0 + nconf] - self.conf_start[conf0])
        e = np.zeros(n)
        f = np.zeros((n, 3))
        self._check(self.lib.omdg_nn_predict(self.h, int(conf0), int(nconf), 1 if fp32 else 0, _dp(e), _dp(f)))
        return e, f

    def save(self, path):
        self._check(self.lib.omdg_nn_save(self.h, path.encode()))

    def load(self, path):
        self._check(self.lib.omdg_nn_load(self.h, path.encode()))


def _dp(a):
    return None if a is None else a.ctypes.data_as(_P(_d))


def _ip(a):
    return None if a is None else a.ctypes.data_as(_P(_i))


class Context:
    """One simulation box on one GPU (omdg_ctx)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        self.h = _vp()
        self._check(self.lib.omdg_create(ctypes.byref(self.h), device), "omdg_create")
        self.n = 0

    def _check(self, rc, what=""):
        if rc != OMDG_OK:
            msg = self.lib.omdg_last_error(self.h).decode() if self.h else what
            raise OMDGError(rc, msg or what)

    def close(self):
        if self.h:
            self.lib.omdg_destroy(self.h)
            self.h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---------------------------------------------------------------- setup
    def set_box(self, lo, hi, periodic=(True, True, True)):
        lo = np.ascontiguousarray(lo, dtype=np.float64)
        hi = np.ascontiguousarray(hi, dtype=np.float64)
        p = np.ascontiguousarray([1 if q else 0 for q in periodic], dtype=np.int32)
        self._check(self.lib.omdg_set_box(self.h, _dp(lo), _dp(hi), _ip(p)))

    def set_atoms(self, x, v=None, types=None, masses=(1.0,), znum=None):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        n = len(x)
        v = None if v is None else np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
        t = np.zeros(n, dtype=np.int32) if types is None else np.ascontiguousarray(types, dtype=np.int32)
        m = np.ascontiguousarray(masses, dtype=np.float64)
        z = None if znum is None else np.ascontiguousarray(znum, dtype=np.float64)
        self._check(self.lib.omdg_set_atoms(self.h, n, _dp(x), _dp(v), _ip(t), len(m), _dp(m), _dp(z)))
        self.n = n

    def num_atoms(self):
        """omdg_num_atoms: the library's atom count (host buffers are sized from it)."""
        n = _i()
        self._check(self.lib.omdg_num_atoms(self.h, ctypes.byref(n)))
        self.n = n.value
        return n.value

    def get_state(self):
        n = self.num_atoms()
        x = np.zeros((n, 3))
        v = np.zeros((n, 3))
        f = np.zeros((n, 3))
        e = np.zeros(n)
        w = np.zeros(n)
        self._check(self.lib.omdg_get_state(self.h, _dp(x), _dp(v), _dp(f), _dp(e), _dp(w)))
        return {"x": x, "v": v, "f": f, "pot": e, "vir": w}

    def set_positions(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        self._check(self.lib.omdg_set_positions(self.h, _dp(x)))

    def set_velocities(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
        self._check(self.lib.omdg_set_velocities(self.h, _dp(v)))

    def set_state(self, x=None, v=None):
        """Positions and/or velocities in one call (pinned arrays are read in place)."""
        x = None if x is None else np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        v = None if v is None else np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
        self._check(self.lib.omdg_set_state(self.h, _dp(x), _dp(v)))

    def add_eam(self, table_file, ta=0, tb=0):
        self._check(self.lib.omdg_add_eam(self.h, ta, tb, table_file.encode()))

    def add_pair_table(self, table_file, ta=0, tb=0, fp64=False):
        self._check(self.lib.omdg_add_pair_table(self.h, ta, tb, table_file.encode(), 1 if fp64 else 0))

    def add_sw(self, param_file, ta=0, tb=0):
        self._check(self.lib.omdg_add_sw(self.h, ta, tb, param_file.encode()))

    def add_tersoff(self, param_file, ta=0, tb=0):
        self._check(self.lib.omdg_add_tersoff(self.h, ta, tb, param_file.encode()))

    def add_zbl(self, ta, tb, rc, width):
        self._check(self.lib.omdg_add_zbl(self.h, ta, tb, float(rc), float(width)))

    def set_replicas(self, natoms, lo, hi, periodic=(1, 1, 0)):
        natoms = np.ascontiguousarray(natoms, dtype=np.int32)
        lo = np.ascontiguousarray(lo, dtype=np.float64).reshape(-1, 3)
        hi = np.ascontiguousarray(hi, dtype=np.float64).reshape(-1, 3)
        per = (ctypes.c_int * 3)(*[1 if p else 0 for p in periodic])
        self._check(self.lib.omdg_set_replicas(self.h, len(natoms), _ip(natoms), _dp(lo), _dp(hi), per))
        self.nrep = len(natoms)

    def replica_ledger(self):
        k = np.zeros(self.nrep)
        p = np.zeros(self.nrep)
        self._check(self.lib.omdg_replica_ledger(self.h, self.nrep, _dp(k), _dp(p)))
        return k, p

    def set_thermo_detector(self, on=True, ercut=-1.0):
        self._check(self.lib.omdg_set_thermo_detector(self.h, 1 if on else 0, float(ercut)))

    def local_thermo(self):
        t, d, v = np.zeros(self.n), np.zeros(self.n), np.zeros((self.n, 3))
        self._check(self.lib.omdg_local_thermo(self.h, _dp(t), _dp(d), _dp(v)))
        return {"temperature": t, "density": d, "vcm": v}

    def set_ttm(self, table_file, atom_volume, electron_temperature=-1.0, pulse_offset=0.0):
        self._check(self.lib.omdg_set_ttm(self.h, table_file.encode(), float(atom_volume),
                                          float(electron_temperature), float(pulse_offset)))

    def set_ttm_grid(self, grid, origin=(0.0, 0.0, 0.0)):
        """omdg_set_ttm_grid: the electron temperature on an FDTD grid's cells
        (None detaches)."""
        o = np.ascontiguousarray(origin, dtype=np.float64)
        self._check(self.lib.omdg_set_ttm_grid(self.h, grid.h if grid is not None else None, _dp(o)))
        self._ttm_grid = grid  # keep it alive while coupled

    def ttm_state(self):
        te, een, aen, tl = _d(), _d(), _d(), _d()
        self._check(self.lib.omdg_ttm_state(self.h, ctypes.byref(te), ctypes.byref(een), ctypes.byref(aen),
                                            ctypes.byref(tl)))
        return {"electron_temperature": te.value, "int_een": een.value, "int_aen": aen.value,
                "lattice_temperature": tl.value}

    def add_nn(self, model_file, tersoff_fallback=None, ta=0, tb=0):
        fb = tersoff_fallback.encode() if tersoff_fallback else None
        self._check(self.lib.omdg_add_nn(self.h, ta, tb, model_file.encode(), fb))

    def nn_fallback_atoms(self):
        n = _l()
        self._check(self.lib.omdg_nn_fallback_atoms(self.h, ctypes.byref(n)))
        return n.value

    def max_cut_radius(self):
        r = _d()
        self._check(self.lib.omdg_max_cut_radius(self.h, ctypes.byref(r)))
        return r.value

    def set_neighbor(self, skin=0.3, rebuild_every=0):
        self._check(self.lib.omdg_set_neighbor(self.h, float(skin), int(rebuild_every)))

    def build_neighbors(self):
        self._check(self.lib.omdg_build_neighbors(self.h))

    def neighbors(self):
        """Canonical tuples as CSR (offsets, j, code), rows sorted by (j, code)."""
        n = self.n
        off = np.zeros(n + 1, dtype=np.int32)
        cnt = _l()
        rc = self.lib.omdg_get_neighbors(self.h, _ip(off), None, None, 0, ctypes.byref(cnt))
        if rc not in (OMDG_OK, -1):
            self._check(rc)
        j = np.zeros(max(1, cnt.value), dtype=np.int32)
        c = np.zeros(max(1, cnt.value), dtype=np.int32)
        self._check(self.lib.omdg_get_neighbors(self.h, _ip(off), _ip(j), _ip(c), cnt.value, ctypes.byref(cnt)))
        return off, j[:cnt.value], c[:cnt.value]

    # ----------------------------------------------------------------- run
    def compute_forces(self):
        self._check(self.lib.omdg_compute_forces(self.h))

    def set_timestep(self, dt):
        self._check(self.lib.omdg_set_timestep(self.h, float(dt)))

    def set_first_step_mode(self, reference=True):
        self._check(self.lib.omdg_set_first_step_mode(self.h, 1 if reference else 0))

    def set_thermostat(self, temperature, tau):
        self._check(self.lib.omdg_set_thermostat(self.h, float(temperature), float(tau)))

    def set_compat(self, key, on=True):
        self._check(self.lib.omdg_set_compat(self.h, key.encode(), 1 if on else 0))

    def step(self, nsteps=1):
        self._check(self.lib.omdg_step(self.h, int(nsteps)))

    def step_io(self, nsteps=1, x_in=None, v_in=None, x_out=None, v_out=None, f_out=None):
        """Upload, nsteps steps and read-back in one call (omdg_step_io); outputs are
        caller-provided float64 (n, 3) arrays, written in place (pinned ones while
        the last step runs)."""
        arr = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64).reshape(-1, 3)  # noqa: E731
        for a in (x_out, v_out, f_out):
            if a is not None and not (a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]):
                raise ValueError("outputs must be C-contiguous float64 arrays")
        self._check(self.lib.omdg_step_io(self.h, _dp(arr(x_in)), _dp(arr(v_in)), int(nsteps), _dp(x_out),
                                          _dp(v_out), _dp(f_out)))

    def step_async(self, nsteps=1):
        self._check(self.lib.omdg_step_async(self.h, int(nsteps)))

    def sync(self):
        self._check(self.lib.omdg_sync(self.h))

    def get_state_into(self, x=None, v=None, f=None, pot=None, vir=None):
        """Read state into caller-provided float64 arrays (e.g. pinned buffers)."""
        self._check(self.lib.omdg_get_state(self.h, _dp(x), _dp(v), _dp(f), _dp(pot), _dp(vir)))

    def ledger(self):
        k, p, b, w = _d(), _d(), _d(), _d()
        self._check(self.lib.omdg_ledger(self.h, ctypes.byref(k), ctypes.byref(p), ctypes.byref(b), ctypes.byref(w)))
        return {"kinetic": k.value, "potential": p.value, "base_potential": b.value, "virial": w.value,
                "energy": k.value + p.value - b.value}

    # ---- output
    WM = {"append": 1, "velocity": 2, "force": 4, "deadatom": 8, "bare": 16, "ghost": 32, "potential": 64,
          "virial": 128, "tid": 256, "gid": 512, "nid": 1024}

    def dump_atoms(self, path, mode, posprec=5, valprec=5, material="", info=(), gid=None):
        """omdg_dump_atoms: the reference's data file (mode: WM_* bits or names)."""
        if not isinstance(mode, int):
            mode = sum(self.WM[m] for m in mode)
        g = None if gid is None else np.ascontiguousarray(gid, dtype=np.int32)
        lines = _strings(list(info))
        self._check(self.lib.omdg_dump_atoms(self.h, path.encode(), int(mode), int(posprec), int(valprec),
                                             material.encode(), len(info), lines, None if g is None else _ip(g)))

    def dump_thermo(self, path, mode=0, posprec=5, valprec=5, material="", info=(), aux_format=None):
        """omdg_dump_thermo: ThermoDetector's data file of the current state; returns the
        system temperature and pressure and the local averages."""
        if not isinstance(mode, int):
            mode = sum(self.WM[m] for m in mode)
        lines = _strings(list(info))
        out = (_d * 5)()
        self._check(self.lib.omdg_dump_thermo(self.h, path.encode(), int(mode), int(posprec), int(valprec),
                                              material.encode(), len(info), lines,
                                              aux_format.encode() if aux_format else None, out))
        return dict(zip(("temperature", "pressure", "avg_temperature", "avg_density", "avg_pressure"), out))

    def monitor_append(self, path, every=1, header=False):
        """omdg_monitor_append: SysMonitor's md.out lines of the last step call."""
        self._check(self.lib.omdg_monitor_append(self.h, path.encode(), int(every), 1 if header else 0))

    # ---- modifies of the impact runs
    def set_groups(self, member):
        """member: per atom, bit g set = in group g (0..7)."""
        m = np.ascontiguousarray(member, dtype=np.uint8)
        self._check(self.lib.omdg_set_groups(self.h, m.ctypes.data_as(_P(ctypes.c_ubyte))))

    def set_active(self, active):
        a = np.ascontiguousarray(active, dtype=np.int32)
        self._check(self.lib.omdg_set_active(self.h, _ip(a)))

    def get_active(self):
        a = np.zeros(self.num_atoms(), dtype=np.int32)
        self._check(self.lib.omdg_get_active(self.h, _ip(a)))
        return a.astype(bool)

    def add_force_damper(self, group, factor):
        self._check(self.lib.omdg_add_force_damper(self.h, int(group), float(factor)))

    def add_coord_clamp(self, group, axes="xyz"):
        self._check(self.lib.omdg_add_coord_clamp(self.h, int(group), axes.encode()))

    def add_range_limiter(self, group, border):
        self._check(self.lib.omdg_add_range_limiter(self.h, int(group), float(border)))

    def set_dynamic_timestep(self, maxpath, max_dt=0.001, update=5):
        self._check(self.lib.omdg_set_dynamic_timestep(self.h, float(maxpath), float(max_dt), int(update)))

    def add_energy_source(self, energy, start, width):
        self._check(self.lib.omdg_add_energy_source(self.h, float(energy), float(start), float(width)))

    def get_timestep(self):
        dt, el = _d(), _d()
        self._check(self.lib.omdg_get_timestep(self.h, ctypes.byref(dt), ctypes.byref(el)))
        return dt.value, el.value

    def save_simulation(self, path, containers, gid=None, flag=None, aux=None, restart_vars=()):
        """omdg_save_simulation: the reference's checkpoint from this context."""
        conts = (ContainerDesc * len(containers))(*containers)
        g = None if gid is None else np.ascontiguousarray(gid, dtype=np.int32)
        f = None if flag is None else np.ascontiguousarray(flag, dtype=np.int32)
        a = None if aux is None else np.ascontiguousarray(aux, dtype=np.float64)
        labels = _strings([l for l, _ in restart_vars])
        values = _strings([v for _, v in restart_vars])
        self._check(self.lib.omdg_save_simulation(self.h, path.encode(), len(containers), conts,
                                                  None if g is None else _ip(g), None if f is None else _ip(f),
                                                  None if a is None else _dp(a), len(restart_vars), labels, values))

    def load_simulation(self, path, cap=64):
        """omdg_load_simulation: resume from a checkpoint; returns its containers."""
        conts = (ContainerDesc * cap)()
        nc = _i()
        self._check(self.lib.omdg_load_simulation(self.h, path.encode(), cap, conts, ctypes.byref(nc)))
        self.num_atoms()
        return list(conts)[:min(cap, nc.value)]

    def ledger_history(self, cap=1 << 16):
        k = np.zeros(cap)
        p = np.zeros(cap)
        rows = _i()
        self._check(self.lib.omdg_ledger_history(self.h, _dp(k), _dp(p), cap, ctypes.byref(rows)))
        return k[:rows.value].copy(), p[:rows.value].copy()

    def stats(self):
        r, l = _l(), _l()
        self._check(self.lib.omdg_stats(self.h, ctypes.byref(r), ctypes.byref(l)))
        return {"rebuilds": r.value, "launches": l.value}

    def replica_builds(self, nrep):
        """omdg_replica_builds: list builds per replica."""
        out = np.zeros(int(nrep), dtype=np.int32)
        self._check(self.lib.omdg_replica_builds(self.h, _ip(out), int(nrep)))
        return out

    def wide_centres(self):
        """Centres the last SW/Tersoff force pass sent to the dense second pass."""
        k = _i()
        self._check(self.lib.omdg_wide_centres(self.h, ctypes.byref(k)))
        return k.value

    def tile_counts(self):
        """omdg_tile_counts: (tiles of the last build, tiles staged in shared memory)."""
        t, st = _i(), _i()
        self._check(self.lib.omdg_tile_counts(self.h, ctypes.byref(t), ctypes.byref(st)))
        return t.value, st.value

    def stream(self):
        s = _vp()
        self._check(self.lib.omdg_get_stream(self.h, ctypes.byref(s)))
        return s.value

    def set_launch(self, key, value):
        self._check(self.lib.omdg_set_launch(self.h, key.encode(), int(value)))

    def get_launch(self, key):
        v = _i()
        self._check(self.lib.omdg_get_launch(self.h, key.encode(), ctypes.byref(v)))
        return v.value

    def launch_shapes(self):
        keys = ("eam_block", "eam_lanes", "eam_stage", "eam_ctas_per_sm", "pair_block", "pair_lanes", "tb_block",
                "tb_lanes", "tb_persistent", "fuse_kick", "nbr_hshift", "build_lanes", "io_blocks", "nn_fused", "eam_tile",
                "tile_x", "tile_y", "tile_z", "tile_cap")
        return {k: self.get_launch(k) for k in keys}

    def autotune(self, reps=3):
        ms = _d()
        self._check(self.lib.omdg_autotune(self.h, int(reps), ctypes.byref(ms)))
        return ms.value

    def set_profiling(self, on=True):
        self._check(self.lib.omdg_set_profiling(self.h, 1 if on else 0))

    def kernel_times(self, cap=64):
        buf = ctypes.create_string_buffer(4096)
        ms = np.zeros(cap)
        calls = np.zeros(cap, dtype=np.int64)
        nk = _i()
        self._check(self.lib.omdg_kernel_times(self.h, buf, 4096, _dp(ms), calls.ctypes.data_as(_P(_l)), cap,
                                               ctypes.byref(nk)))
        names = buf.value.decode().split(";") if nk.value else []
        return {names[k]: (float(ms[k]), int(calls[k])) for k in range(nk.value)}
