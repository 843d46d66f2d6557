"""Generates the golden fixtures under tests/golden/ from the REFERENCE's own code.

Run here, where the Object-MD sources exist (python tests/golden/make_golden.py);
the GPU tests only read the committed outputs.  Steps:

1. Build the reference CPU path (oracle/ref/Makefile -> oracle/_ref/ref_driver*).
2. Write the tables the configurations use into tests/golden/tables/:
   - eam.aluminum5000: the reference's tables/eam.aluminum (PAIR, EDENS,
     EMBED; 1000 knots each) resampled to 5000 knots over the same ranges by
     evaluating the reference spline (TableReader::read restated in
     oracle/omd_oracle.c, which is pinned to the reference below);
   - pair.lj.argon: analytic 12-6 LJ (sigma 3.405, eps 0.0104, rc 2.5 sigma);
   - sw.silicon and tersoff.silicon27 parameter files.
3. Generate seeded atom configurations (objectmd_gb300.inputs) and run the
   reference on them: static forces, per-atom energies, virials and the
   neighbour tuples, plus a short NVE trajectory.  The reference's own test
   inputs are run too: its silicon clusters (test/check-verlet-list), its
   impact replica (test/si-impact/atom.dat) and the two-element combination
   of test/two_elements/two.cpp on a generated Pt slab.
4. Save each case as <case>.npz with its Import file.

A single group of cases: python tests/golden/make_golden.py <name> with
<name> one of ttm, checkpoint, output, thermo, modifies, impact, fdtd,
example, lj4000, clusters, impact_replica, ar_pt.
"""
from __future__ import annotations

import os
import shutil
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from objectmd_gb300 import inputs  # noqa: E402
from oracle import oracle as oc  # noqa: E402

REF = os.environ.get("OMD_REFERENCE", "")  # the Object-MD source tree (required to generate)
GOLD = os.path.join(ROOT, "tests", "golden")
TABLES = os.path.join(GOLD, "tables")


def resample_section(spec: dict, n_new: int):
    """Evaluate the reference spline of one table section on a finer grid.

    The stored quantity is resampled (for RMULT tables that is r*phi), so the
    new table reads back the same function through TableReader semantics.
    """
    t = oc.Table(dict(spec, rmult=0))
    lo = spec["off"]
    hi = spec["off"] + (spec["n"] - 1) * spec["dr"]
    dr = (hi - lo) / (n_new - 1)
    r = lo + dr * np.arange(n_new)
    r[-1] = min(r[-1], hi)
    vals = np.array([t.read(x)[0] for x in r])
    return dr, lo, vals


def write_eam5000(path):
    src = os.path.join(REF, "tables", "eam.aluminum")
    out = ["# Object-MD table: tables/eam.aluminum resampled to 5000 knots per section",
           "# (reference spline evaluated at the new knots; same ranges and formats)"]
    for name in ("PAIR", "EDENS", "EMBED"):
        spec = oc.parse_table(src, name)
        dr, off, vals = resample_section(spec, 5000)
        out.append("#$%s NumberOfData %d" % (name, 5000))
        out.append("#$%s Spacing %.17g" % (name, dr))
        out.append("#$%s Offset %.17g" % (name, off))
        if spec["rmult"]:
            out.append("#$%s Format RMULT" % name)
        out.append("#$%s --" % name)
        out += ["%.17g" % v for v in vals]
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")


def table_dir():
    """OMD_TABLE for reference runs: the reference tables plus the generated ones."""
    d = tempfile.mkdtemp(prefix="omdtab_")
    if REF:
        for f in os.listdir(os.path.join(REF, "tables")):
            os.symlink(os.path.join(REF, "tables", f), os.path.join(d, f))
    for f in os.listdir(TABLES):
        dst = os.path.join(d, f)
        if os.path.lexists(dst):
            os.remove(dst)
        os.symlink(os.path.join(TABLES, f), dst)
    return d


def save_case(name, import_file, res, **extra):
    a = res["atoms"]
    payload = dict(nid=a[:, 0].astype(np.int32), tid=a[:, 1].astype(np.int32), x=a[:, 2:5], v=a[:, 5:8],
                   f=a[:, 8:11], pot=a[:, 11], vir=a[:, 12])
    if "nbr" in res:
        payload["nbr"] = res["nbr"].astype(np.int32)
    if "ledger" in res:
        payload["ledger"] = res["ledger"]
    for k in ("potential", "kinetic", "base_potential", "virial", "max_cut_radius"):
        if k in res["summary"]:
            payload["summary_" + k] = np.array(res["summary"][k])
    payload.update(extra)
    np.savez_compressed(os.path.join(GOLD, name + ".npz"), **payload)
    shutil.copy(import_file, os.path.join(GOLD, name + ".dat"))
    print("wrote", name, "atoms", len(a), "tuples", len(res.get("nbr", [])))


def ttm_case(tdir, work):
    """TTM_Homogen with an intensive ThermoDetector on a free EAM Al cluster
    (no periodic images: no ghost atoms): electron temperature trace, kinetic
    trace and the final per-atom local temperatures and densities."""
    with open(os.path.join(TABLES, "ttm.aluminum"), "w") as fh:
        fh.write(inputs.ttm_table_text())
    x, v, (lo, hi) = inputs.aluminium_cluster(ncell=6, temp=300.0)
    f = os.path.join(work, "ttm_al_cluster.dat")
    inputs.write_import(f, x, v, box=(lo, hi), periodic=(False, False, False), species=("aluminum",))
    vol, te0, steps, dt = 16.6, 5000.0, 60, 0.002
    res = oc.run_reference(f, "eam", "aluminum5000", steps=steps, dt=dt, table_dir=tdir,
                           ttm=(os.path.join(TABLES, "ttm.aluminum"), vol, te0))
    th = res["thermo"]
    save_case("ttm_al_cluster", f, res, box_lo=lo, box_hi=hi, steps=np.array(steps), dt=np.array(dt),
              atom_volume=np.array(vol), te0=np.array(te0), ttm=res["ttm"], local_temp=th[:, 1], local_dens=th[:, 2])


def checkpoint_case(tdir):
    """The reference's own binary checkpoint: EAM Al 500 saved after 5 steps
    (MDSystemGrid::SaveSimulation), and its state at Step 10, continued from
    that file (CONTINUE_MODE).  The file is stored compressed in an npz."""
    f = os.path.join(GOLD, "eam_al_500.dat")
    path = os.path.join(tempfile.mkdtemp(prefix="omdck_"), "eam_al_500.bin")
    oc.run_reference(f, "eam", "aluminum5000", steps=5, dt=0.002, table_dir=tdir, save=path)
    res = oc.run_reference(f, "eam", "aluminum5000", steps=10, dt=0.002, table_dir=tdir, cont=path)
    a = res["atoms"]
    raw = np.frombuffer(open(path, "rb").read(), dtype=np.uint8)
    np.savez_compressed(os.path.join(GOLD, "checkpoint_eam_al_500.npz"), binary=raw, dt=np.array(0.002),
                        x10=a[:, 2:5], v10=a[:, 5:8], f10=a[:, 8:11], pot10=a[:, 11], ledger=res["ledger"])
    print("wrote checkpoint_eam_al_500", raw.size, "bytes")


def output_case(tdir):
    """The reference's output path on EAM Al 500, 6 steps of 2 fs:
    DumpAtoms (velocity, force, potential, id, nid) and SysMonitor's md.out
    every 2 steps; a second run writes DumpAtoms (velocity, id, nid) and the
    binary checkpoint of the same final state."""
    f = os.path.join(GOLD, "eam_al_500.dat")
    work = tempfile.mkdtemp(prefix="omdout_")
    dump1, md, dump2, ck = (os.path.join(work, n) for n in ("dump1.dat", "md.out", "dump2.dat", "final.bin"))
    oc.run_reference(f, "eam", "aluminum5000", steps=6, dt=0.002, table_dir=tdir, dump=(dump1, 2 | 4 | 64 | 256 | 1024),
                     monitor=(md, 2))
    oc.run_reference(f, "eam", "aluminum5000", steps=6, dt=0.002, table_dir=tdir, dump=(dump2, 2 | 256 | 1024),
                     save=ck)
    raw = lambda p: np.frombuffer(open(p, "rb").read(), dtype=np.uint8)  # noqa: E731
    np.savez_compressed(os.path.join(GOLD, "output_eam_al_500.npz"), dump_full=raw(dump1), monitor=raw(md),
                        dump_state=raw(dump2), checkpoint=raw(ck), dt=np.array(0.002), steps=np.array(6))
    print("wrote output_eam_al_500")


def thermo_case(tdir):
    """ThermoDetector's data file (intensive, ercut = the EAM cutoff) of EAM
    Al FCC 8^3 = 2048 atoms (periodic, 300 K) after 6 steps of 2 fs, with the
    binary checkpoint of the same state.  The box is large enough for atoms
    farther than two cutoffs from every face, where the reference's ghost
    copies do not enter the local temperatures."""
    x, v, (lo, hi) = inputs.eam_aluminium(ncell=8, a=4.05, sigma=0.05, temp=300.0, seed_pos=12, seed_vel=13)
    work = tempfile.mkdtemp(prefix="omdthermo_")
    f = os.path.join(work, "eam_al_2048.dat")
    inputs.write_import(f, x, v, box=(lo, hi), periodic=(True, True, True), species=("aluminum",))
    ck = os.path.join(work, "final.bin")
    res = oc.run_reference(f, "eam", "aluminum5000", steps=6, dt=0.002, table_dir=tdir, thermodump=True, save=ck)
    raw = lambda b: np.frombuffer(b, dtype=np.uint8)  # noqa: E731
    # SysMonitor with the detector's slots, every 2 of 6 steps, on a free EAM
    # Al cluster (no ghost copies: the local averages are the reference's too)
    cx, cv, (clo, chi) = inputs.aluminium_cluster(ncell=6, temp=300.0)
    cf = os.path.join(work, "al_cluster.dat")
    inputs.write_import(cf, cx, cv, box=(clo, chi), periodic=(False, False, False), species=("aluminum",))
    md = os.path.join(work, "md.out")
    oc.run_reference(cf, "eam", "aluminum5000", steps=6, dt=0.002, table_dir=tdir, thermodump=True, monitor=(md, 2))
    np.savez_compressed(os.path.join(GOLD, "thermo_eam_al_2048.npz"), thermo_dump=raw(res["thermo_dump"]),
                        checkpoint=raw(open(ck, "rb").read()), thermo=res["thermo"], monitor=raw(open(md, "rb").read()),
                        cluster_x=cx, cluster_v=cv, cluster_lo=clo, cluster_hi=chi)
    print("wrote thermo_eam_al_2048")


MODIFY_CASES = {  # the impact-run modifies on every atom of an EAM Al slab
    "damp_clamp": dict(damp=0.05, clamp="xyz"),
    "dyndt": dict(dyndt=(0.02, 0.004, 3)),
    "range": dict(range_border=1.0),
    "source": dict(source=(0.05, 0.01, 0.02)),
}


def modifies_case(tdir, work):
    """EAM Al 500-atom slab (free z), its top atom launched upward at 60 A/ps,
    30 steps of 2 fs with ForceDamper + CoordClamp, DynamicTimeStep or
    RangeLimiter: the reference's trajectories, time steps and active flags."""
    x, v, (lo, hi) = inputs.eam_aluminium(ncell=5, a=4.05, sigma=0.05, temp=300.0, seed_pos=41, seed_vel=42)
    top = int(np.argmax(x[:, 2]))
    v[top] = [5.0, -3.0, 60.0]
    f = os.path.join(work, "eam_al_slab.dat")
    inputs.write_import(f, x, v, box=(lo, hi), periodic=(True, True, False), species=("aluminum",))
    out = dict(box_lo=lo, box_hi=hi, top=np.array(top), steps=np.array(30), dt=np.array(0.002))
    for name, kw in MODIFY_CASES.items():
        res = oc.run_reference(f, "eam", "aluminum5000", steps=30, dt=0.002, table_dir=tdir, **kw)
        a = res["atoms"]
        out.update({name + "_x": a[:, 2:5], name + "_v": a[:, 5:8], name + "_times": res["times"],
                    name + "_active": res["active"][:, 1].astype(np.int32), name + "_ledger": res["ledger"]})
    np.savez_compressed(os.path.join(GOLD, "modifies_eam_al_slab.npz"), **out)
    shutil.copy(f, os.path.join(GOLD, "eam_al_slab.dat"))
    print("wrote modifies_eam_al_slab")


def lj4000_case(tdir, work):
    """Lennard-Jones argon as configured for the plain FP64 method: FCC 10^3
    cells = 4000 atoms, a = 5.26 A, Maxwell-Boltzmann 100 K (seed 1, zero net
    momentum), the 2.5 sigma LJ table, skin 0.3 A, 1000 NVE steps of 1 fs on
    the reference's TForcePair; its final atoms and ledger."""
    x, v, (lo, hi) = inputs.lj_argon(ncell=10, a=5.26, temp=100.0, seed_vel=1)
    f = os.path.join(work, "lj_ar_4000.dat")
    inputs.write_import(f, x, v, box=(lo, hi), species=("argon",))
    res = oc.run_reference(f, "pair", "lj.argon", steps=1000, dt=0.001, table_dir=tdir)
    save_case("lj_ar_4000", f, res, box_lo=lo, box_hi=hi, steps=np.array(1000), dt=np.array(0.001))


def impact_slab(site, height, speed, seed):
    """Si diamond slab 6 x 6 x 3 cells (864 atoms, periodic x/y, free z, 300 K)
    and one Ar atom `height` A above surface atom number `site` (of 9 on a
    3 x 3 grid), moving down at `speed` A/ps.  Si is type 0 ("target"), Ar
    type 1 ("projectile"), the convention of the reference's test/si-impact
    (which has one projectile: the reference needs a projectile-projectile
    force as soon as there are two, integrator.cpp:133-143)."""
    a = 5.431
    x, lo, hi = inputs.lattice(inputs.DIAMOND_BASIS, (6, 6, 3), a, 0.125)
    x = inputs.perturb(x, 0.03, seed, lo, hi, (True, True, False))
    v = inputs.maxwell_boltzmann(len(x), 300.0, inputs.md_mass("silicon"), seed + 1)
    top = np.where(x[:, 2] > x[:, 2].max() - 0.5)[0]
    gx, gy = site // 3, site % 3
    want = np.array([(gx + 0.3) * 2 * a, (gy + 0.3) * 2 * a])
    s = top[np.argmin(np.sum((x[top, :2] - want) ** 2, axis=1))]
    ar = x[s] + np.array([0.25, -0.15, height])
    lo = np.array([lo[0], lo[1], lo[2]])
    hi = np.array([hi[0], hi[1], x[:, 2].max() + 12.0])
    types = np.concatenate([np.zeros(len(x), dtype=np.int32), [1]]).astype(np.int32)
    return (np.vstack([x, ar]), np.vstack([v, [0.0, 0.0, -speed]]), types, lo, hi)


def impact_case(tdir, work):
    """Stillinger-Weber Si (every triplet) plus the reference's own Ar-Si table
    (tables/pair.ar-si.zbl: universal ZBL splined to zero over 3.0-3.2 A, knots
    to 5.1 A) through TForcePair between projectile and target, as in
    test/si-impact/main.cpp:70-71.  The table is written to tests/golden/tables
    for the GPU runs.  Static: 9 runs, the Ar atom 0.6-3.1 A above a surface
    atom.  Trajectory: the Ar atom 3.5 A above, moving down at 200 A/ps
    (83 eV), 80 steps of 0.5 fs."""
    shutil.copy(os.path.join(REF, "tables", "pair.ar-si.zbl"), os.path.join(TABLES, "pair.ar-si.zbl"))
    out = {}
    hs = [0.6, 0.9, 1.2, 1.6, 2.0, 2.4, 2.7, 2.9, 3.1]
    xs, fs, ps, vs = [], [], [], []
    for k, h in enumerate(hs):
        x, v, t, lo, hi = impact_slab(k, h, 0.0, 71)
        f = os.path.join(work, "impact_static%d.dat" % k)
        inputs.write_import(f, x, v, types=t, box=(lo, hi), periodic=(True, True, False),
                            species=("silicon", "argon"), names=("target", "projectile"))
        res = oc.run_reference(f, "sw", "silicon", steps=0, table_dir=tdir, swfix=True, pair2="ar-si.zbl")
        a = res["atoms"]
        xs.append(x)
        fs.append(a[:, 8:11])
        ps.append(a[:, 11])
        vs.append(a[:, 12])
    out.update(static_x0=np.array(xs), static_v0=v, types=t, box_lo=lo, box_hi=hi, static_f=np.array(fs),
               static_pot=np.array(ps), static_vir=np.array(vs), heights=np.array(hs))
    x, v, t, lo, hi = impact_slab(4, 3.5, 200.0, 73)
    f = os.path.join(work, "impact_nve.dat")
    inputs.write_import(f, x, v, types=t, box=(lo, hi), periodic=(True, True, False), species=("silicon", "argon"),
                        names=("target", "projectile"))
    res = oc.run_reference(f, "sw", "silicon", steps=80, dt=0.0005, table_dir=tdir, swfix=True, pair2="ar-si.zbl")
    a = res["atoms"]
    out.update(nve_x0=x, nve_v0=v, nve_lo=lo, nve_hi=hi, nve_x=a[:, 2:5], nve_v=a[:, 5:8], nve_f=a[:, 8:11],
               nve_ledger=res["ledger"], steps=np.array(80), dt=np.array(0.0005))
    np.savez_compressed(os.path.join(GOLD, "impact_ar_si_slab.npz"), **out)
    print("wrote impact_ar_si_slab")


def fdtd_map(nx, ny, nz, cell):
    """The map string of an nx x ny x nz grid (index k nx ny + i + j nx), one
    character per cell from cell(i, j, k)."""
    return "".join(cell(i, j, k) for k in range(nz) for j in range(ny) for i in range(nx))


def fdtd_specs():
    """Specs for oracle/_ref/fdtd_driver (oracle/ref/fdtd_driver.cpp)."""
    def slab(i, j, k):  # x, y periodic; z: '.' above, a free top, the bulk, a held bottom, one dead column
        if k == 0:
            return "." if (i, j) == (2, 2) else "v"
        if k == 1:
            return "t"
        if k == 6:
            return "b"
        return "d" if (i, j) == (5, 0) else "a"

    specs = {
        # a TTM-like slab: symbols per layer, block and per-symbol values,
        # ranged and future sources (the future one never applies), an
        # external vector entry, a cell outside the symbol map
        "slab3d": "\n".join([
            "dim 6 5 7",
            "symbol a pppp++ t pppp-+ b pppp+- v ------ d pp--++",
            "map " + fdtd_map(6, 5, 7, slab),
            "spacestep 2.0",
            "timestep 0.05",
            "cell * 300 @ 2,2,1,3,3,1=1000 @ 0,4,5=450.5",
            "conductivity a 2.0 t 1.5 b 3.0 @ 0,0,3,5,4,4=0.5 d 0",
            "capacity * 1.0 a 2.5 @ 1,1,2=4.0",
            "source t 50.0:0:4 @ 0,0,6=20:2:3 a 1.0:7:9",
            "ext 17 5.0",
            "ext 100 -2.5",
            "steps 12",
        ]),
        # one symbol with every face occupied: the first cell at each edge
        # clears that face for the cells after it and for every later step
        "flat2d_cleared": "\n".join([
            "dim 7 5 1",
            "symbol a ++++",
            "map " + fdtd_map(7, 5, 1, lambda i, j, k: "." if (i, j) == (6, 4) else "a"),
            "spacestep 1.0",
            "timestep 0.1",
            "cell @ 3,2,0=100 @ 6,4,0=1",
            "steps 5",
        ]),
        # nz = 2 is 2D; periodic x, free y edges, cells of zero conductivity
        # (K = 0 between two of them, K = 0 * c / c beside one)
        "edges2d": "\n".join([
            "dim 8 6 2",
            "symbol a pp++ u pp-+ w pp+- z pp++",
            "map " + fdtd_map(8, 6, 1, lambda i, j, k: "u" if j == 0 else ("w" if j == 5 else
                                                                              ("z" if (i in (3, 4) and j == 2) else "a"))),
            "spacestep 0.5",
            "timestep 0.01",
            "cell * 10 @ 0,0,0,1,5,0=40 z 80",
            "conductivity * 1 z 0 @ 7,3,0=3.5",
            "capacity w 2 u 0.5",
            "source @ 6,1,0=100:0:7",
            "ext 9 1.25",
            "steps 10",
        ]),
    }
    return specs


def fdtd_case():
    """Cell vectors of the reference's FDTDSolver on each spec."""
    import subprocess

    drv = os.path.join(ROOT, "oracle", "_ref", "fdtd_driver")
    out = {}
    for name, spec in fdtd_specs().items():
        txt = subprocess.run([drv], input=spec, capture_output=True, text=True, check=True).stdout
        rows = [[float(v) for v in ln.split()[2:]] for ln in txt.splitlines() if ln.startswith("step ")]
        out[name + "_spec"] = np.array(spec)
        out[name + "_rows"] = np.array(rows)
    np.savez_compressed(os.path.join(GOLD, "fdtd_cases.npz"), **out)
    print("wrote fdtd_cases")


def example_case():
    """The reference's example system (test/example/example.cpp) run by the
    reference (oracle/ref/example_fixture.cpp): the state after FirstRun,
    atoms 0 and 10 and the energies after every step, the final state."""
    import subprocess

    for name in ("eam.platinum", "def.platinum"):
        dst = os.path.join(TABLES, name)
        shutil.copyfile(os.path.join(REF, "tables", name), dst)
        os.chmod(dst, 0o644)
    work = tempfile.mkdtemp(prefix="omdex_")
    env = dict(os.environ, OMD_TABLE=TABLES)
    subprocess.run([os.path.join(ROOT, "oracle", "_ref", "example_fixture")], cwd=work, env=env, check=True,
                   capture_output=True)
    start = np.loadtxt(os.path.join(work, "start.txt"))
    end = np.loadtxt(os.path.join(work, "end.txt"))
    box = np.loadtxt(os.path.join(work, "box.txt"))
    steps = np.loadtxt(os.path.join(work, "steps.txt"))
    np.savez_compressed(os.path.join(GOLD, "example_pt_fcc111.npz"), x0=start[:, :3], v0=start[:, 3:],
                        box_lo=box[:3], box_hi=box[3:6], dt=box[6], base_potential=box[7],
                        traj0=steps[:, 0:3], traj10=steps[:, 3:6], kinetic=steps[:, 6], potential=steps[:, 7],
                        x_end=end[:, :3], v_end=end[:, 3:])
    print("wrote example_pt_fcc111", len(start), "atoms", len(steps), "steps")


def read_cluster(path):
    """Positions (first three columns) of one of the reference's own silicon
    test clusters (test/check-verlet-list: dimer, trimer, tetra, 1x1x1)."""
    rows = []
    with open(path) as fh:
        for line in fh:
            t = line.split()
            if t and not line.startswith("#"):
                rows.append([float(v) for v in t[:3]])
    return np.array(rows)


def clusters_case(tdir, work):
    """SW Si on the reference's own test clusters, free boundaries: the
    reference built without the sw.cpp:261 guard (every triplet) and as
    shipped, with its full neighbour tuples."""
    for name in ("dimer", "trimer", "tetra", "1x1x1"):
        x = read_cluster(os.path.join(REF, "test", "check-verlet-list", name))
        lo, hi = x.min(0) - 5.0, x.max(0) + 5.0
        f = os.path.join(work, "sw_si_%s.dat" % name)
        inputs.write_import(f, x, None, box=(lo, hi), periodic=(False, False, False), species=("silicon",))
        res = oc.run_reference(f, "sw", "silicon", steps=0, dump_nbr=True, table_dir=tdir, swfix=True)
        asis = oc.run_reference(f, "sw", "silicon", steps=0, table_dir=tdir, swfix=False)
        save_case("sw_si_%s" % name, f, res, box_lo=lo, box_hi=hi, f_asis=asis["atoms"][:, 8:11],
                  pot_asis=asis["atoms"][:, 11])


def impact_replica_case(tdir, work):
    """The reference's own impact replica (test/si-impact/atom.dat: a Si slab
    of 10,648 atoms, periodic x/y, free z, and one Ar atom) with its
    potentials (test/si-impact/main.cpp:70-71: SW between target atoms, the
    Ar-Si table between projectile and target).  Static forces and energies
    with the Ar atom over the aim point of test/si-impact/omd-parameter
    (28.52, 31.27) at 0.5-2.0 A above the top layer."""
    x, v, t, (lo, hi), per = inputs.read_import(os.path.join(REF, "test", "si-impact", "atom.dat"))
    order = np.argsort(t, kind="stable")  # targets first: nid follows the containers' order
    x, v, t = x[order], v[order], t[order]
    top = x[t == 0, 2].max()
    hs = [0.5, 1.4, 2.0]
    fs, ps, xs = [], [], []
    for k, h in enumerate(hs):
        xk = x.copy()
        xk[t == 1] = [28.52, 31.27, top + h]
        f = os.path.join(work, "impact_replica%d.dat" % k)
        inputs.write_import(f, xk, v, types=t, box=(lo, hi), periodic=per, species=("silicon", "argon"),
                            names=("target", "projectile"))
        res = oc.run_reference(f, "sw", "silicon", steps=0, table_dir=tdir, swfix=True, pair2="ar-si.zbl")
        a = res["atoms"]
        fs.append(a[:, 8:11])
        ps.append(a[:, 11])
        xs.append(xk[t == 1][0])
    np.savez_compressed(os.path.join(GOLD, "impact_replica.npz"), x0=x, types=t, box_lo=lo, box_hi=hi,
                        periodic=np.array(per), ar=np.array(xs), heights=np.array(hs), f=np.array(fs),
                        pot=np.array(ps))
    print("wrote impact_replica", len(x), "atoms")


def ar_pt_case(tdir, work):
    """Two atom types with EAM on one of them, as test/two_elements/two.cpp
    combines them: EAM platinum between Pt atoms (type 0, "target") and the
    reference's Ar-Pt table (tables/pair.ar-pt.zbl) between the Ar atom
    (type 1, "projectile") and Pt.  An FCC Pt slab of 6 x 6 x 3 cells
    (a = 3.924, periodic x/y, free z, Gaussian displacements 0.05 A) with the
    Ar atom 1.2-2.8 A above a surface atom.  Static forces and energies."""
    shutil.copy(os.path.join(REF, "tables", "pair.ar-pt.zbl"), os.path.join(TABLES, "pair.ar-pt.zbl"))
    tdir = table_dir()  # with the table just written
    a = 3.924
    x, lo, hi = inputs.lattice(inputs.FCC_BASIS, (6, 6, 3), a, 0.25)
    x = inputs.perturb(x, 0.05, 81, lo, hi, (True, True, False))
    top = np.where(x[:, 2] > x[:, 2].max() - 0.5)[0]
    s = top[np.argmin(np.sum((x[top, :2] - np.array([2.6 * a, 3.1 * a])) ** 2, axis=1))]
    hi = np.array([hi[0], hi[1], x[:, 2].max() + 12.0])
    types = np.concatenate([np.zeros(len(x), dtype=np.int32), [1]]).astype(np.int32)
    hs = [1.2, 2.0, 2.8]
    xs, fs, ps = [], [], []
    for k, h in enumerate(hs):
        xk = np.vstack([x, x[s] + np.array([0.3, -0.2, h])])
        f = os.path.join(work, "ar_pt%d.dat" % k)
        inputs.write_import(f, xk, None, types=types, box=(lo, hi), periodic=(True, True, False),
                            species=("platinum", "argon"), names=("target", "projectile"))
        res = oc.run_reference(f, "eam", "platinum", steps=0, table_dir=tdir, pair2="ar-pt.zbl")
        at = res["atoms"]
        xs.append(xk)
        fs.append(at[:, 8:11])
        ps.append(at[:, 11])
    np.savez_compressed(os.path.join(GOLD, "ar_pt_slab.npz"), x0=np.array(xs), types=types, box_lo=lo, box_hi=hi,
                        heights=np.array(hs), f=np.array(fs), pot=np.array(ps))
    print("wrote ar_pt_slab", len(types), "atoms")


def main(only=None):
    os.makedirs(TABLES, exist_ok=True)
    if not REF:
        raise SystemExit("make_golden.py: set OMD_REFERENCE to the Object-MD source tree")
    if not oc.build_reference(REF):
        raise SystemExit("reference sources not found at %s" % REF)
    if only == "ttm":
        ttm_case(table_dir(), tempfile.mkdtemp(prefix="omdgold_"))
        return
    if only == "checkpoint":
        checkpoint_case(table_dir())
        return
    if only == "output":
        output_case(table_dir())
        return
    if only == "thermo":
        thermo_case(table_dir())
        return
    if only == "modifies":
        modifies_case(table_dir(), tempfile.mkdtemp(prefix="omdgold_"))
        return
    if only == "impact":
        impact_case(table_dir(), tempfile.mkdtemp(prefix="omdgold_"))
        return
    if only == "fdtd":
        fdtd_case()
        return
    if only == "example":
        example_case()
        return
    if only == "ar_pt":
        ar_pt_case(table_dir(), tempfile.mkdtemp(prefix="omdgold_"))
        return
    if only == "impact_replica":
        impact_replica_case(table_dir(), tempfile.mkdtemp(prefix="omdgold_"))
        return
    if only == "clusters":
        clusters_case(table_dir(), tempfile.mkdtemp(prefix="omdgold_"))
        return
    if only == "lj4000":
        lj4000_case(table_dir(), tempfile.mkdtemp(prefix="omdgold_"))
        return
    write_eam5000(os.path.join(TABLES, "eam.aluminum5000"))
    with open(os.path.join(TABLES, "pair.lj.argon"), "w") as fh:
        fh.write(inputs.lj_table_text())
    with open(os.path.join(TABLES, "sw.silicon"), "w") as fh:
        fh.write(inputs.sw_param_text())
    with open(os.path.join(TABLES, "tersoff.silicon27"), "w") as fh:
        fh.write(inputs.tersoff_param_text(2.7, 0.15))
    tdir = table_dir()
    work = tempfile.mkdtemp(prefix="omdgold_")

    # EAM Al, static, two sizes
    for name, ncell in (("eam_al_500", 5), ("eam_al_4000", 10)):
        x, v, (lo, hi) = inputs.eam_aluminium(ncell=ncell, a=4.05, sigma=0.05, temp=300.0, seed_pos=2, seed_vel=3)
        f = os.path.join(work, name + ".dat")
        inputs.write_import(f, x, v, box=(lo, hi), species=("aluminum",))
        res = oc.run_reference(f, "eam", "aluminum5000", steps=0, dump_nbr=True, table_dir=tdir)
        save_case(name, f, res, box_lo=lo, box_hi=hi)

    # EAM Al, NVE trajectory, list rebuilt every step (comm.refresh unset)
    x, v, (lo, hi) = inputs.eam_aluminium(ncell=5, a=4.05, sigma=0.05, temp=300.0, seed_pos=12, seed_vel=13)
    f = os.path.join(work, "eam_al_nve.dat")
    inputs.write_import(f, x, v, box=(lo, hi), species=("aluminum",))
    res = oc.run_reference(f, "eam", "aluminum5000", steps=20, dt=0.002, table_dir=tdir)
    save_case("eam_al_nve", f, res, box_lo=lo, box_hi=hi, steps=np.array(20), dt=np.array(0.002))

    # table LJ Ar (analytic LJ table), static and NVE
    x, v, (lo, hi) = inputs.lj_argon(ncell=5, a=5.26, temp=100.0, seed_vel=1)
    x = inputs.perturb(x, 0.05, 9, lo, hi)
    f = os.path.join(work, "lj_ar_500.dat")
    inputs.write_import(f, x, v, box=(lo, hi), species=("argon",))
    res = oc.run_reference(f, "pair", "lj.argon", steps=0, dump_nbr=True, table_dir=tdir)
    save_case("lj_ar_500", f, res, box_lo=lo, box_hi=hi)
    res = oc.run_reference(f, "pair", "lj.argon", steps=50, dt=0.001, table_dir=tdir)
    save_case("lj_ar_nve", f, res, box_lo=lo, box_hi=hi, steps=np.array(50), dt=np.array(0.001))

    # SW Si, static: fixed reference build (every triplet) and as-is build
    x, v, (lo, hi) = inputs.diamond_silicon(ncell=3, a=5.431, sigma=0.08, temp=1000.0, seed_pos=4, seed_vel=5)
    f = os.path.join(work, "sw_si_216.dat")
    inputs.write_import(f, x, v, box=(lo, hi), species=("silicon",))
    res = oc.run_reference(f, "sw", "silicon", steps=0, dump_nbr=True, table_dir=tdir, swfix=True)
    asis = oc.run_reference(f, "sw", "silicon", steps=0, table_dir=tdir, swfix=False)
    save_case("sw_si_216", f, res, box_lo=lo, box_hi=hi, f_asis=asis["atoms"][:, 8:11],
              pot_asis=asis["atoms"][:, 11])
    x, v, (lo, hi) = inputs.diamond_silicon(ncell=5, a=5.431, sigma=0.03, temp=1000.0, seed_pos=4, seed_vel=5)
    f = os.path.join(work, "sw_si_1000.dat")
    inputs.write_import(f, x, v, box=(lo, hi), species=("silicon",))
    res = oc.run_reference(f, "sw", "silicon", steps=0, dump_nbr=True, table_dir=tdir, swfix=True)
    save_case("sw_si_1000", f, res, box_lo=lo, box_hi=hi)

    # Berendsen thermostat on EAM Al
    x, v, (lo, hi) = inputs.eam_aluminium(ncell=5, a=4.05, sigma=0.05, temp=600.0, seed_pos=22, seed_vel=23)
    f = os.path.join(work, "eam_al_tc.dat")
    inputs.write_import(f, x, v, box=(lo, hi), species=("aluminum",))
    res = oc.run_reference(f, "eam", "aluminum5000", steps=20, dt=0.002, tcontrol=(300.0, 0.05), table_dir=tdir)
    save_case("eam_al_tc", f, res, box_lo=lo, box_hi=hi, steps=np.array(20), dt=np.array(0.002),
              tcontrol=np.array([300.0, 0.05]))

    # TableReader known answers from the reference's own TableReader: the
    # 5000-knot PAIR section (RMULT) and EMBED section (PLAIN), including the
    # edge rules just below the first knot and past the last one.
    for sec in ("PAIR", "EMBED"):
        spec = oc.parse_table(os.path.join(TABLES, "eam.aluminum5000"), sec)
        top = spec["off"] + (spec["n"] - 1) * spec["dr"]
        r = np.concatenate([np.linspace(max(spec["off"] - 0.9 * spec["dr"], 1e-3), top + 0.9 * spec["dr"], 509),
                            spec["off"] + spec["dr"] * np.array([0.0, 1.0, 2.5, spec["n"] - 2, spec["n"] - 1.0])])
        rfile = os.path.join(work, "r_%s.txt" % sec)
        np.savetxt(rfile, r, fmt="%.17g")
        out = tempfile.mkdtemp(prefix="omdtabref_")
        import subprocess
        subprocess.check_call([oc.REF_DRIVER, out, "tabfile", os.path.join(TABLES, "eam.aluminum5000"), "tabname",
                               sec, "rfile", rfile], cwd=out)
        tab = np.loadtxt(os.path.join(out, "table.txt"))
        np.savez_compressed(os.path.join(GOLD, "table_%s.npz" % sec.lower()), r=tab[:, 0], val=tab[:, 1],
                            dval=tab[:, 2])
        print("wrote table_%s" % sec.lower(), len(tab))
    ttm_case(tdir, work)
    checkpoint_case(tdir)
    modifies_case(tdir, work)
    lj4000_case(tdir, work)
    impact_case(tdir, work)
    output_case(tdir)
    thermo_case(tdir)
    fdtd_case()
    example_case()
    print("done")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
