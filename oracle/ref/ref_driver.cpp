/*
 * ref_driver -- runs the UNMODIFIED Object-MD reference force path on one
 * rank and writes what the parity tests compare against.  Test
 * infrastructure only: it is built (by oracle/ref/Makefile) from the
 * reference's own sources and links nothing of this project's product.
 *
 * The program is an ordinary Object-MD application, written the way the
 * reference's own test programs are (test/example/example.cpp:5-34): an
 * MDSystemGrid subclass whose CreateSystem/CreateGadget/SystemSetting pick a
 * potential, an iterator and the periodic box.  Everything else - the
 * linked-cell Verlet list, the periodic ghost images, the force loop, the
 * velocity-Verlet integrator - is the reference's code.
 *
 * usage: ref_driver <outdir> key value ...     (keys below; all values text)
 *   import      <file>   atoms in the reference Import format (container.cpp:290)
 *   kind        eam|pair|sw        force kernel family
 *   table       <name>   table / parameter name searched in $OMD_TABLE
 *   pair2       <name>   optional projectile-target pair table (two-species inputs)
 *   steps       <n>      0 = one static force evaluation (system.cpp:1034 RunStatic)
 *   dt          <ps>     time step
 *   skin        <A>      comm.tolerance (absolute)
 *   refresh     <n>      comm.refresh (0 = every step)
 *   tcontrol    <T> <tau>  Berendsen TempController (TempController.h:78-91)
 *   ttm         <file> <atom_volume> <Te0>  TTM_Homogen (TTM_Homogen_SCNA.h) with an
 *                        intensive ThermoDetector (ThermoDetector.h); writes ttm.txt
 *                        (step Te int_Een int_Aen avg_temp) and thermo.txt (nid T_i n_i)
 *   dump_nbr    0|1      write the neighbour tuples of the final list
 *   time_only   0|1      only print the RunKernel wall time
 *   damp        <factor> ForceDamper on every atom (damp.factor, damp.target -)
 *   clamp       <axes>   CoordClamp("-", axes)
 *   dyndt       <maxpath> <max> <update>  DynamicTimeStep(maxpath, max, update)
 *   range       <border> RangeLimiter("-", border)
 *                        (with any of these: times.txt = Step TimeStep ElapsedTime
 *                        per step, active.txt = nid flag&FLAG_ACTIVE at the end)
 *   source      <energy> <start> <width>  EnergySource, pulse mode (source.* parameters)
 *   dump        <file> <mode>  after the run, DumpAtoms(file, mode) (container.cpp:417-519)
 *   monitor     <file> <every> SysMonitor(file) with monitor.every (SysMonitor.h)
 *   thermodump  <name>   an intensive ThermoDetector (ThermoDetector.h) whose data
 *                        file (DataDumper::Measure) is written once after the run:
 *                        <outdir>/<name>.001
 *   save        <file>   after the run, the reference's binary checkpoint
 *                        (MDSystemGrid::SaveSimulation, systemgrid.cpp:848-852)
 *   continue    <file>   resume from a binary checkpoint (CONTINUE_MODE,
 *                        system.cpp:218-222, 1004-1019); `steps` is then the
 *                        Step to stop at, not a count
 *
 * Outputs in <outdir>: atoms.txt (nid x y z vx vy vz fx fy fz potential virial
 * for local atoms sorted by nid), nbr.txt (nid_i nid_j sx sy sz), ledger.txt
 * (step kinetic potential energy), summary.txt.
 */
#include <omd/systemgrid.h>
#include <omd/integrator.h>
#include <potential/team.h>
/* tpair.h names omd types unqualified, as it does inside the reference's omd.h */
using namespace omd;
#include <potential/tpair.h>
#include <potential/sw.h>
#include <modify/VerletList.h>
#include <modify/VerletListFull.h>
#include <modify/TempController.h>
#include <modify/ForceDamper.h>
#include <modify/CoordClamp.h>
#include <modify/DynamicTimeStep.h>
#include <modify/RangeLimiter.h>
#include <modify/EnergySource.h>
#include <detect/ThermoDetector.h>
#include <detect/SysMonitor.h>
#include <misc/TTM_Homogen_SCNA.h>

#include <sys/time.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

using namespace omd;

static double wall_now() {
    struct timeval tv;
    gettimeofday(&tv, 0);
    return tv.tv_sec + 1e-6 * tv.tv_usec;
}

struct NbrTuple {
    int i, j, sx, sy, sz;
    bool operator<(const NbrTuple& o) const {
        if (i != o.i) return i < o.i;
        if (j != o.j) return j < o.j;
        if (sx != o.sx) return sx < o.sx;
        if (sy != o.sy) return sy < o.sy;
        return sz < o.sz;
    }
};

class OracleSim;

/* Records every (at,to) pair the iterator visits in its half loop. */
class PairRecorder : public MDGadget {
public:
    std::vector<std::pair<int, int> > pairs;
    bool PreIterationNode(int) { return true; }
    void IterationNode(int at, int to) { pairs.push_back(std::make_pair(at, to)); }
};

class OracleSim : public MDSystemGrid {
public:
    std::map<std::string, std::vector<std::string> > opt;
    std::string outdir;
    int nsteps;
    double t_begin, t_end;
    FILE* ledger;
    FILE* ttmlog;
    FILE* timelog;
    ThermoDetector* thermo;

    OracleSim(int& argc, char**& argv, const std::string& od,
              const std::map<std::string, std::vector<std::string> >& o)
        : MDSystemGrid(argc, argv), opt(o), outdir(od), nsteps(0), t_begin(0), t_end(0), ledger(0), ttmlog(0),
          timelog(0),
          thermo(0) {
        nsteps = atoi(get("steps", "0").c_str());
    }

    std::string get(const std::string& k, const std::string& def, int idx = 0) {
        std::map<std::string, std::vector<std::string> >::iterator it = opt.find(k);
        if (it == opt.end() || (int)it->second.size() <= idx) return def;
        return it->second[idx];
    }

    void CreateSystem() { Import(get("import", "")); }

    void CreateGadget() {
        SetIntegrator(new MDIntegrator(atof(get("dt", "0.001").c_str())));
        std::string kind = get("kind", "eam");
        std::string table = get("table", "aluminum");
        std::string pair2 = get("pair2", "");
        ForceKernel* k = 0;
        if (kind == "eam") {
            k = new TForceEAM(table);
            AddModify(new VerletList);
        } else if (kind == "pair") {
            k = new TForcePair(table);
            AddModify(new VerletList);
        } else if (kind == "sw") {
            k = new StillingerWeber(table);
            AddModify(new VerletListFull);
        } else {
            die("unknown kind " + kind);
        }
        /* Two-species inputs name their containers "target" and "projectile"
           (the convention of test/si-impact/atom.dat). */
        if (pair2.empty()) {
            AddForce(k);
        } else {
            AddForce(k, "target", "target");
            AddForce(new TForcePair(pair2), "projectile", "target");
        }
        if (opt.count("ttm") || opt.count("thermodump")) {
            // sample time beyond the run: no dump files during it
            thermo = new ThermoDetector(1e30, -1.0, outdir + "/" + get("thermodump", "thermo"));
            thermo->SetIntensive(true);
            AddDetector(thermo);
        }
        if (opt.count("ttm")) AddModify(new TTM_Homogen());
        if (opt.count("tcontrol"))
            AddModify(new TempController(atof(get("tcontrol", "300", 0).c_str()),
                                         atof(get("tcontrol", "0.1", 1).c_str())));
        /* the impact-run modifies, in test/si-impact/main.cpp's order */
        if (opt.count("damp")) AddModify(new ForceDamper);
        if (opt.count("clamp")) AddModify(new CoordClamp("-", get("clamp", "xyz")));
        if (opt.count("dyndt"))
            AddModify(new DynamicTimeStep(atof(get("dyndt", "0.1", 0).c_str()), atof(get("dyndt", "0.001", 1).c_str()),
                                          atoi(get("dyndt", "5", 2).c_str())));
        if (opt.count("range")) AddModify(new RangeLimiter("-", atof(get("range", "1000", 0).c_str())));
        if (opt.count("monitor")) AddDetector(new SysMonitor(get("monitor", "md.out", 0)));
        if (opt.count("source")) AddModify(new EnergySource);
    }

    void SystemSetting() {}

    bool CheckRun() {
        bool base = MDSystemGrid::CheckRun();
        if (ledger && Step > 0)
            fprintf(ledger, "%d %.17g %.17g %.17g\n", Step, Kinetic, Potential, Energy);
        if (timelog) fprintf(timelog, "%d %.17g %.17g\n", Step, Integrator->TimeStep, ElapsedTime);
        if (ttmlog && Step > 0)
            fprintf(ttmlog, "%d %.17g %.17g %.17g %.17g\n", Step, GetMessageSlot("e_temp:")->AsDouble(),
                    GetMessageSlot("int_Een:")->AsDouble(), GetMessageSlot("int_Aen:")->AsDouble(),
                    thermo->GetTemperatureAvg());
        return base && Step < nsteps;
    }

    void BeforeRun() {
        if (get("time_only", "0") == "0") {
            ledger = fopen((outdir + "/ledger.txt").c_str(), "w");
            if (ledger)
                fprintf(ledger, "%d %.17g %.17g %.17g\n", 0, Kinetic, BasePotential, 0.0);
            if (opt.count("ttm")) ttmlog = fopen((outdir + "/ttm.txt").c_str(), "w");
            if (opt.count("damp") || opt.count("clamp") || opt.count("dyndt") || opt.count("range") ||
                opt.count("source"))
                timelog = fopen((outdir + "/times.txt").c_str(), "w");
        }
        t_begin = wall_now();
    }

    void AfterRun() {
        t_end = wall_now();
        int nloc = GetLocalAtomNumber();
        FILE* s = fopen((outdir + "/summary.txt").c_str(), "w");
        if (s) {
            fprintf(s, "local_atoms %d\nall_atoms %d\nsteps %d\nseconds %.9g\n", nloc, GetNAtom(), Step,
                    t_end - t_begin);
            fprintf(s, "potential %.17g\nkinetic %.17g\nbase_potential %.17g\nvirial %.17g\n", Potential,
                    Kinetic, BasePotential, Virial);
            fprintf(s, "box %.17g %.17g %.17g %.17g %.17g %.17g\n", Box.x0, Box.y0, Box.z0, Box.x1, Box.y1,
                    Box.z1);
            fprintf(s, "max_cut_radius %.17g\n", GetMaxCutRadius());
            fclose(s);
        }
        if (ledger) {
            fprintf(ledger, "%d %.17g %.17g %.17g\n", Step, Kinetic, Potential, Energy);
            fclose(ledger);
            ledger = 0;
        }
        if (get("time_only", "0") != "0") {
            printf("atom_steps_per_s %.6g local_atoms %d steps %d seconds %.6f\n",
                   (double)nloc * Step / (t_end - t_begin), nloc, Step, t_end - t_begin);
            return;
        }
        std::vector<int> order(nloc);
        for (int i = 0; i < nloc; i++) order[i] = i;
        std::sort(order.begin(), order.end(), CompareNid(this));
        FILE* f = fopen((outdir + "/atoms.txt").c_str(), "w");
        for (int k = 0; k < nloc; k++) {
            Atom& a = Atoms(order[k]);
            fprintf(f, "%d %d %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", a.nid, a.tid,
                    a.x, a.y, a.z, a.vx, a.vy, a.vz, a.fx, a.fy, a.fz, a.potential, a.virial);
        }
        fclose(f);
        if (get("dump_nbr", "0") != "0") DumpNeighbours();
        if (opt.count("dump")) DumpAtoms(get("dump", "dump.dat", 0), atoi(get("dump", "0", 1).c_str()));
        if (opt.count("save")) SaveSimulation(get("save", ""));
        if (opt.count("thermodump")) thermo->Measure();  // the detector's data file of the final state
        if (timelog) {
            fclose(timelog);
            timelog = 0;
            FILE* t = fopen((outdir + "/active.txt").c_str(), "w");
            for (int k = 0; k < nloc; k++) fprintf(t, "%d %d\n", Atoms(order[k]).nid, Atoms(order[k]).flag & FLAG_ACTIVE);
            fclose(t);
        }
        if (ttmlog) {
            fclose(ttmlog);
            ttmlog = 0;
        }
        if (thermo) {
            FILE* t = fopen((outdir + "/thermo.txt").c_str(), "w");
            for (int k = 0; k < nloc; k++) {
                Atom& a = Atoms(order[k]);
                fprintf(t, "%d %.17g %.17g\n", a.nid, a.aux[thermo->GetAuxTempIndex()],
                        a.aux[thermo->GetAuxDensIndex()]);
            }
            fclose(t);
        }
    }

    struct CompareNid {
        OracleSim* s;
        CompareNid(OracleSim* ss) : s(ss) {}
        bool operator()(int a, int b) const { return s->Atoms(a).nid < s->Atoms(b).nid; }
    };

    /* Image vector of atom idx relative to its owner, in box lengths. */
    void ImageOf(int idx, const std::map<int, int>& owner, int& sx, int& sy, int& sz) {
        Atom& g = Atoms(idx);
        Atom& o = Atoms(owner.find(g.nid)->second);
        sx = (int)lround((g.x - o.x) / Box.lx);
        sy = (int)lround((g.y - o.y) / Box.ly);
        sz = (int)lround((g.z - o.z) / Box.lz);
    }

    void DumpNeighbours() {
        int nloc = GetLocalAtomNumber();
        std::map<int, int> owner;
        for (int i = 0; i < nloc; i++) owner[Atoms(i).nid] = i;
        PairRecorder rec;
        GetIterator()->IterateHalf(&rec);
        std::vector<NbrTuple> t;
        for (size_t k = 0; k < rec.pairs.size(); k++) {
            int at = rec.pairs[k].first, to = rec.pairs[k].second;
            bool gat = at >= nloc, gto = to >= nloc;
            int sx, sy, sz;
            if (!gat && !gto) {
                NbrTuple a = {Atoms(at).nid, Atoms(to).nid, 0, 0, 0};
                NbrTuple b = {Atoms(to).nid, Atoms(at).nid, 0, 0, 0};
                t.push_back(a);
                t.push_back(b);
            } else if (!gat && gto) {
                ImageOf(to, owner, sx, sy, sz);
                NbrTuple a = {Atoms(at).nid, Atoms(to).nid, sx, sy, sz};
                t.push_back(a);
            } else if (gat && !gto) {
                ImageOf(at, owner, sx, sy, sz);
                NbrTuple a = {Atoms(to).nid, Atoms(at).nid, sx, sy, sz};
                t.push_back(a);
            }
        }
        std::sort(t.begin(), t.end());
        FILE* f = fopen((outdir + "/nbr.txt").c_str(), "w");
        for (size_t k = 0; k < t.size(); k++)
            fprintf(f, "%d %d %d %d %d\n", t[k].i, t[k].j, t[k].sx, t[k].sy, t[k].sz);
        fclose(f);
    }
};

int main(int argc, char** argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: ref_driver <outdir> key value ...\n");
        return 2;
    }
    std::string outdir = argv[1];
    std::map<std::string, std::vector<std::string> > opt;
    for (int i = 2; i < argc;) {
        std::string key = argv[i++];
        int nval = (key == "tcontrol" || key == "dump" || key == "monitor") ? 2
                   : ((key == "ttm" || key == "dyndt" || key == "source") ? 3 : 1);
        for (int k = 0; k < nval && i < argc; k++) opt[key].push_back(argv[i++]);
    }
    /* Table mode: the reference TableReader itself (treader.cpp) evaluated at
       the r values listed one per line in file `rfile`; prints r val dval. */
    if (opt.count("tabfile")) {
        /* default-construct, then open(): the path TForceEAM::Init takes (team.cpp:211);
           the two-argument constructor resets the format to PLAIN after opening */
        TableReader t;
        t.open(opt["tabfile"][0], opt.count("tabname") ? opt["tabname"][0] : std::string(""));
        FILE* rf = fopen(opt["rfile"][0].c_str(), "r");
        FILE* of = fopen((outdir + "/table.txt").c_str(), "w");
        double r;
        while (rf && fscanf(rf, "%lf", &r) == 1) {
            double v, dv;
            t.read(r, v, dv);
            fprintf(of, "%.17g %.17g %.17g\n", r, v, dv);
        }
        if (rf) fclose(rf);
        fclose(of);
        return 0;
    }
    /* Reference parameters go through the reference's own ParamHandler argv path. */
    std::vector<std::string> args;
    args.push_back(argv[0]);
    args.push_back("comm.tolerance");
    args.push_back(opt.count("skin") ? opt["skin"][0] : std::string("0.3"));
    if (opt.count("refresh") && atoi(opt["refresh"][0].c_str()) > 0) {
        args.push_back("comm.refresh");
        args.push_back(opt["refresh"][0]);
    }
    args.push_back("time.step");
    args.push_back(opt.count("dt") ? opt["dt"][0] : std::string("0.001"));
    args.push_back("time.max");
    args.push_back("1e30");
    args.push_back("--silent");
    if (opt.count("source")) {  // EnergySource::ReadParameter (EnergySource.h:78-83)
        args.push_back("source.energy");
        args.push_back(opt["source"][0]);
        args.push_back("source.start");
        args.push_back(opt["source"][1]);
        args.push_back("source.width");
        args.push_back(opt["source"][2]);
        args.push_back("source.mode");
        args.push_back("pulse");
    }
    if (opt.count("monitor")) {  // SysMonitor::ReadParameter (SysMonitor.h)
        args.push_back("monitor.every");
        args.push_back(opt["monitor"][1]);
    }
    if (opt.count("damp")) {  // ForceDamper::ReadParameter (ForceDamper.h:24-27)
        args.push_back("damp.factor");
        args.push_back(opt["damp"][0]);
        args.push_back("damp.target");
        args.push_back("-");
    }
    if (opt.count("continue")) {
        args.push_back("continue");
        args.push_back(opt["continue"][0]);
    }
    if (!opt.count("steps") || atoi(opt["steps"][0].c_str()) == 0) args.push_back("mode.static");
    if (opt.count("ttm")) {
        args.push_back("ttmsc.electron-phonon_file");
        args.push_back(opt["ttm"][0]);
        args.push_back("ttmsc.atom_volume");
        args.push_back(opt["ttm"][1]);
        args.push_back("ttmsc.electron_init_temperature");
        args.push_back(opt["ttm"][2]);
    }
    std::vector<char*> cargs;
    for (size_t i = 0; i < args.size(); i++) cargs.push_back(const_cast<char*>(args[i].c_str()));
    cargs.push_back(0);
    int cargc = (int)args.size();
    char** cargv = &cargs[0];
    OracleSim sim(cargc, cargv, outdir, opt);
    return sim.Run();
}
