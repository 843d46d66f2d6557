/*
 * GPUIntegrator: the reference's velocity-Verlet integrator (MDIntegrator,
 * include/omd/integrator.h:41-69, src/omd/integrator.cpp) with the step
 * evaluated on one GB300 through libomdg's C ABI (include/omdg.h).
 *
 * An Object-MD application swaps one line,
 *     SetIntegrator(new MDIntegrator(dt));   ->   SetIntegrator(new GPUIntegrator(dt));
 * and keeps its AddForce / AddModify / AddDetector calls.  The header is
 * C++98 and compiles against the reference's own headers; link the
 * application with libomdg.so.
 *
 *   Init       MDIntegrator::Init (the kernel matrix, each kernel's Init, which
 *              resolves its table under $OMD_TABLE, MaxCutRadius, time.step),
 *              then one context: the box and PBoundary, the atoms in Atoms
 *              order (type = tid, mass and Z per container), one omdg_add_* per
 *              registered kernel with the file it read, the time step, the
 *              Verlet skin (verlet.radtole, 0.3 A when unset; rebuilds on
 *              displacement) and the reference's first step (FirstRun's forces
 *              are zeroed, system.cpp:860-873).  The host embedding handler
 *              that TForceEAM::Init adds (team.cpp:215-221) is deactivated: the
 *              device evaluates the whole EAM.
 *   Iterate    (FirstRun, static runs) as MDIntegrator::Iterate
 *              (integrator.cpp:202-216): PRE_CALCULATION modifies, the forces
 *              on the device for the current Atoms, POST_FORCE modifies.
 *   Integrate  one RunKernel step (integrator.cpp:225-259) on the device from
 *              the current Atoms (positions, velocities, FLAG_ACTIVE): kick,
 *              drift, list refresh, forces, kick; then positions, velocities,
 *              forces, potentials and virials back into Atoms, so that
 *              MeasurePotential / MeasureKinetic, the POST_INTEGRATION
 *              modifies, the detectors and InlineFunction see the step as
 *              they do with MDIntegrator, and the PRE_CALCULATION modifies
 *              (the host Verlet list the detectors iterate) run once per step.
 *
 * Force kernels: TForceEAM, TForcePair (FP32 with compensated sums) and
 * Tersoff are found by their PrintInfo line, which names the file they read;
 * a StillingerWeber kernel needs its parameter file through SetForceFile.
 * Host force modifies (POST_FORCE) do not act inside the device step: use
 * the library's device modifies (omdg_add_force_damper, ...).
 */
#ifndef OMDG_GPU_INTEGRATOR_H
#define OMDG_GPU_INTEGRATOR_H

#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include <omd/integrator.h>
#include <omd/system.h>

#include "omdg.h"

namespace omd {

class GPUIntegrator : public MDIntegrator {
    omdg_ctx* ctx;
    int device;
    std::vector<double> xs, vs, fs, pots, virs;
    std::vector<int> active;
    std::vector<std::pair<ForceKernel*, std::string> > files;

    void check(int rc, const std::string& what) {
        if (rc == OMDG_OK) return;
        std::ostringstream os;
        os << "GPUIntegrator: " << what << " returned " << rc;
        if (ctx) os << ": " << omdg_last_error(ctx);
        else os << " (OMDG_ECUDA = " << OMDG_ECUDA << ": no usable GB300)";
        die(os.str());
    }

    // The file a kernel read, from its PrintInfo line ("table=<path>" in
    // team.cpp:239-244, "Table=<path>" in tpair.h:53 and tersoff.h:411).
    static std::string printed_file(ForceKernel* fk) {
        std::ostringstream os;
        fk->PrintInfo(os);
        const std::string s = os.str();
        const char* keys[2] = {"table=", "Table="};
        for (int k = 0; k < 2; k++) {
            std::string::size_type p = s.find(keys[k]);
            if (p == std::string::npos) continue;
            p += 6;
            std::string::size_type e = s.find_first_of(" )\n", p);
            return s.substr(p, e == std::string::npos ? std::string::npos : e - p);
        }
        return "";
    }

    std::string file_of(ForceKernel* fk) {
        for (size_t k = 0; k < files.size(); k++)
            if (files[k].first == fk) return files[k].second;
        return printed_file(fk);
    }

    void gather() {
        const int n = System->GetNAtom();
        for (int i = 0; i < n; i++) {
            const Atom& a = System->Atoms(i);
            xs[3 * i] = a.x;
            xs[3 * i + 1] = a.y;
            xs[3 * i + 2] = a.z;
            vs[3 * i] = a.vx;
            vs[3 * i + 1] = a.vy;
            vs[3 * i + 2] = a.vz;
        }
    }

    // FLAG_ACTIVE (base.h:230) as the device holds it
    void sync_active() {
        const int n = System->GetNAtom();
        bool changed = false;
        for (int i = 0; i < n; i++) {
            const int on = (System->Atoms(i).flag & FLAG_ACTIVE) ? 1 : 0;
            if (on != active[i]) changed = true;
            active[i] = on;
        }
        if (changed) check(omdg_set_active(ctx, &active[0]), "omdg_set_active");
    }

    void scatter(bool xv) {
        const int n = System->GetNAtom();
        for (int i = 0; i < n; i++) {
            Atom& a = System->Atoms(i);
            if (xv) {
                a.x = xs[3 * i];
                a.y = xs[3 * i + 1];
                a.z = xs[3 * i + 2];
                a.vx = vs[3 * i];
                a.vy = vs[3 * i + 1];
                a.vz = vs[3 * i + 2];
            }
            a.fx = fs[3 * i];
            a.fy = fs[3 * i + 1];
            a.fz = fs[3 * i + 2];
            a.potential = pots[i];
            a.virial = virs[i];
        }
    }

public:
    explicit GPUIntegrator(OMD_FLOAT time_step = -1.0, int gpu = 0)
        : MDIntegrator(time_step), ctx(NULL), device(gpu) {
        set_name("GB300 VERLET INTEGRATOR");
    }

    virtual ~GPUIntegrator() {
        if (ctx) omdg_destroy(ctx);
    }

    // The parameter or table file of a kernel whose PrintInfo does not name one.
    GPUIntegrator* SetForceFile(ForceKernel* fk, const std::string& path) {
        files.push_back(std::make_pair(fk, path));
        return this;
    }

    virtual void Init(MDSystem* sys) {
        MDIntegrator::Init(sys);
        for (int i = 0; i < (int)sys->Modifies.size(); i++)
            if (sys->Modifies[i]->type_of("EMBEDDING_FUNCTION")) sys->Modifies[i]->Deactivate();
        check(omdg_create(&ctx, device), "omdg_create");
        const double lo[3] = {sys->Box.x0, sys->Box.y0, sys->Box.z0};
        const double hi[3] = {sys->Box.x1, sys->Box.y1, sys->Box.z1};
        const int per[3] = {(sys->PBoundary & PERIODIC_X) ? 1 : 0, (sys->PBoundary & PERIODIC_Y) ? 1 : 0,
                            (sys->PBoundary & PERIODIC_Z) ? 1 : 0};
        check(omdg_set_box(ctx, lo, hi, per), "omdg_set_box");
        const int n = sys->GetNAtom();
        const int ntypes = (int)sys->SystemAtoms.size();
        xs.assign(3 * (size_t)n, 0.0);
        vs.assign(3 * (size_t)n, 0.0);
        fs.assign(3 * (size_t)n, 0.0);
        pots.assign(n, 0.0);
        virs.assign(n, 0.0);
        active.assign(n, 1);
        std::vector<int> type(n);
        std::vector<double> mass(ntypes), znum(ntypes);
        for (int t = 0; t < ntypes; t++) {
            mass[t] = sys->SystemAtoms[t]->M;
            znum[t] = sys->SystemAtoms[t]->Z;
        }
        for (int i = 0; i < n; i++) type[i] = sys->Atoms(i).tid;
        gather();
        check(omdg_set_atoms(ctx, n, &xs[0], &vs[0], &type[0], ntypes, &mass[0], &znum[0]), "omdg_set_atoms");
        // the kernel matrix MDIntegrator::Init filled (integrator.cpp:85-97):
        // each kernel once, with the type pair it serves
        std::vector<ForceKernel*> done;
        for (int a = 0; a < NType; a++)
            for (int b = a; b < NType; b++) {
                ForceKernel* fk = Forces[a][b];
                bool seen = fk == NULL;
                for (size_t q = 0; q < done.size() && !seen; q++) seen = done[q] == fk;
                if (seen) continue;
                done.push_back(fk);
                const std::string file = file_of(fk);
                if (fk->type_of("TABLE_FORCE_EAM"))
                    check(omdg_add_eam(ctx, a, b, file.c_str()), "omdg_add_eam " + file);
                else if (fk->type_of("TABLE PAIR FORCE"))
                    check(omdg_add_pair_table(ctx, a, b, file.c_str(), 0), "omdg_add_pair_table " + file);
                else if (fk->type_of("tersoff_bond_order"))
                    check(omdg_add_tersoff(ctx, a, b, file.c_str()), "omdg_add_tersoff " + file);
                else if (!file.empty())
                    check(omdg_add_sw(ctx, a, b, file.c_str()), "omdg_add_sw " + file);
                else
                    die("GPUIntegrator: no device kernel for " + fk->get_name() + " (SetForceFile names its file)");
            }
        check(omdg_set_timestep(ctx, TimeStep), "omdg_set_timestep");
        double skin = -1.0;
        SysParam->peek("verlet.radtole", skin, -1.0);
        check(omdg_set_neighbor(ctx, skin > 0.0 ? skin : 0.3, 0), "omdg_set_neighbor");
        check(omdg_set_first_step_mode(ctx, 1), "omdg_set_first_step_mode");
        sync_active();
    }

    virtual void Iterate() {
        SyncData(SYNC_SPACE);
        System->ExecuteModifies(MODIFY_PRE_CALCULATION);
        gather();
        sync_active();
        check(omdg_set_state(ctx, &xs[0], &vs[0]), "omdg_set_state");
        check(omdg_compute_forces(ctx), "omdg_compute_forces");
        check(omdg_get_state(ctx, NULL, NULL, &fs[0], &pots[0], &virs[0]), "omdg_get_state");
        scatter(false);
        SyncData(SYNC_FORCE);
        System->ExecuteModifies(MODIFY_POST_FORCE);
    }

    virtual void Integrate() {
        gather();
        sync_active();
        check(omdg_step_io(ctx, &xs[0], &vs[0], 1, &xs[0], &vs[0], &fs[0]), "omdg_step_io");
        check(omdg_get_state(ctx, NULL, NULL, NULL, &pots[0], &virs[0]), "omdg_get_state");
        scatter(true);
        System->ExecuteModifies(MODIFY_PRE_CALCULATION);  // host lists the detectors iterate
    }
};

}  // namespace omd

#endif
