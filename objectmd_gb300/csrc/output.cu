// Output path: the reference's data file (AtomContainer::DumpAtoms,
// container.cpp:417-519) and SysMonitor's md.out lines (SysMonitor.h), both
// fed from device state (one read-back per dump) and the device ledger ring
// (per-step Step, ElapsedTime, TimeStep and energies, copied at omdg_sync).
// Text is formatted as the reference formats it (iostream fixed/scientific
// with the container's precisions; DataSlot printf formats).
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <string>
#include <vector>

#include "device_common.cuh"

using namespace omdg;

namespace {

Context* C(omdg_ctx* c) { return static_cast<Context*>(c); }

}  // namespace

extern "C" {

int omdg_dump_atoms(omdg_ctx* ctx, const char* path, int mode, int posprec, int valprec, const char* material,
                    int ninfo, const char* const* info, const int* gid) {
    Context* c = C(ctx);
    if (!c || !path || posprec < 0 || valprec < 0 || posprec > 30 || valprec > 30 || ninfo < 0 ||
        (ninfo > 0 && !info))
        return OMDG_EINVAL;
    if (c->n == 0) return set_error(c, OMDG_ESTATE, "no atoms");
    if (mode & OMDG_WM_ZIP) return set_error(c, OMDG_EINVAL, "WM_ZIP (a gzip child process) is not supported");
    cudaSetDevice(c->device);
    const int n = c->n;
    std::vector<double> x(3 * (size_t)n), v(3 * (size_t)n), f(3 * (size_t)n), pot(n), vir(n);
    int rc = omdg_get_state(ctx, x.data(), v.data(), f.data(), pot.data(), vir.data());
    if (rc) return rc;
    std::vector<unsigned> flag;
    if (c->flags_used) {
        flag.resize(n);
        if ((rc = io_get_flags(c, flag.data()))) return rc;
    }
    std::ofstream out(path, (mode & OMDG_WM_APPEND) ? std::ios::app : std::ios::trunc);
    if (!out.good()) return set_error(c, OMDG_EFILE, std::string("unable to create file ") + path);
    if (!(mode & OMDG_WM_BARE) && !(mode & OMDG_WM_APPEND)) {
        out << "#####################################\n"
            << "#  Object-MD data file\n"
            << "#  (c) 2005 Rosandi\n#\n";
        out << "#$ Box " << c->box.lo[0] << " " << c->box.lo[1] << " " << c->box.lo[2] << " " << c->box.hi[0] << " "
            << c->box.hi[1] << " " << c->box.hi[2] << "\n";
        for (int i = 0; i < ninfo; i++) out << '#' << (info[i] ? info[i] : "") << '\n';
        if (material && material[0]) out << "#$ Material " << material << "\n";
        out << "#$ Fields x y z";
        if (mode & OMDG_WM_VELOCITY) out << " vx vy vz";
        if (mode & OMDG_WM_FORCE) out << " fx fy fz";
        if (mode & OMDG_WM_POTENTIAL) out << " pot";
        if (mode & OMDG_WM_VIRIAL) out << " vir";
        if (mode & OMDG_WM_TID) out << " id";
        if (mode & OMDG_WM_GID) out << " gid";
        if (mode & OMDG_WM_NID) out << " nid";
        out << " --\n";
    }
    for (int i = 0; i < n; i++) {
        if (!flag.empty() && !(flag[i] & 1u) && !(mode & OMDG_WM_DEADATOM)) continue;  // inactive atoms
        out << std::fixed << std::setprecision(posprec);
        out << x[3 * i] << " " << x[3 * i + 1] << " " << x[3 * i + 2] << " ";
        out << std::scientific << std::setprecision(valprec);
        if (mode & OMDG_WM_VELOCITY) out << v[3 * i] << " " << v[3 * i + 1] << " " << v[3 * i + 2] << " ";
        if (mode & OMDG_WM_FORCE) out << f[3 * i] << " " << f[3 * i + 1] << " " << f[3 * i + 2] << " ";
        if (mode & OMDG_WM_POTENTIAL) out << pot[i] << " ";
        if (mode & OMDG_WM_VIRIAL) out << vir[i] << " ";
        if (mode & OMDG_WM_TID) out << c->caller_type[i] << " ";
        if (mode & OMDG_WM_GID) out << (gid ? gid[i] : 0) << " ";
        if (mode & OMDG_WM_NID) out << i << " ";
        out << "\n";
    }
    out.close();
    if (out.fail()) return set_error(c, OMDG_EFILE, std::string("error writing ") + path);
    return OMDG_OK;
}

int omdg_monitor_append(omdg_ctx* ctx, const char* path, int every, int header) {
    Context* c = C(ctx);
    if (!c || !path || every < 1) return OMDG_EINVAL;
    FILE* fo = std::fopen(path, header ? "w" : "a");
    if (!fo) return set_error(c, OMDG_EFILE, std::string("unable to create file ") + path);
    if (header) std::fputs("#@ t: dt: Ek: Ep: E: \n", fo);  // SysMonitor::Measure's label line
    for (int k = 0; k < c->last_rows; k++) {
        const double* r = c->h_ledger + (size_t)LEDGER_W * k;
        const int step = (int)r[4];
        if (step == 0 || step % every) continue;  // Detect: Step % every; Measure skips Step 0
        const double ep = r[1] - c->base_potential;             // RelPotential
        const double e = r[0] + r[1] - c->base_potential;       // MechanicEnergy
        std::fprintf(fo, "%d %0.6E %0.3E %0.10E %0.10E %0.10E \n", step, r[5], r[6], r[0], ep, e);
    }
    const bool ok = !std::ferror(fo);
    std::fclose(fo);
    return ok ? OMDG_OK : set_error(c, OMDG_EFILE, std::string("error writing ") + path);
}

}  // extern "C"
