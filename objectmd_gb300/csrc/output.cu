// Output path: the reference's data file (AtomContainer::DumpAtoms,
// container.cpp:417-519) and SysMonitor's md.out lines (SysMonitor.h), both
// fed from device state (one read-back per dump) and the device ledger ring
// (per-step Step, ElapsedTime, TimeStep and energies, copied at omdg_sync).
// Text is formatted as the reference formats it (iostream fixed/scientific
// with the container's precisions; DataSlot printf formats).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <string>
#include <vector>

#include "device_common.cuh"

using namespace omdg;

namespace {

Context* C(omdg_ctx* c) { return static_cast<Context*>(c); }

// Per-atom columns printed between x y z and the write mode's fields, as
// DumpAtoms prints the printable aux variables (container.cpp:467-490).
struct AuxColumns {
    std::vector<std::string> names;
    std::vector<const double*> data;  // caller order, one value per atom
    std::string format;               // printf format of every column
};

std::string fmt(const char* f, double v) {
    char buf[128];
    std::snprintf(buf, sizeof(buf), f, v);
    return buf;
}

// AtomContainer::DumpAtoms (container.cpp:417-519) from a state read back
// in caller order.
int write_data_file(Context* c, const char* path, int mode, int posprec, int valprec, const char* material,
                    const std::vector<std::string>& info, const AuxColumns* aux, const int* gid) {
    if (mode & OMDG_WM_ZIP) return set_error(c, OMDG_EINVAL, "WM_ZIP (a gzip child process) is not supported");
    const int n = c->n;
    std::vector<double> x(3 * (size_t)n), v(3 * (size_t)n), f(3 * (size_t)n), pot(n), vir(n);
    int rc = omdg_get_state(static_cast<omdg_ctx*>(c), x.data(), v.data(), f.data(), pot.data(), vir.data());
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
        for (const std::string& l : info) out << '#' << l << '\n';
        if (material && material[0]) out << "#$ Material " << material << "\n";
        out << "#$ Fields x y z";
        if (aux)
            for (const std::string& name : aux->names) out << " " << name;
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
        if (aux)
            for (const double* col : aux->data) out << fmt(aux->format.c_str(), col[i]) << " ";
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

bool dump_args_ok(const char* path, int posprec, int valprec, int ninfo, const char* const* info) {
    return path && posprec >= 0 && valprec >= 0 && posprec <= 30 && valprec <= 30 && ninfo >= 0 &&
           (ninfo == 0 || info);
}

std::vector<std::string> info_lines(int ninfo, const char* const* info) {
    std::vector<std::string> v;
    for (int i = 0; i < ninfo; i++) v.push_back(info[i] ? info[i] : "");
    return v;
}

}  // namespace

extern "C" {

int omdg_dump_atoms(omdg_ctx* ctx, const char* path, int mode, int posprec, int valprec, const char* material,
                    int ninfo, const char* const* info, const int* gid) {
    Context* c = C(ctx);
    if (!c || !dump_args_ok(path, posprec, valprec, ninfo, info)) return OMDG_EINVAL;
    if (c->n == 0) return set_error(c, OMDG_ESTATE, "no atoms");
    cudaSetDevice(c->device);
    return write_data_file(c, path, mode, posprec, valprec, material, info_lines(ninfo, info), nullptr, gid);
}

int omdg_dump_thermo(omdg_ctx* ctx, const char* path, int mode, int posprec, int valprec, const char* material,
                     int ninfo, const char* const* info, const char* aux_format, double* summary) {
    Context* c = C(ctx);
    if (!c || !dump_args_ok(path, posprec, valprec, ninfo, info)) return OMDG_EINVAL;
    if (c->n == 0) return set_error(c, OMDG_ESTATE, "no atoms");
    const double ercut = thermo_ercut(c);
    if (!(ercut > 0)) return set_error(c, OMDG_ESTATE, "the thermo detector is off (omdg_set_thermo_detector)");
    cudaSetDevice(c->device);
    const int n = c->n;
    std::vector<double> temp(n), dens(n), x(3 * (size_t)n), v(3 * (size_t)n), vir(n);
    int rc = omdg_local_thermo(ctx, temp.data(), dens.data(), nullptr);
    if (rc) return rc;
    if ((rc = omdg_get_state(ctx, x.data(), v.data(), nullptr, nullptr, vir.data()))) return rc;
    std::vector<unsigned> flag;
    if (c->flags_used) {
        flag.resize(n);
        if ((rc = io_get_flags(c, flag.data()))) return rc;
    }
    auto active = [&](int i) { return flag.empty() || (flag[i] & 1u); };
    const double fac_t = 2.0 / 3.0 / 8.61734279e-05;  // MDUnit temperature factor (unit.h:115-131)
    const double fac_p = 160.22;                        // MD_GIGAPASCAL (conversion.h:39)
    const double volcut = 4.0 * M_PI * ercut * ercut * ercut / 3.0;  // ThermoDetector::Init
    // ExtractTemperature / ExtractPressure (ThermoDetector.h:232-296): the
    // neighbour count from the density, sum m|v - v_cm|^2 from the
    // temperature, the local pressure from both and the atom's virial
    std::vector<double> pres(n);
    double avg_t = 0, avg_d = 0, avg_p = 0;
    int navg = 0, npres = 0;
    for (int i = 0; i < n; i++) {
        const double nneig = std::round(dens[i] * volcut);
        const double sumek = 2.0 * temp[i] * nneig / fac_t;
        pres[i] = nneig == 0 ? 0.0 : fac_p * (dens[i] * vir[i] / 6.0 + sumek / (3.0 * volcut));
        if (!active(i)) continue;
        avg_p += pres[i];
        npres++;
        if (nneig < 2) continue;
        avg_t += temp[i];
        avg_d += dens[i];
        navg++;
    }
    avg_t = navg > 0 ? avg_t / navg : 0.0;
    avg_d = navg > 0 ? avg_d / navg : 0.0;
    avg_p = npres > 0 ? avg_p / npres : 0.0;
    // MeasureSystemTempPres (ThermoDetector.h:329-420): kinetic temperature
    // about the centre-of-mass velocity, pressure over the atoms' bounding box
    double cm[3] = {0, 0, 0}, mass = 0, lo[3], hi[3], vsum = 0, twoek = 0;
    for (int d = 0; d < 3; d++) lo[d] = DBL_MAX, hi[d] = -DBL_MAX;
    int natom = 0;
    for (int i = 0; i < n; i++) {
        if (!active(i)) continue;
        const double m = c->mass[c->caller_type[i]];
        for (int d = 0; d < 3; d++) {
            cm[d] += m * v[3 * (size_t)i + d];
            lo[d] = std::min(lo[d], x[3 * (size_t)i + d]);
            hi[d] = std::max(hi[d], x[3 * (size_t)i + d]);
        }
        mass += m;
        vsum += vir[i];
        natom++;
    }
    for (int d = 0; d < 3; d++) cm[d] /= mass;
    for (int i = 0; i < n; i++) {
        if (!active(i)) continue;
        const double* vi = &v[3 * (size_t)i];
        const double ax = vi[0] - cm[0], ay = vi[1] - cm[1], az = vi[2] - cm[2];
        twoek += c->mass[c->caller_type[i]] * (ax * ax + ay * ay + az * az);
    }
    double vol = 1.0;
    for (int d = 0; d < 3; d++) vol *= (hi[d] - lo[d]) > 0.0 ? (hi[d] - lo[d]) : 1.0;
    const double sys_t = fac_t * 0.5 * twoek / natom;
    const double sys_p = fac_p * (0.5 * vsum + twoek) / (3.0 * vol);  // System->Virial is half the atoms' sum
    if (summary) {
        summary[0] = sys_t;
        summary[1] = sys_p;
        summary[2] = avg_t;
        summary[3] = avg_d;
        summary[4] = avg_p;
    }
    // the detector's volume (pushed when it initialises), the caller's lines,
    // then ThermoDetector::Measure's and DataDumper::Measure's
    std::vector<std::string> lines = {"$ DetectorVolume " + fmt("%0.5E", volcut) + " Ang^3"};
    for (const std::string& l : info_lines(ninfo, info)) lines.push_back(l);
    lines.push_back("$ Temperature " + fmt("%0.5e", sys_t) + " K (kinetic)");
    lines.push_back("$ Pressure " + fmt("%0.5e", sys_p) + " GPa");
    lines.push_back("$ Time " + fmt("%0.5e", c->elapsed));
    AuxColumns aux;
    aux.names = {"temp", "press", "dens"};
    aux.data = {temp.data(), pres.data(), dens.data()};
    aux.format = aux_format && aux_format[0] ? aux_format : "%0.5e";  // ClaimAuxVariable's default (system.cpp:1312-1314)
    return write_data_file(c, path, mode, posprec, valprec, material, lines, &aux, nullptr);
}

int omdg_monitor_append(omdg_ctx* ctx, const char* path, int every, int header) {
    Context* c = C(ctx);
    if (!c || !path || every < 1) return OMDG_EINVAL;
    FILE* fo = std::fopen(path, header ? "w" : "a");
    if (!fo) return set_error(c, OMDG_EFILE, std::string("unable to create file ") + path);
    // a thermo detector registers four more slots (ThermoDetector.h:118-127)
    const bool thermo = thermo_ercut(c) > 0;
    if (header)  // SysMonitor::Measure's label line
        std::fputs(thermo ? "#@ t: dt: Ek: Ep: E: temp: avtemp: pres: avpres: \n" : "#@ t: dt: Ek: Ep: E: \n", fo);
    for (int k = 0; k < c->last_rows; k++) {
        const double* r = c->h_ledger + (size_t)LEDGER_W * k;
        const int step = (int)r[4];
        if (step == 0 || step % every) continue;  // Detect: Step % every; Measure skips Step 0
        const double ep = r[1] - c->base_potential;             // RelPotential
        const double e = r[0] + r[1] - c->base_potential;       // MechanicEnergy
        std::fprintf(fo, "%d %0.6E %0.3E %0.10E %0.10E %0.10E ", step, r[5], r[6], r[0], ep, e);
        if (thermo) std::fprintf(fo, "%0.3E %0.3E %0.3E %0.3E ", r[8], r[9], r[10], r[11]);
        std::fputs("\n", fo);
    }
    const bool ok = !std::ferror(fo);
    std::fclose(fo);
    return ok ? OMDG_OK : set_error(c, OMDG_EFILE, std::string("error writing ") + path);
}

}  // extern "C"
