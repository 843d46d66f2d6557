// Binary checkpoint codec in the reference's format (MDSystem::SaveSimulation
// / LoadSimulation, system.cpp:726-827; AtomContainer::Save / Load,
// container.cpp:554-680).  Host code only: the context-level save and load
// (api.cu) gather and scatter the device state around it.
#include <cstdio>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "../../include/omdg.h"

static_assert(sizeof(omdg_atom_record) == 232, "Atom record is 232 bytes (base.h:114-125)");
static_assert(sizeof(long long) == 8, "time_t is 8 bytes on LP64");

namespace {

const char kSignature[] = "OMD (c) Y ROSANDI";  // system.cpp:732
const char kEndHeader[] = "== END OF CONFIG HEADER ===";  // system.cpp:759
const char kContainer[] = "$ATOMCONTAINER:";  // container.cpp:563

int fail(char* err, int len, const std::string& msg) {
    if (err && len > 0) {
        std::strncpy(err, msg.c_str(), (size_t)len - 1);
        err[len - 1] = 0;
    }
    return OMDG_EFILE;
}

struct Writer {
    FILE* f;
    bool ok = true;
    void raw(const void* p, size_t n) { ok = ok && std::fwrite(p, 1, n, f) == n; }
    void tag32(const char* s) {  // 32-byte NUL-padded tag
        char b[32];
        std::memset(b, 0, 32);
        std::strncpy(b, s, 31);
        raw(b, 32);
    }
    void str(const char* s) {  // WRITEST: int size (with NUL), bytes
        const int sz = (int)std::strlen(s) + 1;
        raw(&sz, sizeof(int));
        raw(s, (size_t)sz);
    }
    template <class T>
    void val(const T& v) {
        raw(&v, sizeof(T));
    }
};

struct Reader {
    FILE* f;
    bool ok = true;
    void raw(void* p, size_t n) { ok = ok && std::fread(p, 1, n, f) == n; }
    void tag32(char* b) {
        raw(b, 32);
        b[31] = 0;
    }
    bool str(std::string& out) {  // READST
        int sz = 0;
        raw(&sz, sizeof(int));
        if (!ok || sz <= 0 || sz > (1 << 24)) return ok = false;
        std::vector<char> b((size_t)sz);
        raw(b.data(), (size_t)sz);
        b.back() = 0;
        out.assign(b.data());
        return ok;
    }
    template <class T>
    void val(T& v) {
        raw(&v, sizeof(T));
    }
};

void write_vars(Writer& w, const omdg_sim_vars& v) {  // SaveVariables (system.cpp:656-668)
    w.val(v.begin_time);
    w.val(v.step);
    w.val(v.pboundary);
    w.val(v.energy);
    w.val(v.kinetic);
    w.val(v.virial);
    w.val(v.potential);
    w.val(v.base_potential);
    w.val(v.elapsed_time);
    w.raw(v.box, sizeof(v.box));
    w.val(v.write_mode);
}

void read_vars(Reader& r, omdg_sim_vars& v) {  // LoadVariables (system.cpp:670-682)
    r.val(v.begin_time);
    r.val(v.step);
    r.val(v.pboundary);
    r.val(v.energy);
    r.val(v.kinetic);
    r.val(v.virial);
    r.val(v.potential);
    r.val(v.base_potential);
    r.val(v.elapsed_time);
    r.raw(v.box, sizeof(v.box));
    r.val(v.write_mode);
}

void copy_field(char* dst, size_t cap, const std::string& s) {
    std::strncpy(dst, s.c_str(), cap - 1);
    dst[cap - 1] = 0;
}

// Everything after the signature, up to the containers.
struct Header {
    omdg_sim_vars vars;
    char stamp[32];
    std::vector<std::string> labels, values, names;
};

bool read_header(Reader& r, Header& h, std::string& why) {
    char b[32];
    r.tag32(b);
    if (!r.ok || std::string(kSignature) != b) {
        why = "not an Object-MD binary file (signature)";
        return false;
    }
    r.tag32(h.stamp);
    std::memset(&h.vars, 0, sizeof(h.vars));
    read_vars(r, h.vars);
    int nvar = 0;
    r.val(nvar);
    if (!r.ok || nvar < 0 || nvar > (1 << 20)) {
        why = "bad restart-variable count";
        return false;
    }
    for (int i = 0; i < nvar; i++) {
        std::string l, v;
        if (!r.str(l) || !r.str(v)) {
            why = "truncated restart variables";
            return false;
        }
        h.labels.push_back(l);
        h.values.push_back(v);
    }
    int ncont = 0;
    r.val(ncont);
    if (!r.ok || ncont < 0 || ncont > (1 << 16)) {
        why = "bad container count";
        return false;
    }
    for (int i = 0; i < ncont; i++) {
        r.tag32(b);
        h.names.push_back(b);
    }
    r.tag32(b);
    if (!r.ok || std::string(kEndHeader) != b) {
        why = "missing end-of-header mark";
        return false;
    }
    return true;
}

// One container block; the atoms are appended to out when given.
bool read_container(Reader& r, omdg_container_desc& d, std::vector<omdg_atom_record>* out, std::string& why) {
    char b[32];
    r.tag32(b);
    if (!r.ok || std::string(kContainer) != b) {
        why = "missing container mark";
        return false;
    }
    std::string name, mat, file, param;
    if (!r.str(name) || !r.str(mat) || !r.str(file) || !r.str(param)) {
        why = "truncated container strings";
        return false;
    }
    std::memset(&d, 0, sizeof(d));
    copy_field(d.name, sizeof(d.name), name);
    copy_field(d.material, sizeof(d.material), mat);
    copy_field(d.filename, sizeof(d.filename), file);
    copy_field(d.param, sizeof(d.param), param);
    r.val(d.id);
    r.val(d.mass);
    r.val(d.z);
    r.val(d.value);
    r.val(d.posprec);
    r.val(d.valprec);
    r.val(d.write_mode);
    r.val(d.natoms);
    if (!r.ok || d.natoms < 0) {
        why = "bad container header";
        return false;
    }
    if (out) {
        const size_t at = out->size();
        out->resize(at + (size_t)d.natoms);
        r.raw(out->data() + at, sizeof(omdg_atom_record) * (size_t)d.natoms);
    } else {
        r.ok = r.ok && std::fseek(r.f, (long)(sizeof(omdg_atom_record) * (size_t)d.natoms), SEEK_CUR) == 0;
    }
    if (!r.ok) why = "truncated atom records";
    return r.ok;
}

}  // namespace

extern "C" {

int omdg_checkpoint_write(const char* path, const char* stamp, const omdg_sim_vars* vars, int nvar,
                          const char* const* labels, const char* const* values, int ncont,
                          const omdg_container_desc* cont, const omdg_atom_record* atoms, char* err, int err_len) {
    if (!path || !vars || nvar < 0 || ncont < 0 || (nvar > 0 && (!labels || !values)) || (ncont > 0 && !cont))
        return OMDG_EINVAL;
    long total = 0;
    for (int k = 0; k < ncont; k++) {
        if (cont[k].natoms < 0) return OMDG_EINVAL;
        total += cont[k].natoms;
    }
    if (total > 0 && !atoms) return OMDG_EINVAL;
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(err, err_len, std::string("cannot create ") + path);
    Writer w{f};
    w.tag32(kSignature);
    char st[32];
    std::memset(st, 0, 32);
    if (stamp) {
        std::strncpy(st, stamp, 31);
    } else {  // system.cpp:736-739
        std::time_t now;
        std::time(&now);
        std::snprintf(st, 32, "%s", std::ctime(&now));
    }
    w.raw(st, 32);
    write_vars(w, *vars);
    w.val(nvar);
    for (int i = 0; i < nvar; i++) {
        w.str(labels[i] ? labels[i] : "");
        w.str(values[i] ? values[i] : "");
    }
    w.val(ncont);
    for (int k = 0; k < ncont; k++) w.tag32(cont[k].name);
    w.tag32(kEndHeader);
    const omdg_atom_record* a = atoms;
    for (int k = 0; k < ncont; k++) {  // MDSystem::Save: each container appended in order
        const omdg_container_desc& d = cont[k];
        w.tag32(kContainer);
        w.str(d.name);
        w.str(d.material);
        w.str(d.filename);
        w.str(d.param);
        w.val(d.id);
        w.val(d.mass);
        w.val(d.z);
        w.val(d.value);
        w.val(d.posprec);
        w.val(d.valprec);
        w.val(d.write_mode);
        w.val(d.natoms);
        if (d.natoms > 0) w.raw(a, sizeof(omdg_atom_record) * (size_t)d.natoms);
        a += d.natoms;
    }
    const bool ok = w.ok && !std::ferror(f);
    const bool closed = std::fclose(f) == 0;
    return ok && closed ? OMDG_OK : fail(err, err_len, std::string("error writing ") + path);
}

int omdg_checkpoint_info(const char* path, int* ncont, int* natoms, int* nvar, char* err, int err_len) {
    if (!path) return OMDG_EINVAL;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(err, err_len, std::string("cannot open ") + path);
    Reader r{f};
    Header h;
    std::string why;
    bool ok = read_header(r, h, why);
    long total = 0;
    for (size_t k = 0; ok && k < h.names.size(); k++) {
        omdg_container_desc d;
        ok = read_container(r, d, nullptr, why);
        total += d.natoms;
    }
    std::fclose(f);
    if (!ok) return fail(err, err_len, why + " in " + path);
    if (ncont) *ncont = (int)h.names.size();
    if (natoms) *natoms = (int)total;
    if (nvar) *nvar = (int)h.labels.size();
    return OMDG_OK;
}

int omdg_checkpoint_read(const char* path, omdg_sim_vars* vars, char* stamp, int ncont_cap, omdg_container_desc* cont,
                         int natom_cap, omdg_atom_record* atoms, char* var_buf, int var_buf_len, char* err,
                         int err_len) {
    if (!path) return OMDG_EINVAL;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(err, err_len, std::string("cannot open ") + path);
    Reader r{f};
    Header h;
    std::string why;
    bool ok = read_header(r, h, why);
    std::vector<omdg_container_desc> ds;
    std::vector<omdg_atom_record> recs;
    for (size_t k = 0; ok && k < h.names.size(); k++) {
        omdg_container_desc d;
        ok = read_container(r, d, &recs, why);
        ds.push_back(d);
    }
    std::fclose(f);
    if (!ok) return fail(err, err_len, why + " in " + path);
    if ((int)ds.size() > ncont_cap && cont) return fail(err, err_len, "container array too small");
    if ((long)recs.size() > natom_cap && atoms) return fail(err, err_len, "atom array too small");
    if (vars) *vars = h.vars;
    if (stamp) std::memcpy(stamp, h.stamp, 32);
    if (cont) std::copy(ds.begin(), ds.end(), cont);
    if (atoms && !recs.empty()) std::memcpy(atoms, recs.data(), sizeof(omdg_atom_record) * recs.size());
    if (var_buf && var_buf_len > 0) {
        std::string packed;
        for (size_t i = 0; i < h.labels.size(); i++) {
            packed += h.labels[i];
            packed.push_back(0);
            packed += h.values[i];
            packed.push_back(0);
        }
        if ((int)packed.size() > var_buf_len) return fail(err, err_len, "restart-variable buffer too small");
        std::memcpy(var_buf, packed.data(), packed.size());
    }
    return OMDG_OK;
}

}  // extern "C"
