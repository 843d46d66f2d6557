// C ABI of libomdg (include/omdg.h): context lifetime, atom/box upload,
// potential registration, neighbour list control, the step driver (eager or
// a captured CUDA graph with a conditional rebuild node) and read-back.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <map>
#include <sstream>

#include "device_common.cuh"

namespace omdg {

size_t step_state_bytes();
int step_state_init(Context* c);
int step_state_reset(Context* c, int reset_row, int rebuild_every);
int step_state_read(Context* c, long long* step, int* row, int* rebuild);
int step_state_resume(Context* c, long long step, double elapsed);
int step_state_set_dt(Context* c);
int step_state_times(Context* c, double* dt, double* elapsed);
int step_state_fetch(Context* c, unsigned* status, long long* step, int* row, double* elapsed, int rows);
int step_state_rewind(Context* c);
int step_clear_rebuild(Context* c);
int step_flag_requested_replicas(Context* c);
int launch_set_rebuild_cond(Context* c, cudaGraphConditionalHandle h);
int threebody_prepare(Context* c);

int set_error(Context* c, int code, const std::string& msg) {
    if (c) c->last_error = msg;
    return code;
}

int check_cuda(Context* c, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return OMDG_OK;
    return set_error(c, e == cudaErrorMemoryAllocation ? OMDG_ENOMEM : OMDG_ECUDA,
                     std::string(what) + ": " + cudaGetErrorString(e));
}

static int status_error(Context* c, unsigned st);

int check_status(Context* c) {
    unsigned st = 0;
    cudaError_t e = cudaMemcpyAsync(&st, c->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return check_cuda(c, e, "status read");
    return status_error(c, st);
}

static std::string fmt(const char* f, double v) {
    char b[64];
    std::snprintf(b, sizeof(b), f, v);
    return b;
}

// The reference's text for an overlap (CalcSqrDistance, gadget.cpp:149-159):
// the pair's distance, enumeration numbers (caller order) and positions.
static std::string overlap_text(Context* c, unsigned si, unsigned sj) {
    if (si == ~0u || (int)si >= c->n || (int)sj >= c->n) return "CalcSqrDistance: overlapping atoms";
    double p[2][3];
    int nid[2];
    const unsigned ij[2] = {si, sj};
    for (int a = 0; a < 2; a++) {
        cudaMemcpy(&p[a][0], c->x + ij[a], sizeof(double), cudaMemcpyDeviceToHost);
        cudaMemcpy(&p[a][1], c->y + ij[a], sizeof(double), cudaMemcpyDeviceToHost);
        cudaMemcpy(&p[a][2], c->z + ij[a], sizeof(double), cudaMemcpyDeviceToHost);
        cudaMemcpy(&nid[a], c->id + ij[a], sizeof(int), cudaMemcpyDeviceToHost);
    }
    double r2 = 0.0;
    for (int d = 0; d < 3; d++) {
        double dd = p[0][d] - p[1][d];
        if (c->box.periodic[d]) dd -= c->box.L[d] * std::nearbyint(dd / c->box.L[d]);
        r2 += dd * dd;
    }
    return "CalcSqrDistance: overlapping atoms: r=" + fmt("%1.1E", std::sqrt(r2)) + " between atom nid=" +
           std::to_string(nid[0]) + " and nid=" + std::to_string(nid[1]) + " (" + fmt("%0.5E", p[0][0]) + "," +
           fmt("%0.5E", p[0][1]) + "," + fmt("%0.5E", p[0][2]) + ") -- (" + fmt("%0.5E", p[1][0]) + "," +
           fmt("%0.5E", p[1][1]) + "," + fmt("%0.5E", p[1][2]) + ")";
}

// The reference's text for a table read outside its range (TableReader::read,
// treader.cpp:199-218), from the recorded value and table.
static std::string range_text(Context* c, unsigned vbits, unsigned src) {
    const int pi = (int)(src >> 2), sec = (int)(src & 3u);
    if (src == ~0u || pi >= (int)c->pots.size() || sec > 2) return "table read outside its range";
    const Potential& p = c->pots[pi];
    const HostTable& t = sec == 0 ? p.t0 : (sec == 1 ? p.t1 : p.t2);
    float vf;
    std::memcpy(&vf, &vbits, sizeof(vf));
    const double r = vf, rval = r - t.off;
    const int x = (int)(rval / t.dr);
    const double dx = rval - (double)x * t.dr;
    return std::string(x > t.n - 1 ? "high" : "low") + " limit exeeded in " + t.name + "@" + t.file +
           " (read) index=" + std::to_string(x) + " r=" + fmt("%0.5E", r) + " delta=" + fmt("%0.5E", dx) +
           " low_limit=" + fmt("%0.5E", t.off) + " hi_limit=" + fmt("%0.5E", t.max_range());
}

// Maps (and clears) a non-zero device status word; the status block's
// details name the first overlapping pair or out-of-range value.
static int status_error(Context* c, unsigned st) {
    if (!st) return OMDG_OK;
    unsigned det[ST_WORDS];
    cudaMemcpyAsync(det, c->d_status, sizeof(det), cudaMemcpyDeviceToHost, c->stream);
    cudaStreamSynchronize(c->stream);
    static const unsigned blank[ST_RANGE_SRC + 1] = {0u, ~0u, ~0u, ~0u, ~0u};
    cudaMemcpyAsync(c->d_status, blank, sizeof(blank), cudaMemcpyHostToDevice, c->stream);
    cudaStreamSynchronize(c->stream);
    // the list may hold what the bad input made of it: the next use rebuilds it
    if (st & (ERR_OVERLAP | ERR_NONFINITE | ERR_CELL | ERR_TABLE_RANGE)) c->list_valid = false;
    // the reference meets an overlap (gadget.cpp:149) before the table read it would fail
    if (st & ERR_OVERLAP) return set_error(c, OMDG_EOVERLAP, overlap_text(c, det[ST_OV_I], det[ST_OV_J]));
    if (st & ERR_TABLE_RANGE) return set_error(c, OMDG_ERANGE, range_text(c, det[ST_RANGE_V], det[ST_RANGE_SRC]));
    if (st & ERR_NONFINITE) return set_error(c, OMDG_ENONFINITE, "non-finite position or force");
    if (st & ERR_NBR_OVERFLOW) return set_error(c, OMDG_ESTATE, "neighbour capacity exceeded");
    if (st & ERR_TIMEOUT) return set_error(c, OMDG_ECUDA, "a bounded device wait expired (tensor-core kernel)");
    return set_error(c, OMDG_ECUDA, "device status word set");
}

// ------------------------------------------------------------- profiling
static cudaEvent_t take_event(Context* c) {
    if (!c->event_pool.empty()) {
        cudaEvent_t e = c->event_pool.back();
        c->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

static int timer_index(Context* c, const char* name) {
    for (size_t k = 0; k < c->timers.size(); k++)
        if (c->timers[k].name == name) return (int)k;
    c->timers.push_back(KernelTimer{name, 0.0, 0});
    return (int)c->timers.size() - 1;
}

static int g_open_timer = -1;
static cudaEvent_t g_open_event = nullptr;

void prof_begin(Context* c, const char* name) {
    if (!c->profiling) return;
    g_open_timer = timer_index(c, name);
    g_open_event = take_event(c);
    cudaEventRecord(g_open_event, c->stream);
}

void prof_end(Context* c) {
    if (!c->profiling || g_open_timer < 0) return;
    cudaEvent_t e = take_event(c);
    cudaEventRecord(e, c->stream);
    c->pending.push_back(std::make_pair(g_open_timer, std::make_pair(g_open_event, e)));
    g_open_timer = -1;
}

void prof_collect(Context* c) {
    if (c->pending.empty()) return;
    cudaStreamSynchronize(c->stream);
    for (auto& p : c->pending) {
        float ms = 0;
        cudaEventElapsedTime(&ms, p.second.first, p.second.second);
        c->timers[p.first].ms += ms;
        c->timers[p.first].calls++;
        c->event_pool.push_back(p.second.first);
        c->event_pool.push_back(p.second.second);
    }
    c->pending.clear();
}

// ------------------------------------------------------------- memory
template <typename T>
static bool dalloc(T*& p, size_t count) {
    cudaFree(p);
    p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc(&p, count * sizeof(T)) == cudaSuccess;
}

static void free_atoms(Context* c) {
    void* ptrs[] = {c->x,    c->y,     c->z,      c->vx,     c->vy,          c->vz,          c->fx,
                    c->fy,   c->fz,    c->pe,     c->vir,    c->pack,        c->xref,        c->loc,         c->type,
                    c->id,   c->inv,   c->fp,     c->femb,   c->cell,        c->perm,        c->stage_d,
                    c->stage_i, c->cell_sorted, c->f64, c->extra, c->stage_extra, c->nnb, c->d_red, c->aflag,
                    c->snap_d, c->snap_i,
                    c->ters_wide, c->nbmask};
    for (void* p : ptrs) cudaFree(p);
    c->x = c->y = c->z = c->vx = c->vy = c->vz = nullptr;
    c->fx = c->fy = c->fz = c->pe = c->vir = nullptr;
    c->pack = nullptr;
    c->xref = nullptr;
    c->loc = nullptr;
    c->nbmask = nullptr;
    c->nbmask_valid = false;
    c->type = c->id = c->inv = c->ters_wide = nullptr;
    c->fp = c->femb = nullptr;
    c->cell = c->perm = nullptr;
    c->stage_d = nullptr;
    c->stage_i = nullptr;
    c->cell_sorted = nullptr;
    c->f64 = nullptr;
    c->snap_d = nullptr;
    c->snap_i = nullptr;
    c->extra = c->stage_extra = nullptr;
    c->nnb = nullptr;
    c->d_red = nullptr;
    c->aflag = nullptr;
    c->cap = 0;
}

static int alloc_atoms(Context* c, int n) {
    free_atoms(c);
    int cap = n;
    bool ok = dalloc(c->x, cap) && dalloc(c->y, cap) && dalloc(c->z, cap) && dalloc(c->vx, cap) &&
              dalloc(c->vy, cap) && dalloc(c->vz, cap) && dalloc(c->fx, cap) && dalloc(c->fy, cap) &&
              dalloc(c->fz, cap) && dalloc(c->pe, cap) && dalloc(c->vir, cap) && dalloc(c->pack, cap) &&
              dalloc(c->xref, cap) && dalloc(c->loc, cap) && dalloc(c->nbmask, cap) && dalloc(c->type, cap) && dalloc(c->id, cap) && dalloc(c->inv, cap) &&
              dalloc(c->fp, cap) && dalloc(c->femb, cap) && dalloc(c->cell, cap) && dalloc(c->perm, cap) &&
              dalloc(c->stage_d, (size_t)6 * cap) && dalloc(c->stage_i, (size_t)3 * cap) && dalloc(c->aflag, cap) &&
              dalloc(c->cell_sorted, cap) && dalloc(c->nnb, cap) && dalloc(c->ters_wide, (size_t)cap + 1);
    // block partials: the kick's blocks, or a force kernel's with the kick in its epilogue (>= 8 atoms a block)
    int nb = grid_for(cap, 8) + 1;
    ok = ok && dalloc(c->d_red, (size_t)4 * nb);
    ok = ok && dalloc(c->snap_d, (size_t)6 * cap) && dalloc(c->snap_i, (size_t)3 * cap);
    if (ok && !c->snap_state) ok = cudaMalloc(&c->snap_state, step_state_bytes()) == cudaSuccess;
    if (!ok) return set_error(c, OMDG_ENOMEM, "atom arrays");
    c->cap = cap;
    c->red_cap = nb;
    cudaMemsetAsync(c->fx, 0, sizeof(float) * cap, c->stream);
    cudaMemsetAsync(c->fy, 0, sizeof(float) * cap, c->stream);
    cudaMemsetAsync(c->fz, 0, sizeof(float) * cap, c->stream);
    cudaMemsetAsync(c->pe, 0, sizeof(float) * cap, c->stream);
    cudaMemsetAsync(c->vir, 0, sizeof(float) * cap, c->stream);
    return OMDG_OK;
}

void invalidate_graph(Context* c);

// ------------------------------------------------------------- geometry
static void compute_frame(Context* c) {
    BoxGeom& b = c->box;
    double ext = 0;
    for (int d = 0; d < 3; d++) ext = std::max(ext, b.L[d]);
    double P = 2048.0;
    while (P < 8.0 * ext) P *= 2.0;
    for (int d = 0; d < 3; d++) {
        b.org[d] = b.lo[d];
        b.P[d] = P;
        b.Lh[d] = (float)b.L[d];
        b.Ll[d] = (float)(b.L[d] - (double)b.Lh[d]);
    }
}

}  // namespace omdg

using namespace omdg;


// graph state kept beside the context
struct GraphState {
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
    cudaStream_t side = nullptr;
    bool valid = false;
    // the same step with download branches into pinned host arrays
    // (omdg_step_io), keyed by the x, v, f output pointers
    cudaGraphExec_t io_exec = nullptr;
    cudaGraph_t io_graph = nullptr;
    cudaStream_t io_side = nullptr;
    cudaEvent_t io_ev[4] = {};
    double* io_key[3] = {};
    long io_kernels = 0;
    bool io_valid = false;
};
static std::map<Context*, GraphState> g_graphs;

namespace omdg {
void invalidate_graph(Context* c) {
    auto it = g_graphs.find(c);
    if (it == g_graphs.end()) return;
    GraphState& gs = it->second;
    if (gs.exec) cudaGraphExecDestroy(gs.exec);
    if (gs.graph) cudaGraphDestroy(gs.graph);
    if (gs.io_exec) cudaGraphExecDestroy(gs.io_exec);
    if (gs.io_graph) cudaGraphDestroy(gs.io_graph);
    gs.exec = gs.io_exec = nullptr;
    gs.graph = gs.io_graph = nullptr;
    gs.valid = gs.io_valid = false;
}
}  // namespace omdg

extern "C" {

int omdg_create(omdg_ctx** out, int device) {
    if (!out) return OMDG_EINVAL;
    *out = nullptr;
    omdg_ctx* c = new omdg_ctx();
    c->device = device;
    cudaError_t e = cudaSetDevice(device);
    int sms = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (sms > 0) c->num_sms = sms;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_status, sizeof(unsigned) * ST_WORDS);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_flags, sizeof(int) * 8);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_state, step_state_bytes());
    if (e == cudaSuccess) e = cudaMalloc(&c->d_mass, sizeof(double) * MAX_TYPES);
    c->ledger_cap = 1 << 16;
    if (e == cudaSuccess) e = cudaMalloc(&c->d_ledger, sizeof(double) * LEDGER_W * c->ledger_cap);
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_ledger, sizeof(double) * LEDGER_W * c->ledger_cap);
    if (e == cudaSuccess) e = cudaMallocHost(&c->h_sync, 16 + step_state_bytes());
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_status, 0xff, sizeof(unsigned) * ST_WORDS, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_status, 0, sizeof(unsigned), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_flags, 0, sizeof(int) * 8, c->stream);
    if (e != cudaSuccess) {
        delete c;
        return OMDG_ECUDA;
    }
    step_state_init(c);
    *out = c;
    return OMDG_OK;
}

int omdg_destroy(omdg_ctx* c) {
    if (!c) return OMDG_OK;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    invalidate_graph(c);
    auto it = g_graphs.find(c);
    if (it != g_graphs.end()) {
        GraphState& gs = it->second;
        if (gs.side) cudaStreamDestroy(gs.side);
        if (gs.io_side) cudaStreamDestroy(gs.io_side);
        for (cudaEvent_t ev : gs.io_ev)
            if (ev) cudaEventDestroy(ev);
        g_graphs.erase(it);
    }
    free_atoms(c);
    cudaFree(c->snap_state);
    cudaFree(c->nbr);
    cudaFree(c->rev);
    cudaFree(c->slot_buf);
    tile_release(c);
    cudaFree(c->cell_count);
    cudaFree(c->cell_start);
    cudaFree(c->cell_fill);
    cudaFree(c->cell_tile_sum);
    cudaFree(c->d_rep_start);
    cudaFree(c->d_rep_of);
    cudaFree(c->d_rep_geom);
    cudaFree(c->d_rep_shift);
    cudaFree(c->d_rep_sums);
    cudaFree(c->d_rep_flag);
    cudaFree(c->d_rep_builds);
    cudaFree(c->d_cell_rep);
    cudaFree(c->d_status);
    cudaFree(c->d_flags);
    cudaFree(c->d_state);
    cudaFree(c->d_mass);
    cudaFree(c->d_ledger);
    cudaFreeHost(c->h_ledger);
    cudaFreeHost(c->h_sync);
    for (auto& p : c->pots) {
        for (int k = 0; k < 3; k++) {
            cudaFree(p.d_coef[k]);
            cudaFree(p.d_coef64[k]);
            if (k == 0) cudaFree(p.d_coef2);
        }
        nn_release(p);
    }
    ttm_release(c);
    for (auto e : c->event_pool) cudaEventDestroy(e);
    cudaStreamDestroy(c->stream);
    delete c;
    return OMDG_OK;
}

const char* omdg_last_error(omdg_ctx* c) { return c ? c->last_error.c_str() : "null context"; }

int omdg_get_stream(omdg_ctx* c, void** stream) {
    if (!c || !stream) return OMDG_EINVAL;
    *stream = (void*)c->stream;
    return OMDG_OK;
}

int omdg_set_replicas(omdg_ctx* c, int nrep, const int* natoms, const double* lo, const double* hi,
                      const int periodic[3]) {
    if (!c || nrep <= 0 || !natoms || !lo || !hi || !periodic) return OMDG_EINVAL;
    std::vector<int> start(nrep + 1, 0);
    double blo[3] = {1e300, 1e300, 1e300}, bhi[3] = {-1e300, -1e300, -1e300};
    for (int r = 0; r < nrep; r++) {
        if (natoms[r] <= 0) return set_error(c, OMDG_EINVAL, "a replica without atoms");
        start[r + 1] = start[r] + natoms[r];
        for (int d = 0; d < 3; d++) {
            if (!(hi[3 * r + d] > lo[3 * r + d])) return set_error(c, OMDG_EINVAL, "replica box hi must exceed lo");
            blo[d] = std::min(blo[d], lo[3 * r + d]);
            bhi[d] = std::max(bhi[d], hi[3 * r + d]);
        }
    }
    c->nrep = nrep;
    c->rep_start = start;
    c->rep_lo.assign(lo, lo + 3 * nrep);
    c->rep_hi.assign(hi, hi + 3 * nrep);
    for (int d = 0; d < 3; d++) {
        c->rep_periodic[d] = periodic[d] ? 1 : 0;
        // the context box bounds every replica; periodicity lives in the replicas
        c->box.lo[d] = blo[d];
        c->box.hi[d] = bhi[d];
        c->box.L[d] = bhi[d] - blo[d];
        c->box.periodic[d] = 0;
    }
    cudaFree(c->d_rep_geom);
    cudaFree(c->d_rep_shift);
    cudaFree(c->d_rep_of);
    cudaFree(c->d_rep_sums);
    cudaFree(c->d_rep_start);
    cudaFree(c->d_rep_flag);
    cudaFree(c->d_rep_builds);
    cudaFree(c->d_cell_rep);
    c->d_rep_start = nullptr;
    c->d_rep_geom = c->d_rep_shift = nullptr;
    c->d_rep_of = nullptr;
    c->rep_of_cap = 0;
    c->d_rep_sums = nullptr;
    c->d_rep_flag = c->d_rep_builds = c->d_cell_rep = nullptr;
    c->have_box = true;
    compute_frame(c);
    c->list_valid = false;
    invalidate_graph(c);
    return OMDG_OK;
}

int omdg_set_box(omdg_ctx* c, const double lo[3], const double hi[3], const int periodic[3]) {
    if (!c || !lo || !hi || !periodic) return OMDG_EINVAL;
    if (c->nrep > 0) return set_error(c, OMDG_ESTATE, "the context is in replica mode");
    for (int d = 0; d < 3; d++) {
        if (!(hi[d] > lo[d])) return set_error(c, OMDG_EINVAL, "box hi must exceed lo");
        c->box.lo[d] = lo[d];
        c->box.hi[d] = hi[d];
        c->box.L[d] = std::fabs(hi[d] - lo[d]);  // system.cpp:852-854
        c->box.periodic[d] = periodic[d] ? 1 : 0;
    }
    c->have_box = true;
    compute_frame(c);
    c->list_valid = false;
    invalidate_graph(c);
    return OMDG_OK;
}

int omdg_set_atoms(omdg_ctx* c, int n, const double* x, const double* v, const int* type, int ntypes,
                   const double* mass_by_type, const double* z_by_type) {
    if (!c || n <= 0 || !x || !type || ntypes <= 0 || ntypes > MAX_TYPES || !mass_by_type) return OMDG_EINVAL;
    if (n > MAX_ATOMS) return set_error(c, OMDG_EINVAL, "too many atoms");
    if (!c->have_box) return set_error(c, OMDG_ESTATE, "set the box first");
    if (c->nrep > 0 && c->rep_start.back() != n)
        return set_error(c, OMDG_EINVAL, "n differs from the sum of the replicas' atom counts");
    cudaSetDevice(c->device);
    for (int i = 0; i < n; i++)
        if (type[i] < 0 || type[i] >= ntypes) return set_error(c, OMDG_EINVAL, "atom type out of range");
    int rc = alloc_atoms(c, n);
    if (rc) return rc;
    c->n = n;
    c->ntypes = ntypes;
    c->caller_type.assign(type, type + n);
    c->flags_used = false;
    c->elapsed = 0.0;
    c->step = 0;
    c->resume = false;
    for (int t = 0; t < MAX_TYPES; t++) {
        c->mass[t] = t < ntypes ? mass_by_type[t] : 0.0;
        c->zat[t] = (t < ntypes && z_by_type) ? z_by_type[t] : 0.0;
    }
    std::vector<double> hx(n), hy(n), hz(n), hvx(n, 0.0), hvy(n, 0.0), hvz(n, 0.0);
    std::vector<int> hid(n);
    for (int i = 0; i < n; i++) {
        hx[i] = x[3 * i];
        hy[i] = x[3 * i + 1];
        hz[i] = x[3 * i + 2];
        if (v) {
            hvx[i] = v[3 * i];
            hvy[i] = v[3 * i + 1];
            hvz[i] = v[3 * i + 2];
        }
        hid[i] = i;
    }
    cudaStream_t s = c->stream;
    cudaMemcpyAsync(c->x, hx.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(c->y, hy.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(c->z, hz.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(c->vx, hvx.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(c->vy, hvy.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(c->vz, hvz.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(c->type, type, sizeof(int) * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(c->id, hid.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(c->inv, hid.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s);
    const std::vector<unsigned> active(n, 1u);  // FLAG_ACTIVE, no groups
    cudaMemcpyAsync(c->aflag, active.data(), sizeof(unsigned) * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(c->d_mass, c->mass, sizeof(double) * MAX_TYPES, cudaMemcpyHostToDevice, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return check_cuda(c, e, "atom upload");
    if (c->use_f64 && !dalloc(c->f64, (size_t)4 * n)) return set_error(c, OMDG_ENOMEM, "FP64 force arrays");
    if (c->f64) cudaMemsetAsync(c->f64, 0, sizeof(double) * 4 * n, s);
    c->list_valid = false;
    c->first_run_done = false;
    c->maxnb = 0;
    cudaFree(c->nbr);
    cudaFree(c->rev);
    cudaFree(c->slot_buf);
    c->nbr = nullptr;
    c->rev = nullptr;
    c->slot_buf = nullptr;
    invalidate_graph(c);
    return integrate_pack(c);
}

int omdg_num_atoms(omdg_ctx* c, int* n) {
    if (!c || !n) return OMDG_EINVAL;
    *n = c->n;
    return OMDG_OK;
}

}  // extern "C"

// ------------------------------------------------------------- read-back
namespace omdg {
static int fetch_ids(Context* c, std::vector<int>& id) {
    id.resize(c->n);
    cudaError_t e = cudaMemcpyAsync(id.data(), c->id, sizeof(int) * c->n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return check_cuda(c, e, "id read");
}

template <typename T>
static int fetch(Context* c, const T* d, std::vector<T>& h, size_t count) {
    h.resize(count);
    cudaError_t e = cudaMemcpyAsync(h.data(), d, sizeof(T) * count, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return check_cuda(c, e, "read-back");
}
}  // namespace omdg

extern "C" {

int omdg_get_state(omdg_ctx* c, double* x, double* v, double* f, double* pot, double* vir) {
    if (!c) return OMDG_EINVAL;
    if (c->n == 0) return set_error(c, OMDG_ESTATE, "no atoms");
    cudaSetDevice(c->device);
    int rc = v ? resolve_thermostat(c) : OMDG_OK;
    if (rc) return rc;
    rc = io_get_state(c, x, v, f, pot, vir);
    if (rc) return rc;
    return check_cuda(c, cudaStreamSynchronize(c->stream), "state read-back");
}

// Positions set by the caller refresh the packs; the list stays valid
// unless an atom moved more than skin/2 since it was built (the upload's
// displacement check then requests the rebuild the next step takes).
// Velocities given by the caller replace any pending thermostat factor.
// The call returns once the caller's arrays have been read.
int omdg_set_state(omdg_ctx* c, const double* x, const double* v) {
    if (!c) return OMDG_EINVAL;
    if (c->n == 0) return set_error(c, OMDG_ESTATE, "no atoms");
    if (!x && !v) return OMDG_OK;
    cudaSetDevice(c->device);
    int rc = v ? drop_thermostat_factor(c) : OMDG_OK;
    if (rc) return rc;
    if ((rc = io_set_state(c, x, v))) return rc;
    return check_cuda(c, cudaStreamSynchronize(c->stream), "state upload");
}

int omdg_set_positions(omdg_ctx* c, const double* x) {
    if (!c || !x) return OMDG_EINVAL;
    return omdg_set_state(c, x, nullptr);
}

int omdg_set_velocities(omdg_ctx* c, const double* v) {
    if (!c || !v) return OMDG_EINVAL;
    return omdg_set_state(c, nullptr, v);
}

}  // extern "C"

// ------------------------------------------------------------- potentials
namespace omdg {

static int upload_table(Context* c, Potential& p, int k, HostTable& t, bool fp64) {
    std::vector<float4> h(t.n);
    for (int i = 0; i < t.n; i++) h[i] = make_float4((float)t.a[i], (float)t.b[i], (float)t.c[i], (float)t.d[i]);
    if (cudaMalloc(&p.d_coef[k], sizeof(float4) * t.n) != cudaSuccess)
        return set_error(c, OMDG_ENOMEM, "table upload");
    cudaMemcpy(p.d_coef[k], h.data(), sizeof(float4) * t.n, cudaMemcpyHostToDevice);
    DevTable& d = p.dt[k];
    d.src = (int)c->pots.size() * 4 + k;  // the potential is appended after its tables
    d.coef = p.d_coef[k];
    d.coef64 = nullptr;
    if (fp64) {
        std::vector<double4_32a> h64(t.n);
        for (int i = 0; i < t.n; i++) h64[i] = make_double4_32a(t.a[i], t.b[i], t.c[i], t.d[i]);
        if (cudaMalloc(&p.d_coef64[k], sizeof(double4_32a) * t.n) != cudaSuccess)
            return set_error(c, OMDG_ENOMEM, "table upload");
        cudaMemcpy(p.d_coef64[k], h64.data(), sizeof(double4_32a) * t.n, cudaMemcpyHostToDevice);
        d.coef64 = p.d_coef64[k];
    }
    d.off = (float)t.off;
    d.dr = (float)t.dr;
    d.inv_dr = (float)(1.0 / t.dr);
    d.off64 = t.off;
    d.dr64 = t.dr;
    d.n = t.n;
    d.rmult = t.rmult ? 1 : 0;
    d.allow_lo = t.allow_lo;
    d.allow_hi = t.allow_hi;
    d.out_lo = (float)t.out_lo;
    d.out_hi = (float)t.out_hi;
    d.rc = (float)t.max_range();
    d.rc64 = t.max_range();
    return OMDG_OK;
}

// A pair table contributes nothing beyond the start of its negligible tail
// (|value| and |slope| below 1e-9 eV and eV/A per pair there): such tails
// come from tables splined to zero well before their last knot, like the
// reference's Ar-Si ZBL table (zero past 3.2 A, knots to 5.1 A).  The list
// radius follows that shorter range; the reference's CutRadius (the whole
// table, tpair.h:59) stays what omdg_max_cut_radius reports.
constexpr double TABLE_TAIL_TOL = 1e-9;

void update_rc(Context* c) {
    // integrator.cpp:108-113: the largest CutRadius over all force kernels
    double m = -1.0, ref = -1.0;
    for (auto& p : c->pots) {
        if (p.kind == POT_PAIR)
            p.rc_list = c->table_full_range ? p.rc : std::min(p.rc, table_negligible_from(p.t0, TABLE_TAIL_TOL));
        else
            p.rc_list = p.rc;
        m = std::max(m, p.rc_list);
        ref = std::max(ref, p.rc);
    }
    c->rc_ref = ref;
    // the detector's cutoff (its own, else the reference's CutRadius) must be in the list too
    if (c->ttm) m = std::max(m, thermo_ercut(c));
    c->rc_max = m;
    c->list_valid = false;
    c->maxnb = 0;
    invalidate_graph(c);
}

static int check_types(Context* c, int ta, int tb) {
    if (ta < 0 || tb < 0 || ta >= MAX_TYPES || tb >= MAX_TYPES) return set_error(c, OMDG_EINVAL, "bad type id");
    for (auto& p : c->pots)
        if ((p.ta == ta && p.tb == tb) || (p.ta == tb && p.tb == ta))
            return set_error(c, OMDG_EINVAL, "interaction for these types is already assigned (integrator.cpp:90-93)");
    return OMDG_OK;
}

// whitespace 'key value...' parameter file (param.cpp:77-98)
static bool read_params(const std::string& file, std::map<std::string, std::vector<std::string>>& kv) {
    std::ifstream fl(file.c_str());
    if (!fl.good()) return false;
    std::string line;
    while (std::getline(fl, line)) {
        size_t h = line.find('#');
        if (h != std::string::npos) line = line.substr(0, h);
        std::istringstream ss(line);
        std::string k, v;
        if (!(ss >> k)) continue;
        std::vector<std::string> vals;
        while (ss >> v) vals.push_back(v);
        kv[k] = vals;
    }
    return true;
}

static bool pnum(std::map<std::string, std::vector<std::string>>& kv, const char* k, double& out, int idx = 0) {
    auto it = kv.find(k);
    if (it == kv.end() || (int)it->second.size() <= idx) return false;
    out = std::strtod(it->second[idx].c_str(), nullptr);
    return true;
}

}  // namespace omdg

extern "C" {

int omdg_add_eam(omdg_ctx* c, int ta, int tb, const char* file) {
    if (!c || !file) return OMDG_EINVAL;
    if (ta != tb) return set_error(c, OMDG_EINVAL, "EAM between different types is not supported");
    int rc = check_types(c, ta, tb);
    if (rc) return rc;
    if (c->use_f64) return set_error(c, OMDG_EINVAL, "EAM cannot be combined with FP64 kernels");
    Potential p;
    p.kind = POT_EAM;
    p.ta = ta;
    p.tb = tb;
    std::string err;
    if ((rc = table_load(file, "PAIR", p.t0, err)) || (rc = table_load(file, "EDENS", p.t1, err)) ||
        (rc = table_load(file, "EMBED", p.t2, err)))
        return set_error(c, rc, err);
    if ((rc = upload_table(c, p, 0, p.t0, false)) || (rc = upload_table(c, p, 1, p.t1, false)) ||
        (rc = upload_table(c, p, 2, p.t2, false)))
        return rc;
    p.rc = p.t0.max_range();  // team.cpp:212
    c->pots.push_back(p);
    update_rc(c);
    return OMDG_OK;
}

int omdg_add_pair_table(omdg_ctx* c, int ta, int tb, const char* file, int fp64) {
    if (!c || !file) return OMDG_EINVAL;
    int rc = check_types(c, ta, tb);
    if (rc) return rc;
    if (fp64) {
        for (auto& q : c->pots)
            if (!q.fp64) return set_error(c, OMDG_EINVAL, "FP64 kernels cannot be mixed with FP32 kernels");
    } else if (c->use_f64) {
        return set_error(c, OMDG_EINVAL, "FP32 kernels cannot be mixed with FP64 kernels");
    }
    Potential p;
    p.kind = POT_PAIR;
    p.ta = ta;
    p.tb = tb;
    p.fp64 = fp64 != 0;
    std::string err;
    if ((rc = table_load(file, "", p.t0, err))) return set_error(c, rc, err);
    if ((rc = upload_table(c, p, 0, p.t0, p.fp64))) return rc;
    p.rc = p.t0.max_range();  // tpair.h:59
    c->pots.push_back(p);
    if (p.fp64 && !c->use_f64) {
        c->use_f64 = true;
        if (c->n > 0) {
            if (!dalloc(c->f64, (size_t)4 * c->n)) return set_error(c, OMDG_ENOMEM, "FP64 force arrays");
            cudaMemset(c->f64, 0, sizeof(double) * 4 * c->n);
        }
    }
    update_rc(c);
    return OMDG_OK;
}

int omdg_add_sw(omdg_ctx* c, int ta, int tb, const char* file) {
    if (!c || !file) return OMDG_EINVAL;
    int rc = check_types(c, ta, tb);
    if (rc) return rc;
    if (c->use_f64) return set_error(c, OMDG_EINVAL, "SW cannot be combined with FP64 kernels");
    std::map<std::string, std::vector<std::string>> kv;
    if (!read_params(file, kv)) return set_error(c, OMDG_EFILE, std::string("can not read ") + file);
    Potential p;
    p.kind = POT_SW;
    p.ta = ta;
    p.tb = tb;
    SWParams& s = p.sw;
    // sw.cpp:35-62
    bool ok = pnum(kv, "sw.epsilon", s.eps) && pnum(kv, "sw.A", s.A) && pnum(kv, "sw.B", s.B) &&
              pnum(kv, "sw.p", s.p) && pnum(kv, "sw.q", s.q) && pnum(kv, "sw.sigma", s.sigma) &&
              pnum(kv, "sw.a", s.a) && pnum(kv, "sw.lambda", s.lambda) && pnum(kv, "sw.gamma", s.gamma) &&
              pnum(kv, "sw.invers_cos0", s.icos0);
    if (!ok) return set_error(c, OMDG_EFILE, std::string("incomplete SW parameters in ") + file);
    s.usezbl = 0;
    auto z = kv.find("zbl");
    if (z != kv.end() && !z->second.empty()) {
        std::string v = z->second[0];
        s.usezbl = (v == "yes" || v == "true" || v == "1") ? 1 : 0;
    }
    if (s.usezbl) {
        ok = pnum(kv, "spline.range", s.sx0, 0) && pnum(kv, "spline.range", s.sx1, 1) &&
             pnum(kv, "spline.coeff", s.sa0, 0) && pnum(kv, "spline.coeff", s.sa1, 1) &&
             pnum(kv, "spline.coeff", s.sa2, 2) && pnum(kv, "spline.coeff", s.sa3, 3);
        if (!ok) return set_error(c, OMDG_EFILE, "incomplete SW ZBL spline parameters");
    }
    // sw.cpp:65-91
    s.rc = s.a * s.sigma;
    s.c1 = s.A * s.eps * s.p * s.B * std::pow(s.sigma, s.p);
    s.c2 = s.A * s.eps * s.q * std::pow(s.sigma, s.q);
    s.c3 = s.A * s.eps * s.B * std::pow(s.sigma, s.p + 1.0);
    s.c4 = s.A * s.eps * std::pow(s.sigma, s.q + 1.0);
    s.c5 = s.A * s.eps * s.B * std::pow(s.sigma, s.p);
    s.c6 = s.A * s.eps * std::pow(s.sigma, s.q);
    s.c7 = s.sigma * s.gamma;
    s.c8 = s.lambda * s.eps;
    s.c9 = 2.0 * s.lambda * s.eps;
    s.c10 = 1.0 / s.icos0;
    double z1 = c->zat[ta], z2 = c->zat[tb];
    if (z1 <= 0 || z2 <= 0) {
        z1 = z2 = 14.0;
    }
    double znor = 0.468521928 / (std::pow(z1, 0.23) + std::pow(z2, 0.23));
    s.zc = 14.39964415 * z1 * z2;
    s.ze0 = 3.2000 / znor;
    s.ze1 = 0.9423 / znor;
    s.ze2 = 0.4029 / znor;
    s.ze3 = 0.2016 / znor;
    p.rc = s.rc;  // sw.cpp:71
    c->pots.push_back(p);
    c->need_rev = true;
    update_rc(c);
    return OMDG_OK;
}

int omdg_add_tersoff(omdg_ctx* c, int ta, int tb, const char* file) {
    if (!c || !file) return OMDG_EINVAL;
    int rc = check_types(c, ta, tb);
    if (rc) return rc;
    if (c->use_f64) return set_error(c, OMDG_EINVAL, "Tersoff cannot be combined with FP64 kernels");
    std::map<std::string, std::vector<std::string>> kv;
    if (!read_params(file, kv)) return set_error(c, OMDG_EFILE, std::string("can not read ") + file);
    Potential p;
    p.kind = POT_TERSOFF;
    p.ta = ta;
    p.tb = tb;
    TersoffParams& t = p.ters;
    // tersoff.h:150-170 key names
    bool ok = pnum(kv, "tersoff.A", t.A) && pnum(kv, "tersoff.B", t.B) && pnum(kv, "tersoff.lambda_1", t.lambda1) &&
              pnum(kv, "tersoff.lambda_2", t.lambda2) && pnum(kv, "tersoff.lambda_3", t.lambda3) &&
              pnum(kv, "tersoff.beta", t.beta) && pnum(kv, "tersoff.n", t.n) && pnum(kv, "tersoff.c", t.c) &&
              pnum(kv, "tersoff.d", t.d) && pnum(kv, "tersoff.h", t.h) && pnum(kv, "tersoff.R", t.R) &&
              pnum(kv, "tersoff.D", t.D);
    if (!ok) return set_error(c, OMDG_EFILE, std::string("incomplete Tersoff parameters in ") + file);
    auto z = kv.find("tersoff.zbl");
    if (z != kv.end() && !z->second.empty() && z->second[0] == "true")
        return set_error(c, OMDG_EINVAL, "tersoff.zbl true is not supported (the reference disables it: tersoff.h:402)");
    p.rc = t.R + t.D;  // tersoff.h:183
    c->pots.push_back(p);
    c->need_rev = true;
    update_rc(c);
    return OMDG_OK;
}

int omdg_add_zbl(omdg_ctx* c, int ta, int tb, double rcut, double width) {
    if (!c || !(rcut > 0) || width < 0 || width >= rcut) return OMDG_EINVAL;
    int rc = check_types(c, ta, tb);
    if (rc) return rc;
    if (c->use_f64) return set_error(c, OMDG_EINVAL, "ZBL cannot be combined with FP64 kernels");
    Potential p;
    p.kind = POT_ZBL;
    p.ta = ta;
    p.tb = tb;
    ZBLParams& z = p.zbl;
    z.z1 = c->zat[ta];
    z.z2 = c->zat[tb];
    if (!(z.z1 > 0 && z.z2 > 0)) return set_error(c, OMDG_EINVAL, "ZBL needs atomic numbers (omdg_set_atoms z_by_type)");
    z.rc = rcut;
    z.width = width;
    // sw.cpp:84-91
    double znor = 0.468521928 / (std::pow(z.z1, 0.23) + std::pow(z.z2, 0.23));
    z.zc = 14.39964415 * z.z1 * z.z2;
    z.ze0 = 3.2000 / znor;
    z.ze1 = 0.9423 / znor;
    z.ze2 = 0.4029 / znor;
    z.ze3 = 0.2016 / znor;
    p.rc = rcut;
    c->pots.push_back(p);
    update_rc(c);
    return OMDG_OK;
}

int omdg_max_cut_radius(omdg_ctx* c, double* rc) {
    if (!c || !rc) return OMDG_EINVAL;
    *rc = c->rc_ref;
    return OMDG_OK;
}

int omdg_set_neighbor(omdg_ctx* c, double skin, int rebuild_every) {
    if (!c || skin < 0 || rebuild_every < 0) return OMDG_EINVAL;
    c->skin = skin;
    c->rebuild_every = rebuild_every;
    c->list_valid = false;
    c->maxnb = 0;
    invalidate_graph(c);
    return OMDG_OK;
}

}  // extern "C"

namespace omdg {

// Builds the list, sizing the per-atom capacity from the first build.
static int build_list(Context* c) {
    if (c->pots.empty()) return set_error(c, OMDG_ESTATE, "no force kernel (integrator.cpp:79)");
    nlist_prepare_geometry(c);
    if (int rt = tile_prepare(c)) return rt;
    if (c->nrep > 0) {
        if (c->rep_start.back() != c->n) return set_error(c, OMDG_ESTATE, "replica atom counts do not sum to n");
        int rc = replica_prepare(c);
        if (rc) return rc;
    }
    if (c->maxnb == 0) {
        // first build: estimate from the mean density, then fit to the measured maximum
        double vol = 1.0;
        for (int d = 0; d < 3; d++) vol *= c->box.L[d];
        if (c->nrep > 0) {
            vol = 0.0;
            for (int r = 0; r < c->nrep; r++) {
                double v = 1.0;
                for (int d = 0; d < 3; d++) v *= c->rep_hi[3 * r + d] - c->rep_lo[3 * r + d];
                vol += v;
            }
        }
        double rv = c->rc_max + c->skin;
        double est = c->n / vol * 4.18879 * rv * rv * rv;
        int m = c->nbr_capacity > 0 ? c->nbr_capacity : (int)(2.0 * est) + 32;
        int rc = nlist_reserve(c, m);
        if (rc) return rc;
    }
    for (int attempt = 0; attempt < 4; attempt++) {
        int zero = 0;
        cudaMemcpyAsync(c->d_flags + 1, &zero, sizeof(int), cudaMemcpyHostToDevice, c->stream);
        int rc = nlist_build(c);
        if (rc) return rc;
        int need = 0;
        cudaMemcpyAsync(&need, c->d_flags + 1, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
        cudaError_t e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return check_cuda(c, e, "build");
        unsigned st = 0;
        cudaMemcpy(&st, c->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost);
        if (st & ERR_NBR_OVERFLOW) {
            unsigned clr = st & ~ERR_NBR_OVERFLOW;
            cudaMemcpy(c->d_status, &clr, sizeof(unsigned), cudaMemcpyHostToDevice);
            int m = (int)(1.25 * std::max(need, c->maxnb)) + 16;
            c->maxnb = 0;
            rc = nlist_reserve(c, m);
            if (rc) return rc;
            invalidate_graph(c);
            continue;
        }
        return check_status(c);
    }
    return set_error(c, OMDG_ESTATE, "neighbour list did not fit");
}

int forces_compute(Context* c) {
    if (c->pots.empty()) return set_error(c, OMDG_ESTATE, "no force kernel");
    c->kick_fused = false;
    bool first = true;
    for (auto& p : c->pots) {
        if (p.fallback_only) continue;  // run by the potential that owns it
        if (c->nrep > 0 && p.kind != POT_TERSOFF && p.kind != POT_ZBL && !(p.kind == POT_PAIR && !p.fp64))
            return set_error(c, OMDG_EINVAL, "replica mode evaluates Tersoff, ZBL and FP32 pair-table kernels only");
        int rc = OMDG_OK;
        switch (p.kind) {
            case POT_EAM: rc = eam_launch(c, p, first); break;
            case POT_PAIR: rc = pair_launch(c, p, first); break;
            case POT_SW: rc = sw_launch(c, p, first); break;
            case POT_TERSOFF: rc = tersoff_launch(c, p, first); break;
            case POT_ZBL: rc = zbl_launch(c, p, first); break;
            case POT_NN: rc = nn_launch(c, p, first); break;
        }
        if (rc) return rc;
        first = false;
    }
    return post_force_modifies(c);  // MODIFY_POST_FORCE (integrator.cpp:215)
}

// Eager rebuild of the list when the device asks for it (reads the flag).
static int eager_maybe_rebuild(Context* c) {
    int rebuild = 0;
    int rc = step_state_read(c, nullptr, nullptr, &rebuild);
    if (rc) return rc;
    if (rebuild) {
        if ((rc = step_flag_requested_replicas(c))) return rc;
        if ((rc = step_clear_rebuild(c))) return rc;
        c->build_partial = c->nrep > 0;
        rc = nlist_build(c);
        c->build_partial = false;
        if (rc) return rc;
    }
    return OMDG_OK;
}

// io (omdg_step_io): x, v, f pinned host outputs (each may be null).  The
// captured step then forks a branch that writes x once the positions (and
// any rebuild's order) are final, f once the forces are, and v after the
// kick, while the force and kick kernels run; the branch joins before the
// step ends.
static int capture_step(Context* c, GraphState& gs, double* const* io = nullptr) {
    cudaStream_t s = c->stream;
    if (!gs.side) cudaStreamCreateWithFlags(&gs.side, cudaStreamNonBlocking);
    if (io && !gs.io_side) {
        cudaStreamCreateWithFlags(&gs.io_side, cudaStreamNonBlocking);
        for (cudaEvent_t& ev : gs.io_ev) cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    }
    long io_launches = 0;
    // one download on the branch once the main stream's work so far is done
    auto branch = [&](int k, double* x, double* v, double* f) -> int {
        if (!x && !v && !f) return OMDG_OK;
        cudaError_t e2 = cudaEventRecord(gs.io_ev[k], s);
        if (e2 == cudaSuccess) e2 = cudaStreamWaitEvent(gs.io_side, gs.io_ev[k], 0);
        if (e2 != cudaSuccess) return check_cuda(c, e2, "download branch");
        io_launches++;
        return io_rows_to_host(c, gs.io_side, x, v, f);
    };
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return check_cuda(c, e, "capture begin");
    long l0 = c->launches, l1 = 0, l2 = 0;
    int rc = (c->ttm && ttm_active(c)) ? ttm_pre(c) : OMDG_OK;  // PreIntegration (TTM_Homogen_SCNA.h:352)
    if (!rc) rc = energy_source(c);                                 // PreIntegration (EnergySource.h:113)
    if (!rc) rc = integrate_kick_drift(c, 0);
    cudaGraph_t g = nullptr;
    cudaStreamCaptureStatus cst;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    cudaGraphConditionalHandle h = 0;
    if (!rc) {
        e = cudaStreamGetCaptureInfo(s, &cst, nullptr, &g, nullptr, nullptr, nullptr);
        if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, 0, 0);
        if (e != cudaSuccess) rc = check_cuda(c, e, "conditional handle");
    }
    if (!rc) rc = launch_set_rebuild_cond(c, h);
    l1 = c->launches;
    cudaGraphNode_t cond_node = nullptr;
    if (!rc) {
        e = cudaStreamGetCaptureInfo(s, &cst, nullptr, &g, &deps, nullptr, &ndeps);
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeIf;
        cp.conditional.size = 1;
        if (e == cudaSuccess) e = cudaGraphAddNode(&cond_node, g, deps, nullptr, ndeps, &cp);
        if (e == cudaSuccess)
            e = cudaStreamUpdateCaptureDependencies(s, &cond_node, nullptr, 1, cudaStreamSetCaptureDependencies);
        if (e != cudaSuccess) rc = check_cuda(c, e, "conditional node");
        if (!rc) {
            // populate the body: the rebuild pipeline, captured on a side stream
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            e = cudaStreamBeginCaptureToGraph(gs.side, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) rc = check_cuda(c, e, "body capture");
            if (!rc) {
                c->stream = gs.side;
                c->build_in_step = true;
                c->build_partial = c->nrep > 0;  // the flagged replicas only
                rc = nlist_build(c);
                c->build_partial = false;
                c->build_in_step = false;
                c->stream = s;
                cudaGraph_t body_out = nullptr;
                e = cudaStreamEndCapture(gs.side, &body_out);
                if (!rc && e != cudaSuccess) rc = check_cuda(c, e, "body capture end");
            }
        }
    }
    l2 = c->launches;
    if (!rc && io) rc = branch(0, io[0], nullptr, nullptr);
    c->fuse_kick = true;
    if (!rc) rc = forces_compute(c);
    c->fuse_kick = false;
    if (!rc && io) rc = branch(1, nullptr, nullptr, io[2]);
    if (!rc) rc = integrate_kick(c, 0);
    if (!rc && c->ttm) rc = thermo_detect(c, true);  // ExecuteDetectors (system.cpp:976)
    if (!rc && io) rc = branch(2, nullptr, io[1], nullptr);
    if (!rc && io_launches > 0) {  // join the branch
        e = cudaEventRecord(gs.io_ev[3], gs.io_side);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, gs.io_ev[3], 0);
        if (e != cudaSuccess) rc = check_cuda(c, e, "download join");
    }
    long l3 = c->launches;
    // captured launches are counted when the graph replays, not here
    c->graph_step_kernels = (l1 - l0) + (l3 - l2);
    c->graph_body_kernels = l2 - l1;
    c->launches = l0;
    c->captured_builds += 1;
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(s, &graph);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return check_cuda(c, e, "capture end");
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        return check_cuda(c, e, "graph instantiate");
    }
    if (io) {
        gs.io_graph = graph;
        gs.io_exec = exec;
        gs.io_valid = true;
        for (int k = 0; k < 3; k++) gs.io_key[k] = io[k];
        gs.io_kernels = io_launches;
    } else {
        gs.graph = graph;
        gs.exec = exec;
        gs.valid = true;
    }
    // the rebuild count is advanced on the host only for eager builds
    return OMDG_OK;
}

}  // namespace omdg

extern "C" {

int omdg_build_neighbors(omdg_ctx* c) {
    if (!c) return OMDG_EINVAL;
    if (c->n == 0) return set_error(c, OMDG_ESTATE, "no atoms");
    cudaSetDevice(c->device);
    return build_list(c);
}

int omdg_get_neighbors(omdg_ctx* c, int* offsets, int* nbr_j, int* nbr_code, long cap, long* count) {
    if (!c || !offsets || !count) return OMDG_EINVAL;
    if (!c->list_valid) {
        int rc = omdg_build_neighbors(c);
        if (rc) return rc;
    }
    int n = c->n;
    std::vector<int> id, nn;
    std::vector<unsigned> nb;
    int rc = fetch_ids(c, id);
    if (rc) return rc;
    if ((rc = fetch(c, c->nnb, nn, n))) return rc;
    if ((rc = fetch(c, reinterpret_cast<const unsigned*>(c->nbr), nb, nlist_slots(c, c->maxnb)))) return rc;
    // rows in caller order, each sorted by (j, code)
    std::vector<int> sorted_of(n);
    for (int k = 0; k < n; k++) sorted_of[id[k]] = k;
    long total = 0;
    for (int k = 0; k < n; k++) total += nn[k];
    *count = total;
    if (total > cap || !nbr_j || !nbr_code) return set_error(c, OMDG_EINVAL, "neighbour output capacity too small");
    long pos = 0;
    std::vector<std::pair<int, int>> row;
    for (int i = 0; i < n; i++) {
        int k = sorted_of[i];
        row.clear();
        for (int s = 0; s < nn[k]; s++) {
            unsigned e = nb[nbr_at(k, s, c->nbr_hshift, c->maxnb)];
            row.push_back(std::make_pair(id[nbr_index(e)], omdg::nbr_code(e)));
        }
        std::sort(row.begin(), row.end());
        offsets[i] = (int)pos;
        for (auto& pr : row) {
            nbr_j[pos] = pr.first;
            nbr_code[pos] = pr.second;
            pos++;
        }
    }
    offsets[n] = (int)pos;
    return OMDG_OK;
}

int omdg_compute_forces(omdg_ctx* c) {
    if (!c) return OMDG_EINVAL;
    if (c->n == 0) return set_error(c, OMDG_ESTATE, "no atoms");
    cudaSetDevice(c->device);
    int rc;
    if (!c->list_valid && (rc = build_list(c))) return rc;
    else if ((rc = eager_maybe_rebuild(c))) return rc;  // moved more than skin/2 since the build
    if ((rc = threebody_prepare(c))) return rc;
    if ((rc = forces_compute(c))) return rc;
    if ((rc = measure_energies(c, 0))) return rc;
    if (c->ttm && (rc = thermo_detect(c, false))) return rc;
    prof_collect(c);
    if ((rc = check_status(c))) return rc;
    // a non-step evaluation writes the ledger row the next step would use
    int cur = 0;
    if ((rc = step_state_read(c, nullptr, &cur, nullptr))) return rc;
    double row[4];
    cudaMemcpy(row, c->d_ledger + LEDGER_W * (size_t)(cur % c->ledger_cap), sizeof(row), cudaMemcpyDeviceToHost);
    c->last_kin = row[0];
    c->last_pot = row[1];
    c->last_vir = row[2];
    return OMDG_OK;
}

int omdg_set_timestep(omdg_ctx* c, double dt) {
    if (!c || !(dt > 0)) return OMDG_EINVAL;
    c->dt = dt;
    cudaSetDevice(c->device);
    invalidate_graph(c);          // captured TTM kernels carry dt
    return step_state_set_dt(c);  // the step kernels read dt from the step state
}

int omdg_get_timestep(omdg_ctx* c, double* dt, double* elapsed) {
    if (!c) return OMDG_EINVAL;
    cudaSetDevice(c->device);
    return step_state_times(c, dt, elapsed);
}

// ------------------------------------------------------ impact-run modifies

static bool valid_group(int g) { return g >= -1 && g < 8; }

int omdg_set_groups(omdg_ctx* c, const unsigned char* member) {
    if (!c || !member) return OMDG_EINVAL;
    if (c->n == 0) return set_error(c, OMDG_ESTATE, "no atoms");
    cudaSetDevice(c->device);
    std::vector<unsigned> f(c->n);
    for (int i = 0; i < c->n; i++) f[i] = (unsigned)member[i] << 8;
    c->flags_used = true;
    invalidate_graph(c);
    return io_set_flags(c, f.data(), 0xFFu);  // group bits replaced, the active bit kept
}

int omdg_set_active(omdg_ctx* c, const int* active) {
    if (!c || !active) return OMDG_EINVAL;
    if (c->n == 0) return set_error(c, OMDG_ESTATE, "no atoms");
    cudaSetDevice(c->device);
    std::vector<unsigned> f(c->n);
    for (int i = 0; i < c->n; i++) f[i] = active[i] ? 1u : 0u;
    c->flags_used = true;
    c->list_valid = false;  // the list takes active atoms only
    invalidate_graph(c);
    return io_set_flags(c, f.data(), ~1u);
}

int omdg_get_active(omdg_ctx* c, int* active) {
    if (!c || !active) return OMDG_EINVAL;
    if (c->n == 0) return set_error(c, OMDG_ESTATE, "no atoms");
    cudaSetDevice(c->device);
    std::vector<unsigned> f(c->n);
    int rc = io_get_flags(c, f.data());
    if (rc) return rc;
    for (int i = 0; i < c->n; i++) active[i] = (int)(f[i] & 1u);
    return OMDG_OK;
}

int omdg_add_force_damper(omdg_ctx* c, int group, double factor) {
    if (!c || !valid_group(group) || !std::isfinite(factor)) return OMDG_EINVAL;
    if (c->post_ops.size() >= 4) return set_error(c, OMDG_EINVAL, "at most 4 force modifies");
    c->post_ops.push_back({1, group, factor, 0});
    c->flags_used = true;
    invalidate_graph(c);
    return OMDG_OK;
}

int omdg_add_coord_clamp(omdg_ctx* c, int group, const char* axes) {
    if (!c || !valid_group(group)) return OMDG_EINVAL;
    if (c->post_ops.size() >= 4) return set_error(c, OMDG_EINVAL, "at most 4 force modifies");
    // CoordClamp::Init (CoordClamp.h:28-33) tests `if(saxis.find('x'))`: an
    // axis is clamped when its letter is absent or not the first character
    // ("xyz" clamps y and z)
    const std::string a = axes ? axes : "xyz";
    int mask = 0;
    if (a.find('x') != 0) mask |= 1;
    if (a.find('y') != 0) mask |= 2;
    if (a.find('z') != 0) mask |= 4;
    c->post_ops.push_back({2, group, 0.0, mask});
    c->flags_used = true;
    invalidate_graph(c);
    return OMDG_OK;
}

int omdg_add_range_limiter(omdg_ctx* c, int group, double border) {
    if (!c || !valid_group(group) || !std::isfinite(border)) return OMDG_EINVAL;
    c->range_on = true;
    c->range_group = group;
    c->range_border = border;
    c->flags_used = true;
    invalidate_graph(c);
    return OMDG_OK;
}

int omdg_add_energy_source(omdg_ctx* c, double energy, double start, double width) {
    if (!c || !std::isfinite(energy) || !(start > 0) || !std::isfinite(width)) return OMDG_EINVAL;
    if (c->dyn_update > 0) return set_error(c, OMDG_EINVAL, "EnergySource is incompatible with DynamicTimeStep");
    if (c->thermo_tau > 0) return set_error(c, OMDG_EINVAL, "EnergySource with the Berendsen thermostat is not supported");
    // EnergySource::CheckParameter (EnergySource.h:85-95): pulse mode
    if (width < c->dt) width = c->dt;
    c->src_on = true;
    c->src_delta = energy * c->dt / width;
    c->src_start = start;
    c->src_width = width;
    invalidate_graph(c);
    return OMDG_OK;
}

int omdg_set_dynamic_timestep(omdg_ctx* c, double maxpath, double max_dt, int update) {
    if (!c || !(maxpath > 0) || !(max_dt > 0) || update < 1) return OMDG_EINVAL;
    if (c->ttm) return set_error(c, OMDG_EINVAL, "a dynamic time step cannot drive the TTM");
    if (c->src_on) return set_error(c, OMDG_EINVAL, "DynamicTimeStep is incompatible with EnergySource");
    c->dyn_update = update;
    c->dyn_maxpath = maxpath;
    c->dyn_maxdt = max_dt;
    // DynamicTimeStep::Init with no measured velocity: TimeStep = max
    c->dt = max_dt;
    cudaSetDevice(c->device);
    invalidate_graph(c);
    return step_state_set_dt(c);
}

int omdg_set_first_step_mode(omdg_ctx* c, int reference_first_step) {
    if (!c) return OMDG_EINVAL;
    c->reference_first_step = reference_first_step != 0;
    return OMDG_OK;
}

int omdg_set_compat(omdg_ctx* c, const char* key, int on) {
    if (!c || !key) return OMDG_EINVAL;
    std::string k(key);
    if (k == "first_step_zero_force") c->reference_first_step = on != 0;
    else if (k == "thermostat_counts_ghosts") c->thermo_count_ghosts = on != 0;
    else if (k == "pair_table_full_range") {
        c->table_full_range = on != 0;
        update_rc(c);
    } else return set_error(c, OMDG_EINVAL, "unknown compatibility key " + k);
    invalidate_graph(c);
    return OMDG_OK;
}

int omdg_set_thermostat(omdg_ctx* c, double temperature, double tau) {
    if (!c) return OMDG_EINVAL;
    if (tau > 0.0 && c->ttm && ttm_active(c))
        return set_error(c, OMDG_EINVAL, "the Berendsen thermostat and the two-temperature model exclude each other");
    if (tau > 0.0 && c->src_on)
        return set_error(c, OMDG_EINVAL, "EnergySource with the Berendsen thermostat is not supported");
    c->thermo_T = temperature;
    c->thermo_tau = tau;
    invalidate_graph(c);
    return OMDG_OK;
}

int omdg_step_async(omdg_ctx* c, int nsteps) {
    if (!c || nsteps < 0) return OMDG_EINVAL;
    if (c->n == 0) return set_error(c, OMDG_ESTATE, "no atoms");
    cudaSetDevice(c->device);
    int rc;
    if (!c->first_run_done && c->resume) {
        // CONTINUE_MODE (system.cpp:1004-1019): no FirstRun; the stored forces
        // drive the first half-kick and Step, P0 and the ledger continue
        if ((rc = build_list(c))) return rc;
        if ((rc = threebody_prepare(c))) return rc;
        if ((rc = step_state_init(c))) return rc;
        if ((rc = step_state_resume(c, c->resume_step, c->elapsed))) return rc;
        // one eager evaluation does the kernels' first-use setup outside the
        // step graph's capture; the stored forces then replace its result
        if ((rc = forces_compute(c))) return rc;
        if ((rc = check_status(c))) return rc;
        if ((rc = io_set_forces(c, c->resume_f.data()))) return rc;
        if ((rc = step_state_reset(c, 1, c->rebuild_every))) return rc;
        c->last_kin = c->resume_vars[0];
        c->last_pot = c->resume_vars[1];
        c->last_vir = c->resume_vars[2];
        c->base_potential = c->resume_vars[3];
        c->step = c->resume_step;
        c->resume = false;
        c->resume_f.clear();
        c->resume_f.shrink_to_fit();
        c->first_run_done = true;
    }
    if (!c->first_run_done) {
        // FirstRun (system.cpp:860-873): one force evaluation, energies, base potential
        c->begin_time = (long long)std::time(nullptr);
        if ((rc = build_list(c))) return rc;
        if ((rc = threebody_prepare(c))) return rc;
        if ((rc = step_state_init(c))) return rc;
        // TTM's first PreIntegration only measures (TTM_Homogen_SCNA.h:356-366)
        if (c->ttm && (rc = thermo_detect(c, false))) return rc;
        if ((rc = forces_compute(c))) return rc;
        c->first_measure = true;  // DynamicTimeStep's Step-0 update follows this measurement
        rc = measure_energies(c, 0);
        c->first_measure = false;
        if (rc) return rc;
        if ((rc = check_status(c))) return rc;
        double row[4];
        cudaMemcpy(row, c->d_ledger, sizeof(row), cudaMemcpyDeviceToHost);
        c->base_potential = row[1];
        c->last_kin = row[0];
        c->last_pot = row[1];
        c->last_vir = row[2];
        if (c->reference_first_step && (rc = zero_forces(c))) return rc;
        if ((rc = step_state_reset(c, 1, c->rebuild_every))) return rc;
        c->first_run_done = true;
    }
    if (!c->list_valid) {
        if ((rc = build_list(c))) return rc;
        if ((rc = threebody_prepare(c))) return rc;
    }
    if (c->async_steps == 0) {
        c->launches_at_sync = c->launches;
        cudaMemsetAsync(c->d_flags + 6, 0, sizeof(int), c->stream);  // the batch's first rebuild snapshots
    }
    if (c->profiling) {
        for (int k = 0; k < nsteps; k++) {
            if (c->ttm && ttm_active(c) && (rc = ttm_pre(c))) return rc;
            if ((rc = energy_source(c))) return rc;
            if ((rc = integrate_kick_drift(c, k))) return rc;
            c->build_in_step = true;
            rc = eager_maybe_rebuild(c);
            c->build_in_step = false;
            if (rc) return rc;
            c->fuse_kick = true;
            rc = forces_compute(c);
            c->fuse_kick = false;
            if (rc) return rc;
            if ((rc = integrate_kick(c, k))) return rc;
            if (c->ttm && (rc = thermo_detect(c, true))) return rc;
        }
        prof_collect(c);
    } else {
        GraphState& gs = g_graphs[c];
        if (!gs.valid) {
            if ((rc = capture_step(c, gs))) return rc;
        }
        for (int k = 0; k < nsteps; k++) {
            cudaError_t e = cudaGraphLaunch(gs.exec, c->stream);
            if (e != cudaSuccess) return check_cuda(c, e, "graph launch");
        }
        c->graph_steps += nsteps;
    }
    c->async_steps += nsteps;
    if (nsteps > 0 && c->thermo_tau > 0.0) c->lambda_pending = true;
    return OMDG_OK;
}

}  // extern "C"

namespace omdg {

// A neighbour row overflowed in a rebuild of the queued steps.  Every later
// rebuild was skipped; the snapshot holds the input of the queued steps'
// first rebuild (the state after that step's first half-kick and drift), at
// or before the one that overflowed.  Restore it, grow the rows, redo that
// rebuild and the rest of its step, then replay the steps still owed.  The counting sort and the list are deterministic functions of
// that state, so the trajectory is the one an ample capacity gives, bit for
// bit.  (The two-temperature model keeps electron state outside the
// snapshot; a run with it reports the overflow instead.)
static int recover_overflow(omdg_ctx* c) {
    const long owed_total = c->async_steps;
    int need = 0;
    cudaError_t e = cudaMemcpy(&need, c->d_flags + 1, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return check_cuda(c, e, "overflow recovery");
    // restore the rebuild's input and the step state as it was then
    {
        const size_t n = (size_t)c->n, cap = (size_t)c->cap;
        double* dst_d[6] = {c->x, c->y, c->z, c->vx, c->vy, c->vz};
        for (int k = 0; k < 6 && e == cudaSuccess; k++)
            e = cudaMemcpyAsync(dst_d[k], c->snap_d + k * cap, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream);
        int* dst_i[3] = {c->type, c->id, reinterpret_cast<int*>(c->aflag)};
        for (int k = 0; k < 3 && e == cudaSuccess; k++)
            e = cudaMemcpyAsync(dst_i[k], c->snap_i + k * cap, sizeof(int) * n, cudaMemcpyDeviceToDevice, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(c->d_state, c->snap_state, step_state_bytes(), cudaMemcpyDeviceToDevice, c->stream);
        const int zero = 0;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(step_state_halted(c), &zero, sizeof(int), cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return check_cuda(c, e, "overflow recovery");
    }
    int rowk = 0;  // ledger rows restart with the queued steps: the failed step's row is its index
    int rc = step_state_read(c, nullptr, &rowk, nullptr);
    if (rc) return rc;
    // grow the rows (status cleared), then the failed step's rebuild and the rest of that step
    static const unsigned blank[ST_RANGE_SRC + 1] = {0u, ~0u, ~0u, ~0u, ~0u};
    cudaMemcpy(c->d_status, blank, sizeof(blank), cudaMemcpyHostToDevice);
    const int m = (int)(1.25 * std::max(need, c->maxnb)) + 16;
    c->maxnb = 0;
    if ((rc = nlist_reserve(c, m))) return rc;
    invalidate_graph(c);
    if ((rc = build_list(c))) return rc;
    if ((rc = threebody_prepare(c))) return rc;
    c->fuse_kick = true;
    rc = forces_compute(c);
    c->fuse_kick = false;
    if (rc) return rc;
    if ((rc = integrate_kick(c, 0))) return rc;
    if ((rc = check_status(c))) return rc;
    c->overflow_recoveries++;
    const long done = (long)rowk + 1;  // steps finished, the recovered one included
    const long owed = owed_total - done;
    if (owed > 0 && (rc = omdg_step_async(c, (int)owed))) return rc;
    c->async_steps = owed_total;
    return omdg_sync(c);
}

}  // namespace omdg

extern "C" {

int omdg_sync(omdg_ctx* c) {
    if (!c) return OMDG_EINVAL;
    cudaSetDevice(c->device);
    unsigned status = 0;
    long long step = 0;
    int rows = 0;
    double elapsed = 0.0;
    // the queued steps write one ledger row each, from row 0: those rows
    // come back in the same round trip as the step state
    const int expect = (c->async_steps > 0 && c->async_steps <= c->ledger_cap) ? (int)c->async_steps : 0;
    int rc = step_state_fetch(c, &status, &step, &rows, &elapsed, expect);  // waits for the queued steps
    if (rc) return rc;
    if ((status & ERR_NBR_OVERFLOW) && !(status & ~ERR_NBR_OVERFLOW) && c->async_steps > 0 && c->snap_d &&
        !(c->ttm && ttm_active(c)))
        return recover_overflow(c);
    if ((rc = status_error(c, status))) {
        if (rc == OMDG_ESTATE) {
            // a neighbour row overflowed during the run: grow for the next call
            int m = (int)(1.25 * c->maxnb) + 16;
            c->maxnb = 0;
            nlist_reserve(c, m);
            c->list_valid = false;
            invalidate_graph(c);
        }
        c->async_steps = 0;
        return rc;
    }
    if (c->async_steps == 0) return OMDG_OK;
    c->step = step;
    c->elapsed = elapsed;
    const int cap = c->ledger_cap;
    const int nrow = std::min(rows, cap);
    if (nrow > 0 && rows != expect) {
        // (rows == expect: fetched with the step state)  The device ledger
        // is a ring: rows older than `cap` steps were overwritten; the rest
        // come back in order into the pinned copy
        const size_t w = sizeof(double) * LEDGER_W;
        cudaError_t e;
        if (rows <= cap) {
            e = cudaMemcpyAsync(c->h_ledger, c->d_ledger, w * nrow, cudaMemcpyDeviceToHost, c->stream);
        } else {
            const int first = rows % cap;
            e = cudaMemcpyAsync(c->h_ledger, c->d_ledger + (size_t)LEDGER_W * first, w * (cap - first),
                                cudaMemcpyDeviceToHost, c->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(c->h_ledger + (size_t)LEDGER_W * (cap - first), c->d_ledger, w * first,
                                    cudaMemcpyDeviceToHost, c->stream);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return check_cuda(c, e, "ledger read-back");
    }
    if (nrow > 0) {
        c->last_kin = c->h_ledger[LEDGER_W * (nrow - 1)];
        c->last_pot = c->h_ledger[LEDGER_W * (nrow - 1) + 1];
        c->last_vir = c->h_ledger[LEDGER_W * (nrow - 1) + 2];
    }
    c->last_rows = nrow;
    c->last_launches = c->launches - c->launches_at_sync;
    c->async_steps = 0;
    return step_state_rewind(c);
}

int omdg_step(omdg_ctx* c, int nsteps) {
    int rc = omdg_step_async(c, nsteps);
    if (rc) return rc;
    return omdg_sync(c);
}

int omdg_step_io(omdg_ctx* c, const double* x_in, const double* v_in, int nsteps, double* x_out, double* v_out,
                 double* f_out) {
    if (!c || nsteps < 1) return OMDG_EINVAL;
    if (c->n == 0) return set_error(c, OMDG_ESTATE, "no atoms");
    cudaSetDevice(c->device);
    int rc;
    if (x_in || v_in) {
        // read by the upload kernel, which completes before this call returns
        if (v_in && (rc = drop_thermostat_factor(c))) return rc;
        if ((rc = io_set_state(c, x_in, v_in))) return rc;
    }
    const size_t n3 = 3 * (size_t)c->n;
    // overlapped downloads: graph replay, pinned outputs, and no thermostat
    // factor pending on the velocities at the end of the step
    bool overlap = !c->profiling && c->thermo_tau <= 0.0 && (x_out || v_out || f_out);
    for (double* p : {x_out, v_out, f_out})
        if (overlap && p && !host_view(c, p, n3)) overlap = false;
    if (!overlap) {
        if ((rc = omdg_step(c, nsteps))) return rc;
        if (!x_out && !v_out && !f_out) return OMDG_OK;
        return omdg_get_state(c, x_out, v_out, f_out, nullptr, nullptr);
    }
    if ((rc = omdg_step_async(c, nsteps - 1))) return rc;  // also FirstRun and list upkeep
    if (!c->list_valid) {
        if ((rc = build_list(c))) return rc;
        if ((rc = threebody_prepare(c))) return rc;
    }
    GraphState& gs = g_graphs[c];
    double* key[3] = {x_out, v_out, f_out};
    if (!gs.io_valid || gs.io_key[0] != x_out || gs.io_key[1] != v_out || gs.io_key[2] != f_out) {
        if (gs.io_exec) cudaGraphExecDestroy(gs.io_exec);
        if (gs.io_graph) cudaGraphDestroy(gs.io_graph);
        gs.io_exec = nullptr;
        gs.io_graph = nullptr;
        gs.io_valid = false;
        if ((rc = capture_step(c, gs, key))) return rc;
    }
    if (c->async_steps == 0) {
        c->launches_at_sync = c->launches;
        cudaMemsetAsync(c->d_flags + 6, 0, sizeof(int), c->stream);
    }
    cudaError_t e = cudaGraphLaunch(gs.io_exec, c->stream);
    if (e != cudaSuccess) return check_cuda(c, e, "graph launch");
    c->graph_steps += 1;
    c->launches += gs.io_kernels;
    c->async_steps += 1;
    const long rec0 = c->overflow_recoveries;
    if ((rc = omdg_sync(c))) return rc;
    // a replay after a row overflow redid the steps whose outputs the graph wrote
    if (c->overflow_recoveries != rec0 && (x_out || v_out || f_out))
        return omdg_get_state(c, x_out, v_out, f_out, nullptr, nullptr);
    return OMDG_OK;
}

int omdg_replica_ledger(omdg_ctx* c, int nrep, double* kinetic, double* potential) {
    if (!c || nrep != c->nrep) return c ? set_error(c, OMDG_EINVAL, "nrep differs from the context's") : OMDG_EINVAL;
    cudaSetDevice(c->device);
    return replica_sums(c, kinetic, potential);
}

int omdg_ledger(omdg_ctx* c, double* kinetic, double* potential, double* base_potential, double* virial) {
    if (!c) return OMDG_EINVAL;
    if (kinetic) *kinetic = c->last_kin;
    if (potential) *potential = c->last_pot;
    if (base_potential) *base_potential = c->base_potential;
    if (virial) *virial = c->last_vir;
    return OMDG_OK;
}

int omdg_save_simulation(omdg_ctx* c, const char* path, int ncont, const omdg_container_desc* cont, const int* gid,
                         const int* flag, const double* aux, int nvar, const char* const* labels,
                         const char* const* values) {
    if (!c || !path || ncont <= 0 || !cont) return OMDG_EINVAL;
    if (c->n == 0) return set_error(c, OMDG_ESTATE, "no atoms");
    long total = 0;
    for (int k = 0; k < ncont; k++) total += cont[k].natoms;
    if (total != c->n) return set_error(c, OMDG_EINVAL, "the containers' atom counts do not sum to the atom count");
    cudaSetDevice(c->device);
    int rc = omdg_sync(c);
    if (rc) return rc;
    const int n = c->n;
    std::vector<double> x(3 * (size_t)n), v(3 * (size_t)n), f(3 * (size_t)n), pot(n), vir(n);
    if ((rc = omdg_get_state(c, x.data(), v.data(), f.data(), pot.data(), vir.data()))) return rc;
    if (c->resume) f = c->resume_f;  // not stepped since the load: the stored forces
    std::vector<unsigned> dflag;
    if (c->flags_used) {
        dflag.resize(n);
        if ((rc = io_get_flags(c, dflag.data()))) return rc;
    }
    omdg_sim_vars vars;
    std::memset(&vars, 0, sizeof(vars));
    vars.begin_time = c->begin_time;
    vars.step = (int)c->step;
    vars.pboundary = (c->box.periodic[0] ? 1 : 0) | (c->box.periodic[1] ? 2 : 0) | (c->box.periodic[2] ? 4 : 0);
    const double K = c->resume ? c->resume_vars[0] : c->last_kin, P = c->resume ? c->resume_vars[1] : c->last_pot;
    const double W = c->resume ? c->resume_vars[2] : c->last_vir, P0 = c->resume ? c->resume_vars[3] : c->base_potential;
    vars.kinetic = K;
    vars.potential = P;
    vars.virial = W;
    vars.base_potential = P0;
    vars.energy = K + P - P0;  // system.cpp:970
    vars.elapsed_time = c->elapsed;
    for (int d = 0; d < 3; d++) {
        vars.box[2 * d] = c->box.lo[d];
        vars.box[2 * d + 1] = c->box.hi[d];
        vars.box[6 + d] = c->box.L[d];
        vars.box[9 + d] = c->box.L[d] / 2.0;
    }
    std::vector<omdg_atom_record> recs(n);
    for (int i = 0; i < n; i++) {
        omdg_atom_record& a = recs[i];
        std::memset(&a, 0, sizeof(a));
        a.tid = c->caller_type[i];
        a.gid = gid ? gid[i] : 0;
        a.nid = i;
        a.flag = flag ? flag[i] : (dflag.empty() ? OMDG_FLAG_ACTIVE : (int)(dflag[i] & 1u));
        a.x = x[3 * i];
        a.y = x[3 * i + 1];
        a.z = x[3 * i + 2];
        a.vx = v[3 * i];
        a.vy = v[3 * i + 1];
        a.vz = v[3 * i + 2];
        a.fx = f[3 * i];
        a.fy = f[3 * i + 1];
        a.fz = f[3 * i + 2];
        a.potential = pot[i];
        a.virial = vir[i];
        if (aux)
            for (int q = 0; q < OMDG_AUXVAR; q++) a.aux[q] = aux[(size_t)OMDG_AUXVAR * i + q];
    }
    char err[256] = {0};
    rc = omdg_checkpoint_write(path, nullptr, &vars, nvar, labels, values, ncont, cont, recs.data(), err, sizeof(err));
    if (rc) return set_error(c, rc, err[0] ? err : "checkpoint write");
    return OMDG_OK;
}

int omdg_load_simulation(omdg_ctx* c, const char* path, int cap, omdg_container_desc* cont, int* ncont) {
    if (!c || !path) return OMDG_EINVAL;
    char err[256] = {0};
    int nc = 0, na = 0, nv = 0;
    int rc = omdg_checkpoint_info(path, &nc, &na, &nv, err, sizeof(err));
    if (rc) return set_error(c, rc, err);
    if (na <= 0) return set_error(c, OMDG_EFILE, "checkpoint holds no atoms");
    std::vector<omdg_container_desc> ds(nc);
    std::vector<omdg_atom_record> recs(na);
    omdg_sim_vars vars;
    if ((rc = omdg_checkpoint_read(path, &vars, nullptr, nc, ds.data(), na, recs.data(), nullptr, 0, err,
                                   sizeof(err))))
        return set_error(c, rc, err);
    // types are the atoms' tid; each type's mass and Z from the container
    // whose id it is, else from the first container holding such atoms
    int ntypes = 0;
    for (const omdg_atom_record& a : recs) {
        if (a.tid < 0 || a.tid >= MAX_TYPES) return set_error(c, OMDG_EFILE, "atom tid outside 0..7");
        ntypes = std::max(ntypes, a.tid + 1);
    }
    std::vector<double> mass(ntypes, -1.0), znum(ntypes, 0.0);
    for (const omdg_container_desc& d : ds)
        if (d.id >= 0 && d.id < ntypes && mass[d.id] < 0) {
            mass[d.id] = d.mass;
            znum[d.id] = d.z;
        }
    {
        size_t at = 0;
        for (const omdg_container_desc& d : ds) {
            for (int k = 0; k < d.natoms; k++, at++) {
                const int t = recs[at].tid;
                if (mass[t] < 0) {
                    mass[t] = d.mass;
                    znum[t] = d.z;
                }
            }
        }
    }
    for (int t = 0; t < ntypes; t++)
        if (!(mass[t] > 0)) mass[t] = 1.0;  // a type without atoms
    const double lo[3] = {vars.box[0], vars.box[2], vars.box[4]};
    const double hi[3] = {vars.box[1], vars.box[3], vars.box[5]};
    const int per[3] = {vars.pboundary & 1 ? 1 : 0, vars.pboundary & 2 ? 1 : 0, vars.pboundary & 4 ? 1 : 0};
    if ((rc = omdg_set_box(c, lo, hi, per))) return rc;
    std::vector<double> x(3 * (size_t)na), v(3 * (size_t)na), f(3 * (size_t)na);
    std::vector<int> type(na);
    for (int i = 0; i < na; i++) {
        const omdg_atom_record& a = recs[i];
        x[3 * i] = a.x;
        x[3 * i + 1] = a.y;
        x[3 * i + 2] = a.z;
        v[3 * i] = a.vx;
        v[3 * i + 1] = a.vy;
        v[3 * i + 2] = a.vz;
        f[3 * i] = a.fx;
        f[3 * i + 1] = a.fy;
        f[3 * i + 2] = a.fz;
        type[i] = a.tid;
    }
    if ((rc = omdg_set_atoms(c, na, x.data(), v.data(), type.data(), ntypes, mass.data(), znum.data()))) return rc;
    bool any_inactive = false;
    for (const omdg_atom_record& r : recs) any_inactive = any_inactive || !(r.flag & OMDG_FLAG_ACTIVE);
    if (any_inactive) {  // SetActive(false) atoms stay out of the integration and the list
        std::vector<int> act(na);
        for (int i = 0; i < na; i++) act[i] = recs[i].flag & OMDG_FLAG_ACTIVE;
        if ((rc = omdg_set_active(c, act.data()))) return rc;
    }
    c->resume = true;
    c->resume_step = vars.step;
    c->resume_vars[0] = vars.kinetic;
    c->resume_vars[1] = vars.potential;
    c->resume_vars[2] = vars.virial;
    c->resume_vars[3] = vars.base_potential;
    c->resume_f.swap(f);
    c->step = vars.step;
    c->elapsed = vars.elapsed_time;
    c->begin_time = vars.begin_time;
    if (ncont) *ncont = nc;
    if (cont)
        for (int k = 0; k < nc && k < cap; k++) cont[k] = ds[k];
    return OMDG_OK;
}

int omdg_ledger_history(omdg_ctx* c, double* kinetic, double* potential, int cap, int* rows) {
    if (!c || !rows) return OMDG_EINVAL;
    int m = std::min(cap, c->last_rows);
    for (int k = 0; k < m; k++) {
        if (kinetic) kinetic[k] = c->h_ledger[LEDGER_W * k];
        if (potential) potential[k] = c->h_ledger[LEDGER_W * k + 1];
    }
    *rows = m;
    return OMDG_OK;
}

int omdg_stats(omdg_ctx* c, long* rebuilds, long* launches) {
    if (!c) return OMDG_EINVAL;
    int graph_builds = 0;
    if (c->first_run_done) {
        int rc = step_state_graph_rebuilds(c, &graph_builds);
        if (rc) return rc;
    }
    // builds issued eagerly plus those the step graph's conditional node took
    // (capturing the graph issues one build that never ran)
    GraphState& gs = g_graphs[c];
    long eager = c->rebuilds - c->captured_builds;
    if (rebuilds) *rebuilds = eager + graph_builds;
    // kernels issued so far: eager launches plus graph replays
    if (launches) *launches = c->launches + c->graph_steps * c->graph_step_kernels + graph_builds * c->graph_body_kernels;
    (void)gs;
    return OMDG_OK;
}

int omdg_replica_builds(omdg_ctx* c, int* builds, int nrep) {
    if (!c || !builds) return OMDG_EINVAL;
    if (c->nrep == 0 || !c->d_rep_builds) return set_error(c, OMDG_ESTATE, "no replicas built");
    if (nrep != c->nrep) return set_error(c, OMDG_EINVAL, "nrep must be the replica count");
    cudaSetDevice(c->device);
    cudaError_t e = cudaMemcpyAsync(builds, c->d_rep_builds, sizeof(int) * nrep, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return check_cuda(c, e, "omdg_replica_builds");
}

int omdg_wide_centres(omdg_ctx* c, int* count) {
    if (!c || !count) return OMDG_EINVAL;
    *count = 0;
    if (!c->ters_wide) return OMDG_OK;
    int v = 0;
    cudaError_t e = cudaMemcpyAsync(&v, c->ters_wide, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return check_cuda(c, e, "omdg_wide_centres");
    *count = v;
    return OMDG_OK;
}

int omdg_tile_counts(omdg_ctx* c, int* tiles, int* staged) {
    if (!c || !tiles || !staged) return OMDG_EINVAL;
    *tiles = 0;
    *staged = 0;
    if (!c->tile_valid || !c->tile_nst || c->tile_count == 0) return OMDG_OK;
    std::vector<int> nst(c->tile_count);
    cudaError_t e = cudaMemcpyAsync(nst.data(), c->tile_nst, sizeof(int) * nst.size(), cudaMemcpyDeviceToHost,
                                    c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return check_cuda(c, e, "omdg_tile_counts");
    *tiles = c->tile_count;
    for (int v : nst) *staged += v <= c->tile_cap ? 1 : 0;
    return OMDG_OK;
}

int omdg_set_profiling(omdg_ctx* c, int on) {
    if (!c) return OMDG_EINVAL;
    c->profiling = on != 0;
    if (on) c->timers.clear();
    return OMDG_OK;
}

int omdg_kernel_times(omdg_ctx* c, char* name_buf, int name_cap, double* ms, long* calls, int cap, int* nkern) {
    if (!c || !nkern) return OMDG_EINVAL;
    prof_collect(c);
    std::string names;
    int m = std::min(cap, (int)c->timers.size());
    for (int k = 0; k < m; k++) {
        if (k) names += ";";
        names += c->timers[k].name;
        if (ms) ms[k] = c->timers[k].ms;
        if (calls) calls[k] = c->timers[k].calls;
    }
    if (name_buf && name_cap > 0) {
        std::strncpy(name_buf, names.c_str(), name_cap - 1);
        name_buf[name_cap - 1] = 0;
    }
    *nkern = m;
    return OMDG_OK;
}

}  // extern "C"

// ------------------------------------------------------------- launch shapes
namespace omdg {
static int* launch_knob(Context* c, const std::string& k) {
    if (k == "eam_block") return &c->eam_block;
    if (k == "eam_lanes") return &c->eam_lanes;
    if (k == "eam_stage") return &c->eam_stage;
    if (k == "eam_ctas_per_sm") return &c->eam_ctas_per_sm;
    if (k == "pair_block") return &c->pair_block;
    if (k == "pair_lanes") return &c->pair_lanes;
    if (k == "tb_block") return &c->tb_block;
    if (k == "tb_lanes") return &c->tb_lanes;
    if (k == "tb_persistent") return &c->tb_persistent;
    if (k == "fuse_kick") return &c->fuse_kick_on;
    if (k == "nbr_hshift") return &c->nbr_hshift;
    if (k == "build_lanes") return &c->build_lanes;
    if (k == "io_blocks") return &c->io_blocks;
    if (k == "nbr_capacity") return &c->nbr_capacity;
    if (k == "eam_tile") return &c->eam_tile;
    if (k == "nn_fused") return &c->nn_fused;
    if (k == "tile_x") return &c->tile_dim[0];
    if (k == "tile_y") return &c->tile_dim[1];
    if (k == "tile_z") return &c->tile_dim[2];
    if (k == "tile_cap") return &c->tile_cap;
    return nullptr;
}

static bool valid_knob(const std::string& k, int v) {
    auto pow2 = [](int x) { return x > 0 && (x & (x - 1)) == 0; };
    if (k == "eam_lanes" || k == "pair_lanes" || k == "tb_lanes") return pow2(v) && v <= 32;
    if (k == "eam_block" || k == "pair_block" || k == "tb_block") return v >= 32 && v <= 1024 && v % 32 == 0;
    if (k == "nbr_hshift") return v >= 0 && v <= 5;
    if (k == "eam_ctas_per_sm") return v >= 1 && v <= 32;
    if (k == "eam_stage" || k == "tb_persistent" || k == "fuse_kick") return v == 0 || v == 1;
    if (k == "build_lanes") return v == 0 || v == 1 || v == 4 || v == 8;
    if (k == "io_blocks") return v >= 1 && v <= 65535;
    if (k == "nbr_capacity") return v >= 0 && v <= 4096;
    if (k == "eam_tile" || k == "nn_fused") return v == 0 || v == 1;
    if (k == "tile_x" || k == "tile_y" || k == "tile_z") return v >= 1 && v <= 4;
    if (k == "tile_cap") return v >= 64 && v <= 5000;
    return false;
}

// Time one force evaluation (best of reps) with events on the context stream.
static int time_forces(Context* c, int reps, double& best) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    best = 1e30;
    int rc = forces_compute(c);  // warm
    for (int r = 0; r < reps && !rc; r++) {
        cudaEventRecord(a, c->stream);
        rc = forces_compute(c);
        cudaEventRecord(b, c->stream);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (ms < best) best = ms;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (!rc) rc = check_status(c);
    return rc;
}
// Best of `reps` list builds (binning, permutation, list) in milliseconds.
static int time_build(Context* c, int reps, double& best) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    best = 1e30;
    int rc = nlist_build(c);  // warm
    for (int r = 0; r < reps && !rc; r++) {
        cudaEventRecord(a, c->stream);
        rc = nlist_build(c);
        cudaEventRecord(b, c->stream);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (ms < best) best = ms;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (!rc) rc = check_status(c);
    return rc;
}
}  // namespace omdg

extern "C" {

int omdg_set_launch(omdg_ctx* c, const char* key, int value) {
    if (!c || !key) return OMDG_EINVAL;
    std::string k(key);
    int* p = launch_knob(c, k);
    if (!p) return set_error(c, OMDG_EINVAL, "unknown launch key " + k);
    if (!valid_knob(k, value)) return set_error(c, OMDG_EINVAL, "invalid value for " + k);
    if (*p == value) return OMDG_OK;
    *p = value;
    // the build writes tile slots for the tile shape and capacity it sees
    if (k == "build_lanes" || k == "eam_tile" || k == "tile_x" || k == "tile_y" || k == "tile_z" ||
        k == "tile_cap")
        c->list_valid = false;
    if (k == "nbr_capacity") {  // applies at the next first build
        c->list_valid = false;
        c->maxnb = 0;
    }
    if (k == "nbr_hshift") {
        // the list layout changes: reallocate and rebuild before the next use
        int m = c->maxnb;
        c->maxnb = 0;
        cudaFree(c->nbr);
        cudaFree(c->rev);
        cudaFree(c->slot_buf);
        c->nbr = nullptr;
        c->rev = nullptr;
        c->slot_buf = nullptr;
        if (m > 0) {
            int rc = nlist_reserve(c, m);
            if (rc) return rc;
        }
        c->list_valid = false;
    }
    invalidate_graph(c);
    return OMDG_OK;
}

int omdg_get_launch(omdg_ctx* c, const char* key, int* value) {
    if (!c || !key || !value) return OMDG_EINVAL;
    int* p = launch_knob(c, key);
    if (!p) return set_error(c, OMDG_EINVAL, std::string("unknown launch key ") + key);
    *value = *p;
    return OMDG_OK;
}

int omdg_autotune(omdg_ctx* c, int reps, double* best_ms) {
    if (!c || reps < 1) return OMDG_EINVAL;
    if (c->n == 0 || c->pots.empty()) return set_error(c, OMDG_ESTATE, "autotune needs atoms and force kernels");
    cudaSetDevice(c->device);
    bool eam = false, pair = false, tb = false;
    for (auto& p : c->pots) {
        eam |= p.kind == POT_EAM;
        pair |= (p.kind == POT_PAIR && !p.fp64) || p.kind == POT_ZBL;
        tb |= p.kind == POT_SW || p.kind == POT_TERSOFF;
    }
    struct Cand {
        int lanes, block, stage, tile;
    };
    std::vector<Cand> cands;
    const int tile_on = c->eam_tile;
    if (eam) {
        // the tiled passes (where they apply), then the gather passes
        if (tile_on && tiles_apply(c))
            for (int lanes : {4, 8, 16}) cands.push_back(Cand{lanes, 256, 0, 1});
        for (int lanes : {4, 8, 16})
            for (int block : {128, 256})
                for (int stage : {0, 1}) cands.push_back(Cand{lanes, block, stage, 0});
    } else if (pair) {
        for (int lanes : {2, 4, 8, 16})
            for (int block : {128, 256}) cands.push_back(Cand{lanes, block, 0, tile_on});
    } else if (tb) {
        // lanes: the neighbour slice height the rows are laid out in (the
        // three-body kernels run one thread per centre in 128-thread blocks);
        // stage: the Tersoff register pass as one resident grid (persistent)
        for (int lanes : {1, 2, 4})
            for (int stage : {0, 1}) cands.push_back(Cand{lanes, 128, stage, tile_on});
    }
    int rc = OMDG_OK;
    // list build: cell-CTA, 8 or 4 lanes per atom, or one thread per atom
    // (cells holding few atoms leave most of a cell CTA idle)
    if (!c->list_valid && (rc = build_list(c))) return rc;
    {
        int best_bl = c->build_lanes;
        double tbest = 1e30;
        for (int bl : {0, 8, 4, 1}) {
            c->build_lanes = bl;
            double t;
            if ((rc = time_build(c, reps, t))) return rc;
            if (t < tbest) {
                tbest = t;
                best_bl = bl;
            }
        }
        c->build_lanes = best_bl;
        if ((rc = build_list(c))) return rc;
        if ((rc = threebody_prepare(c))) return rc;
    }
    if (cands.empty()) {
        invalidate_graph(c);
        if (best_ms) return time_forces(c, reps, *best_ms);
        return OMDG_OK;
    }
    double best = 1e30;
    Cand win = cands[0];
    for (auto& cd : cands) {
        int hs = 0;
        while ((1 << hs) * cd.lanes < 32 && hs < 5) hs++;
        if (eam) {
            c->eam_lanes = cd.lanes;
            c->eam_block = cd.block;
            c->eam_stage = cd.stage;
            c->eam_ctas_per_sm = cd.block >= 512 ? 2 : 4;
            if (c->eam_tile != cd.tile) {
                c->eam_tile = cd.tile;
                c->list_valid = false;
            }
        } else if (pair) {
            c->pair_lanes = cd.lanes;
            c->pair_block = cd.block;
        } else {
            c->tb_lanes = cd.lanes;
            c->tb_block = cd.block;
            c->tb_persistent = cd.stage;
        }
        if ((rc = omdg_set_launch(c, "nbr_hshift", hs))) return rc;
        if (!c->list_valid && (rc = build_list(c))) return rc;
        if ((rc = threebody_prepare(c))) return rc;
        double t;
        if ((rc = time_forces(c, reps, t))) return rc;
        if (t < best) {
            best = t;
            win = cd;
        }
    }
    int hs = 0;
    while ((1 << hs) * win.lanes < 32 && hs < 5) hs++;
    if (eam) {
        c->eam_lanes = win.lanes;
        c->eam_block = win.block;
        c->eam_stage = win.stage;
        c->eam_ctas_per_sm = win.block >= 512 ? 2 : 4;
        if (c->eam_tile != win.tile) {
            c->eam_tile = win.tile;
            c->list_valid = false;
        }
    } else if (pair) {
        c->pair_lanes = win.lanes;
        c->pair_block = win.block;
    } else {
        c->tb_lanes = win.lanes;
        c->tb_block = win.block;
        c->tb_persistent = win.stage;
    }
    if ((rc = omdg_set_launch(c, "nbr_hshift", hs))) return rc;
    if (!c->list_valid && (rc = build_list(c))) return rc;
    if ((rc = threebody_prepare(c))) return rc;
    invalidate_graph(c);
    if (best_ms) *best_ms = best;
    return OMDG_OK;
}

}  // extern "C"
