// Internal types of libomdg: device-resident state of one simulation box,
// the mixed-precision position pack, spline tables and kernel parameter
// blocks.  Nothing here crosses the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/omdg.h"

namespace omdg {

// ------------------------------------------------------------ error words
// Device kernels never trap: they OR one of these bits into the context's
// device status word; the host maps it to an OMDG_E* code after the launch.
enum : unsigned {
    ERR_TABLE_RANGE = 1u,  // TableReader would die (treader.cpp:199-218)
    ERR_OVERLAP = 2u,      // r^2 < OMD_PROXIMITY (gadget.cpp:149)
    ERR_NBR_OVERFLOW = 4u, // per-atom neighbour capacity exceeded (host grows and rebuilds)
    ERR_NONFINITE = 8u,    // NaN/Inf force or position
    ERR_CELL = 16u,        // atom outside the cell grid of a free axis (host re-grids)
    ERR_TIMEOUT = 32u,     // a bounded device wait (mbarrier) expired
};

// The status block: word 0 the bits above; then the first overlapping pair
// (sorted indices) and the first value read outside a table with its table
// (DevTable::src); ~0 where nothing was recorded.
enum : int { ST_WORDS = 8, ST_OV_I = 1, ST_OV_J = 2, ST_RANGE_V = 3, ST_RANGE_SRC = 4 };

constexpr int CODE_SHIFT = 26;                // nbr entry = j | code << 26
constexpr int INDEX_MASK = (1 << CODE_SHIFT) - 1;
constexpr int MAX_ATOMS = INDEX_MASK;         // 67,108,863
constexpr int MAX_TYPES = 8;                  // MAXATOMTYPE (config.h:25)
constexpr double OMD_PROXIMITY = 1e-6;        // config.h:31

// ------------------------------------------------------------ spline table
// One TableReader (treader.h:28-61): the coefficients are computed on the
// host in FP64 exactly as the reference does; the device holds them as FP32
// (a,b,c,d) per knot and, for FP64 kernels, as FP64.
struct HostTable {
    std::string file, name;
    int n = 0;
    double dr = 0, off = 0;
    bool rmult = false, allow_lo = false, allow_hi = false;
    double out_lo = 0, out_hi = 0;
    double constant = 0;          // the section's 'Constant' parameter (TTM tables), if any
    bool has_constant = false;
    std::vector<double> a, b, c, d;
    double max_range() const { return off + (double)(n - 1) * dr; }
};
int table_load(const std::string& file, const std::string& name, HostTable& t, std::string& err);
void table_coef(HostTable& t);
// Reference evaluation (FP64) used by host-side checks.
bool table_read(const HostTable& t, double r, double& val, double& dval);
// Start of the table's negligible tail: the first knot from which every
// segment stays within tol in value and in slope (per r for RMULT tables);
// max_range() when there is none.
double table_negligible_from(const HostTable& t, double tol);

struct DevTable {
    const float4* coef;    // (a, b, c, d) per knot
    const double4_32a* coef64; // FP64 copy (FP64 kernels only, may be null)
    float off, dr, inv_dr;
    double off64, dr64;
    int n;
    int rmult;
    int allow_lo, allow_hi;
    float out_lo, out_hi;
    float rc;      // max_range as float
    double rc64;   // max_range
    int src;       // potential index * 4 + section (0 PAIR/phi, 1 EDENS, 2 EMBED): names the table in errors
};

// ------------------------------------------------------------ box geometry
// Positions are kept in FP64 (x, y, z).  Force kernels read a 32-byte pack
// per atom: hi = float(X), lo = float(X - hi) with X = (x - org) + P, where
// P is a power of two at least 4x the extent of the box.  All X then share
// one float binade [P, 2P), so hi_i - hi_j is exact and subtracting the
// split periodic length (Lh + Ll) keeps the relative vector accurate to the
// final FP32 rounding (see pair_delta()).
struct BoxGeom {
    double lo[3], hi[3], L[3];
    int periodic[3];
    double org[3];  // origin of the pack frame (box lo, or free-axis minimum minus margin)
    double P[3];    // pack offset (power of two)
    float Lh[3], Ll[3];
    // linked cells (rebuilt with the list)
    int nc[3];
    double cell_org[3], cell_h[3];
};

struct __align__(32) PosPack {
    float4 hi;  // hx, hy, hz, type (bit pattern)
    float4 lo;  // lx, ly, lz, per-atom auxiliary (EAM: F'(rho), written by the density pass)
};

// ------------------------------------------------------------ potentials
enum PotKind { POT_EAM = 1, POT_PAIR = 2, POT_SW = 3, POT_TERSOFF = 4, POT_ZBL = 5, POT_NN = 6 };

struct NNState;  // neural surrogate (nn_potential.cu)
struct TTMCtx;   // local thermodynamics and the two-temperature model (ttm.cu)

struct SWParams {
    double eps, A, B, p, q, sigma, a, lambda, gamma, icos0;
    int usezbl;
    double sx0, sx1, sa0, sa1, sa2, sa3;
    // derived constants (sw.cpp:65-91)
    double rc, c1, c2, c3, c4, c5, c6, c7, c8, c9, c10, zc, ze0, ze1, ze2, ze3;
};

struct TersoffParams {
    double A, B, lambda1, lambda2, lambda3, beta, n, c, d, h, R, D;
};

struct ZBLParams {
    double z1, z2, rc, width;
    double zc, ze0, ze1, ze2, ze3;
};

struct Potential {
    PotKind kind;
    int ta, tb;
    bool fp64 = false;
    HostTable t0, t1, t2;  // EAM: PAIR, EDENS, EMBED; PAIR: phi
    SWParams sw{};
    TersoffParams ters{};
    ZBLParams zbl{};
    double rc = 0;         // CutRadius as the reference sets it
    double rc_list = 0;    // the radius this kernel needs in the neighbour list (<= rc)
    NNState* nn = nullptr; // POT_NN: model, device network and per-atom buffers
    bool fallback_only = false;  // evaluated only for the atoms a POT_NN hands over
    // device copies
    float4* d_coef[3] = {nullptr, nullptr, nullptr};
    float4* d_coef2 = nullptr;  // EAM: PAIR and EDENS knots interleaved
    double4_32a* d_coef64[3] = {nullptr, nullptr, nullptr};
    DevTable dt[3]{};
};

// ------------------------------------------------------------ kernel timing
struct KernelTimer {
    std::string name;
    double ms = 0;
    long calls = 0;
};

// ------------------------------------------------------------ context
struct Context {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;

    // atoms
    int n = 0, cap = 0, ntypes = 0;
    double mass[MAX_TYPES] = {0}, zat[MAX_TYPES] = {0};
    BoxGeom box{};
    bool have_box = false;

    // device per-atom arrays (sorted order)
    double *x = nullptr, *y = nullptr, *z = nullptr;
    double *vx = nullptr, *vy = nullptr, *vz = nullptr;
    float *fx = nullptr, *fy = nullptr, *fz = nullptr;
    float *pe = nullptr, *vir = nullptr;
    PosPack* pack = nullptr;
    float4* xref = nullptr;   // pack-frame position at the last build (FP32)
    float4* loc = nullptr;    // position relative to its cell's corner at the last build (FP32); w = the type
    unsigned* nbmask = nullptr;  // per atom: bit t set when its row holds an atom of type t (cell-local build)
    bool nbmask_valid = false;   // the last build wrote nbmask
    int* type = nullptr;
    int* id = nullptr;        // caller index of sorted atom
    int* inv = nullptr;       // sorted index of caller atom
    float *fp = nullptr, *femb = nullptr;  // EAM F'(rho), F(rho)
    // sort scratch
    int *cell = nullptr, *perm = nullptr;
    int *cell_count = nullptr, *cell_start = nullptr, *cell_fill = nullptr;
    int* cell_tile_sum = nullptr;  // scan tile totals / offsets
    // replica mode (omdg_set_replicas): independent boxes in one atom array,
    // each with its own cell grid and periodic lengths; the counting sort
    // keeps every replica's atoms in its index range
    int nrep = 0;
    std::vector<int> rep_start;          // nrep + 1
    std::vector<double> rep_lo, rep_hi;  // nrep x 3
    int rep_periodic[3] = {1, 1, 0};
    int rep_cells = 0;                   // cells over all replicas
    double rep_hmax = 0.0;               // largest replica cell size (list screening band)
    int* d_rep_of = nullptr;             // replica of each atom (index order)
    int rep_of_cap = 0;
    void* d_rep_geom = nullptr;          // RepGeom[nrep] (nlist.cu)
    void* d_rep_shift = nullptr;         // ShiftF[nrep]: periodic lengths for pair_delta
    double* d_rep_sums = nullptr;        // per-replica ledger sums
    TTMCtx* ttm = nullptr;               // ThermoDetector / TTM_Homogen state (null: off)
    int* d_rep_start = nullptr;          // nrep + 1
    int* d_rep_flag = nullptr;           // per replica: an atom moved past skin/2 (rebuild it)
    int* d_rep_builds = nullptr;         // per replica: list builds so far
    int* d_cell_rep = nullptr;           // replica of each cell (rep_cells)
    bool build_partial = false;          // the build being issued rebuilds only the flagged replicas
    bool fuse_kick = false;              // the forces being issued are a step's: the kick may join them
    bool kick_fused = false;             // the last force launch did the step's second half-kick
    int ncell_cap = 0;
    int* scan_partials = nullptr;
    double* stage_d = nullptr;   // permutation staging: 6 FP64 arrays x cap
    int* stage_i = nullptr;      // permutation staging: 2 int arrays x cap
    unsigned* aflag = nullptr;   // per atom: bit 0 FLAG_ACTIVE (base.h:230), bits 8..15 group membership
    bool flags_used = false;     // an atom was deactivated or a modify acts on groups
    double* extra = nullptr;     // optional per-atom FP64 state carried through sorts
    double* stage_extra = nullptr;
    int extra_n = 0;
    int* cell_sorted = nullptr;
    double* f64 = nullptr;       // FP64 forces (3n) + FP64 per-atom energy (n), FP64 kernels only
    bool use_f64 = false;
    double* d_mass = nullptr;    // mass per type (device)
    double* d_io = nullptr;      // caller-order transfer staging
    int host_ptr_ok = -1;        // registered host memory is addressable by kernels at its own address (-1: not asked)
    size_t io_cap = 0;
    long async_steps = 0;        // steps enqueued since the last omdg_sync
    long launches_at_sync = 0, last_launches = 0;
    long graph_steps = 0;        // graph replays issued
    long graph_step_kernels = 0; // kernels per replay (outside the rebuild body)
    long graph_body_kernels = 0; // kernels in the rebuild body
    long captured_builds = 0;    // list builds issued while capturing (never ran)
    void* d_state = nullptr;     // StepState (integrate.cu)

    // neighbour list: nbr[s*n + i] = j | code << 26, count in nnb[i]
    int* nbr = nullptr;
    int* nnb = nullptr;
    // list overflow inside queued steps: every in-step rebuild first copies the
    // state it reorders (positions, velocities, types, ids, flags) and the step
    // state here; a rebuild that overflows halts later rebuilds, and omdg_sync
    // restores this copy, grows the list and replays from that rebuild
    double* snap_d = nullptr;   // 6 x cap: x, y, z, vx, vy, vz
    int* snap_i = nullptr;      // 3 x cap: type, id, flags
    void* snap_state = nullptr; // StepState
    bool build_in_step = false; // the build being issued belongs to a step (snapshot and halt)
    int nbr_capacity = 0;       // launch key: the first build's row capacity (0: from the density)
    long overflow_recoveries = 0;  // queued steps replayed after a row overflow
    int* rev = nullptr;       // slot of i in row j (three-body kernels)
    float4* slot_buf = nullptr;  // per-slot force contributions (three-body kernels)
    int* ters_wide = nullptr;    // Tersoff centres past the register path: [0] count, then their indices
    int maxnb = 0;
    long nbr_bytes = 0;
    double skin = 0.3;
    int rebuild_every = 0;
    bool list_valid = false;
    bool need_rev = false;
    long rebuilds = 0;
    int steps_since_build = 0;

    // launch shapes (defaults; the tuner may change them)
    int num_sms = 152;
    int io_blocks = 152;       // blocks of the download kernels beside a step (omdg_step_io)
    int build_lanes = 0;       // list build: 1, 4, 8 threads per atom; 0 cell-centric (shared memory)
                               // on grids of >= 8 atoms per cell, else one thread per atom
    int nbr_hshift = 3;        // sliced-ELL slice height H = 2^hshift
    int eam_block = 256;
    int eam_lanes = 4;         // threads per atom
    int eam_stage = 0;         // 1: stage spline knots in shared memory
    double eam_stage_frac = 0.35;
    int eam_ctas_per_sm = 1;
    int pair_block = 256;
    int pair_lanes = 8;
    int tb_block = 128;        // three-body kernels
    int tb_lanes = 1;
    int tb_persistent = 0;     // Tersoff register pass: one resident grid striding over the flattened atoms
    int nn_fused = 0;          // the surrogate's descriptors computed inside its tensor-core network kernel (opt-in:
                               // with four 128-thread CTAs per SM the descriptor work runs slower there)
    int fuse_kick_on = 0;      // a step's second half-kick in the force kernel's epilogue where it can go (opt-in:
                               // with 4 lanes per atom its FP64 work issues at a quarter of the lanes)

    // EAM cell tiles (eam_fast.cu): a tile is a block of tile_dim cells; one
    // CTA stages the packs of the tile's cells and their one-cell halo in
    // shared memory, and the list build also writes every row as 16-bit
    // slots into that staged halo.  A tile whose halo holds more than
    // tile_cap atoms takes the gather path.
    int eam_tile = 0;                 // launch key: the tiled EAM passes where they apply
    int tile_dim[3] = {2, 2, 2};      // launch keys tile_x, tile_y, tile_z: cells per tile
    int tile_cap = 1536;              // launch key: staged atoms per tile (32 bytes of shared memory each)
    bool tile_want = false;           // this context's builds write tile slots (tile_prepare)
    bool tile_valid = false;          // the last build wrote them
    int tile_nt[3] = {0, 0, 0};       // tiles per axis
    int tile_count = 0, tile_hc = 0;  // tiles; halo cells per tile
    int tile_alloc = 0;               // tiles x halo cells allocated
    int tile_stride = 0;              // u16 slots per row of tslot (maxnb rounded up to 8)
    size_t tslot_alloc = 0;           // u16 slots allocated
    unsigned short* tile_sb = nullptr;  // per tile and halo cell: its first staged slot
    int* tile_nst = nullptr;            // per tile: staged atoms
    float4* tile_org = nullptr;         // per tile: its lower corner in the pack frame (FP32)
    unsigned short* tslot = nullptr;    // per atom row: each entry's slot in its tile's staged halo

    // potentials
    std::vector<Potential> pots;
    double rc_max = 0;          // the list radius: largest kernel radius (and the detector's cutoff)
    double rc_ref = 0;          // the reference's CutRadius: largest over the kernels (integrator.cpp:108-113)
    bool table_full_range = false;  // pair tables' negligible tails stay in the list radius (compat)

    // integrator
    double dt = 0.001;
    bool first_run_done = false;
    bool reference_first_step = true;
    long step = 0;
    double thermo_T = 0, thermo_tau = 0;
    // modifies of the impact runs (test/si-impact/main.cpp:73-76)
    struct PostOp {
        int kind;       // 1 ForceDamper, 2 CoordClamp
        int group;      // -1: every atom
        double factor;  // ForceDamper factor
        int axes;       // CoordClamp mask: 1 x, 2 y, 4 z
    };
    std::vector<PostOp> post_ops;   // PostForce, in the order added
    bool range_on = false;          // RangeLimiter
    int range_group = -1;
    double range_border = 0;
    bool src_on = false;            // EnergySource pulse: delta per step, window [start, start + width)
    double src_delta = 0, src_start = 0, src_width = 0;
    int dyn_update = 0;             // DynamicTimeStep (update period; 0: off)
    double dyn_maxpath = 0, dyn_maxdt = 0;
    bool first_measure = false;     // FirstRun's measurement (DynamicTimeStep at Step 0)
    bool thermo_count_ghosts = false;  // reference compatibility (omdg_set_compat)
    bool lambda_pending = false;       // a thermostat factor waits in the step state

    // device status and reductions
    unsigned* d_status = nullptr;   // error bits
    int* d_flags = nullptr;         // [0] rebuild request, [1] row length needed, [2] ghost count,
                                    // [3] largest cell-local coordinate of the last build (float bits),
                                    // [4] blocks done in the current kick (reset by the last block)
    double* d_red = nullptr;        // block partials
    int red_cap = 0;
    double* d_ledger = nullptr;     // per step LEDGER_W doubles: kinetic, potential, virial, lambda,
                                    // Step, ElapsedTime (both before the step's increment), TimeStep, 0,
                                    // and with the thermo detector its system temperature, average
                                    // local temperature, system pressure, average local pressure
    int ledger_cap = 0;
    double* h_ledger = nullptr;     // pinned copy
    void* h_sync = nullptr;         // pinned staging of the status word and the step state
    double base_potential = 0;
    double last_kin = 0, last_pot = 0, last_vir = 0;
    double elapsed = 0;                 // ElapsedTime: the steps' dt summed in order (system.cpp:979)
    long long begin_time = 0;           // SimBeginTime: wall clock (time_t) of the first step or the checkpoint
    std::vector<int> caller_type;       // atom types in caller order (checkpoint records)
    // a run resumed from a checkpoint: applied at the first step instead of FirstRun
    bool resume = false;
    long long resume_step = 0;
    double resume_vars[4] = {0, 0, 0, 0};  // kinetic, potential, virial, base potential
    std::vector<double> resume_f;          // stored forces, caller order
    int last_rows = 0;
    long launches = 0;

    // profiling
    bool profiling = false;
    std::vector<KernelTimer> timers;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
    std::vector<cudaEvent_t> event_pool;
};

// ------------------------------------------------------------ host helpers
int set_error(Context* c, int code, const std::string& msg);
int check_cuda(Context* c, cudaError_t e, const char* what);
int check_status(Context* c);  // reads and clears the device status word

// profiling brackets (no-ops unless profiling)
void prof_begin(Context* c, const char* name);
void prof_end(Context* c);
void prof_collect(Context* c);

// neighbour list (nlist.cu)
int nlist_build(Context* c);
void nlist_prepare_geometry(Context* c);
int nlist_reserve(Context* c, int maxnb);
size_t nlist_slots(const Context* c, int maxnb);
// EAM cell tiles: decide whether the builds write tile slots and size the
// tile tables (host, outside any capture); the slot rows follow maxnb
bool tiles_apply(const Context* c);
int tile_prepare(Context* c);
int tile_reserve_slots(Context* c);
void tile_release(Context* c);

// forces (eam.cu, pair.cu, threebody.cu)
int forces_compute(Context* c);
int eam_launch(Context* c, Potential& p, bool first);
int pair_launch(Context* c, Potential& p, bool first);
int sw_launch(Context* c, Potential& p, bool first);
int tersoff_launch(Context* c, Potential& p, bool first);
int zbl_launch(Context* c, Potential& p, bool first);

// integrator (integrate.cu)
int integrate_kick_drift(Context* c, int step_index);
int integrate_kick(Context* c, int step_index);
int integrate_pack(Context* c);
int measure_energies(Context* c, int row);
int zero_forces(Context* c);
// caller-order x and/or v rows (device-addressable): sorted arrays; for x also the pack and displacement check
int upload_state(Context* c, const double* in_x, const double* in_v);
int resolve_thermostat(Context* c);
int gather_slots(Context* c, bool zero_virial);
// mask: only centres i with mask[i] != 0; mask_count: device count of them
// (0: the pass does no work)
int tersoff_centre(Context* c, Potential& pot, bool first, const int* mask, const int* mask_count = nullptr);
int nn_launch(Context* c, Potential& pot, bool first);
int replica_prepare(Context* c);  // per-replica cell grids and shifts (host, before a build)
int thermo_detect(Context* c, bool after_step);  // local thermodynamics (ttm.cu); after_step: the step advanced the ledger row
const int* step_state_row(Context* c);           // device address of the ledger row counter (integrate.cu)
int* step_state_halted(Context* c);              // device address of the step state's halt flag
size_t step_state_bytes();
double thermo_ercut(const Context* c);  // the detector's cutoff (its own, else the largest force cutoff); -1: off
int ttm_pre(Context* c);          // electron temperature step and rescaling before a step
void ttm_release(Context* c);
bool ttm_active(const Context* c);
int replica_sums(Context* c, double* kinetic, double* potential);  // per-replica ledger (synchronous)
void update_rc(Context* c);         // largest cutoff; drops the list and the step graph
void invalidate_graph(Context* c);
void nn_release(Potential& pot);
int drop_thermostat_factor(Context* c);
int step_state_graph_rebuilds(Context* c, int* nrebuild);

// caller-order transfers (io.cu); asynchronous on the context stream.  Pinned
// or registered host arrays are read and written by the kernels directly;
// other host memory goes through the device staging buffer and one copy.
const double* host_view(Context* c, const double* p, size_t count);
int io_rows_to_host(Context* c, cudaStream_t s, double* x, double* v, double* f);  // pinned outputs, one kernel
int io_get_state(Context* c, double* x, double* v, double* f, double* pot, double* vir);
int io_set_state(Context* c, const double* x, const double* v);
int io_set_forces(Context* c, const double* f);
int energy_source(Context* c);  // EnergySource's PreIntegration scaling (integrate.cu)
int post_force_modifies(Context* c);  // ForceDamper / CoordClamp after the forces (integrate.cu)
int io_set_flags(Context* c, const unsigned* flags, unsigned keep_mask);  // caller order; bits in keep_mask survive
int io_get_flags(Context* c, unsigned* flags);

constexpr int LEDGER_W = 12;  // doubles per ledger row
constexpr int RED_BLOCK = 256;  // threads of the kick kernel's blocks (one 32-byte partial each)

// Atom group g as its flag bit (bits 8..15); -1: every atom.
inline unsigned group_bits(int g) { return g < 0 ? ~0u : (1u << (8 + g)); }

// run-time poll limit of the tensor-core kernels' mbarrier waits (waits.cu)
int tc_wait_polls();

// grid sizing
inline int grid_for(int n, int block) { return (n + block - 1) / block; }

}  // namespace omdg

// The opaque handle of the C ABI is the context itself.
struct omdg_ctx : public omdg::Context {};
