// Linked-cell binning by counting sort and the Verlet-list build
// (replaces VerletList::Update, VerletList.cpp:126-199, and
// VerletListFull::Update, VerletListFull.cpp:138-230, together with the
// periodic ghost images of comhandler.cpp:288-377).
//
// Rebuild pipeline, all on the context stream:
//   1 cell_assign   wrap periodic owners into the box (systemgrid.cpp:129-151),
//                   cell of every atom, per-cell counts
//   2 scan          exclusive scan of the counts -> cell starts
//   3 scatter       atom -> slot in its cell
//   4 cell_sort     sort each cell's slots by previous index (deterministic order)
//   5 permute       reorder every per-atom array into cell order
//   6 pack          FP32 hi/lo position packs + displacement reference
//   7 build         full list, slot-major nbr[s*n+i]; FP32 screen, FP64 tie-break
//   8 reverse       (three-body kernels) slot of i in each neighbour's row
#include <algorithm>
#include <cmath>

#include <climits>

#include "device_common.cuh"

namespace omdg {

struct CellGeom {
    int nc[3];
    double org[3], h[3], inv_h[3];
    int periodic[3];
    double lo[3], L[3];
};

static CellGeom cell_geom(const Context* c) {
    CellGeom g;
    for (int d = 0; d < 3; d++) {
        g.nc[d] = c->box.nc[d];
        g.org[d] = c->box.cell_org[d];
        g.h[d] = c->box.cell_h[d];
        g.inv_h[d] = 1.0 / c->box.cell_h[d];
        g.periodic[d] = c->box.periodic[d];
        g.lo[d] = c->box.lo[d];
        g.L[d] = c->box.L[d];
    }
    return g;
}

// systemgrid.cpp:132-138: an atom is owned iff floor((x - x0) / lx) == 0,
// else it becomes the image x -/+ lx (comhandler.cpp:427-432).  Out of line:
// only atoms that crossed a face get here.
__device__ __noinline__ double wrap_crossed(double p, double lo, double L) {
    const int u = (int)floor(__ddiv_rn(__dsub_rn(p, lo), L));
    if (u < 0) return __dadd_rn(p, L);
    if (u >= 1) return __dadd_rn(p, -L);
    return p;
}

// Cell coordinate along one axis, wrapping p on a periodic axis first.  For
// a = p - x0 and lx positive, floor(a / lx) == 0 is 0 <= a < lx (a < lx gives
// fl(a / lx) < 1, a >= lx gives fl(a / lx) >= 1), tested on the bit patterns
// (non-negative doubles order as integers; NaN fails).  The cell is
// floor(a / h) by the reciprocal (the FP64 pipe divides slowly); cells are
// at least Rv (1 + 1e-12) wide, so a few ulps of misplacement at a face
// never separates a pair within Rv by more than one cell.  Periodic axes
// have their cell origin at x0.
__device__ __forceinline__ int axis_cell_of(double& p, int periodic, double lo, double L, double cell_org,
                                            double inv_h, int nc) {
    double a = __dsub_rn(p, periodic ? lo : cell_org);
    if (periodic) {
        const long long ba = __double_as_longlong(a);
        if (!(ba >= 0 && ba < __double_as_longlong(L))) {
            p = wrap_crossed(p, lo, L);
            a = __dsub_rn(p, lo);
        }
    }
    const int k = (int)floor(__dmul_rn(a, inv_h));
    return k < 0 ? 0 : (k >= nc ? nc - 1 : k);
}

__global__ void k_cell_assign(int n, double* __restrict__ x, double* __restrict__ y, double* __restrict__ z,
                              CellGeom g, int* __restrict__ cell, int* __restrict__ count, unsigned* status) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double p[3] = {x[i], y[i], z[i]};
    const int cx = axis_cell_of(p[0], g.periodic[0], g.lo[0], g.L[0], g.org[0], g.inv_h[0], g.nc[0]);
    const int cy = axis_cell_of(p[1], g.periodic[1], g.lo[1], g.L[1], g.org[1], g.inv_h[1], g.nc[1]);
    const int cz = axis_cell_of(p[2], g.periodic[2], g.lo[2], g.L[2], g.org[2], g.inv_h[2], g.nc[2]);
    x[i] = p[0];
    y[i] = p[1];
    z[i] = p[2];
    int c = (cz * g.nc[1] + cy) * g.nc[0] + cx;
    if (!(isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2]))) {
        // spread non-finite atoms over the cells so that the per-cell work stays
        // bounded; the run is already invalid and the status word says so
        atomicOr(status, ERR_NONFINITE);
        c = i % (g.nc[0] * g.nc[1] * g.nc[2]);
    }
    cell[i] = c;
    atomicAdd(&count[c], 1);
}

// Exclusive scan of count[0..m) into start[0..m] in three launches: each
// block scans a tile of SCAN_TILE cells (k_scan_tiles), one block scans the
// tile totals (k_scan_totals), and k_scan_add adds the tile offsets.  The
// order of every sum is fixed.
constexpr int SCAN_THREADS = 512;
constexpr int SCAN_PER = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_PER;

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(int m, const int* __restrict__ count,
                                                             int* __restrict__ start, int* __restrict__ tile_sum) {
    __shared__ int warp_tot[SCAN_THREADS / 32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int base = blockIdx.x * SCAN_TILE + t * SCAN_PER;
    int v[SCAN_PER];
    int own = 0;
#pragma unroll
    for (int k = 0; k < SCAN_PER; k++) {
        v[k] = base + k < m ? count[base + k] : 0;
        own += v[k];
    }
    int incl = own;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += y;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int w = lane < SCAN_THREADS / 32 ? warp_tot[lane] : 0;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += y;
        }
        if (lane < SCAN_THREADS / 32) warp_tot[lane] = w;  // inclusive
    }
    __syncthreads();
    int run = incl - own + (warp > 0 ? warp_tot[warp - 1] : 0);
#pragma unroll
    for (int k = 0; k < SCAN_PER; k++) {
        if (base + k < m) start[base + k] = run;
        run += v[k];
    }
    if (t == SCAN_THREADS - 1) tile_sum[blockIdx.x] = warp_tot[SCAN_THREADS / 32 - 1];
}

// One block: tile totals -> exclusive tile offsets; start[m] = total.
__global__ void k_scan_totals(int ntiles, int m, int* __restrict__ tile_sum, int* __restrict__ start) {
    __shared__ int sums[1024];
    const int t = threadIdx.x, nt = blockDim.x;
    const int chunk = (ntiles + nt - 1) / nt;
    const int b = t * chunk, e = min(ntiles, b + chunk);
    int s = 0;
    for (int k = b; k < e; k++) s += tile_sum[k];
    sums[t] = s;
    __syncthreads();
    for (int off = 1; off < nt; off <<= 1) {
        const int y = t >= off ? sums[t - off] : 0;
        __syncthreads();
        sums[t] += y;
        __syncthreads();
    }
    int run = sums[t] - s;
    for (int k = b; k < e; k++) {
        const int c = tile_sum[k];
        tile_sum[k] = run;
        run += c;
    }
    if (t == nt - 1) start[m] = sums[t];
}

__global__ void k_scan_add(int m, int* __restrict__ start, const int* __restrict__ tile_off) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < m) start[k] += tile_off[k / SCAN_TILE];
}

// Replica filters of a partial rebuild: only atoms (by index) and cells of
// replicas whose flag is set take part; a null flag array takes everything.
__device__ __forceinline__ bool rep_on(const int* __restrict__ flag, const int* __restrict__ rep, int k) {
    return !flag || flag[rep[k]] != 0;
}

__global__ void k_scatter(int n, const int* __restrict__ cell, const int* __restrict__ start, int* __restrict__ fill,
                          int* __restrict__ perm, const int* __restrict__ rep_of, const int* __restrict__ rflag) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !rep_on(rflag, rep_of, i)) return;
    int c = cell[i];
    int s = start[c] + atomicAdd(&fill[c], 1);
    perm[s] = i;
}

// Atomic slot order is arbitrary; sorting each cell by previous index makes
// the final order (and every later floating-point sum) deterministic.
constexpr int CELL_SORT_MAX = 1024;

// Cells of up to CELL_SORT_SMALL atoms, one thread each: the indices sort in
// registers by an odd-even transposition network (fully unrolled).
constexpr int CELL_SORT_SMALL = 8;

// Cells too large for it go to a queue (big[0] of them, cells from big[1])
// that k_cell_sort_warp then drains, so that the warps do not walk every
// cell of a sparse grid.
__global__ void k_cell_sort_small(int m, const int* __restrict__ start, int* __restrict__ perm,
                                  const int* __restrict__ cell_rep, const int* __restrict__ rflag,
                                  int* __restrict__ big) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= m || !rep_on(rflag, cell_rep, c)) return;
    const int b = start[c], k = start[c + 1] - b;
    if (k > CELL_SORT_SMALL) big[1 + atomicAdd(big, 1)] = c;
    if (k <= 1 || k > CELL_SORT_SMALL) return;
    int v[CELL_SORT_SMALL];
#pragma unroll
    for (int q = 0; q < CELL_SORT_SMALL; q++) v[q] = q < k ? perm[b + q] : INT_MAX;
#pragma unroll
    for (int r = 0; r < CELL_SORT_SMALL; r++) {
#pragma unroll
        for (int q = r & 1; q + 1 < CELL_SORT_SMALL; q += 2) {
            const int lo = min(v[q], v[q + 1]), hi = max(v[q], v[q + 1]);
            v[q] = lo;
            v[q + 1] = hi;
        }
    }
#pragma unroll
    for (int q = 0; q < CELL_SORT_SMALL; q++)
        if (q < k) perm[b + q] = v[q];
}

// Larger cells, one warp each (k_cell_sort_small takes the cells of at most
// `skip` atoms when it runs): for cells of
// up to 32 atoms each lane holds one atom index and its rank (how many of the
// cell's indices are smaller) is counted with shuffles; the lanes then write
// in place.  Cells of more than 32 atoms take lane 0's insertion sort; a
// pathological cell beyond CELL_SORT_MAX is left unsorted (its order is then
// not reproducible) rather than sorted in O(k^2).
__global__ void k_cell_sort_warp(int m, const int* __restrict__ start, int* __restrict__ perm, int skip,
                                 const int* __restrict__ cell_rep, const int* __restrict__ rflag,
                                 const int* __restrict__ big) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    const int total = big ? big[0] : m;  // queued cells, or every cell
    for (int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < total; w += warps) {
        const int c = big ? big[1 + w] : w;
        if (!rep_on(rflag, cell_rep, c)) continue;  // uniform over the warp
        const int b = start[c], k = start[c + 1] - b;
        if (k <= skip) continue;  // empty, single, or sorted by k_cell_sort_small
        if (k <= 32) {
            const int v = lane < k ? perm[b + lane] : INT_MAX;
            int r = 0;
            for (int q = 0; q < k; q++) r += __shfl_sync(0xffffffffu, v, q) < v;
            __syncwarp();
            if (lane < k) perm[b + r] = v;
        } else if (lane == 0 && k <= CELL_SORT_MAX) {
            for (int p = b + 1; p < b + k; p++) {
                const int v = perm[p];
                int q = p - 1;
                while (q >= b && perm[q] > v) {
                    perm[q + 1] = perm[q];
                    q--;
                }
                perm[q + 1] = v;
            }
        }
        __syncwarp();
    }
}


// Per-atom state that survives a rebuild, gathered into staging and copied
// back so every array keeps its address (a captured step graph replays the
// same pointers).
struct AtomArrays {
    double *x, *y, *z, *vx, *vy, *vz;
    int *type, *id;
    unsigned* flag;
    double* extra;   // optional per-atom FP64 state (extra_n values per atom, slot-major)
    int extra_n;
};

// Also writes the sorted atoms' cells and the caller-to-sorted map (the new
// position k of caller atom id[o]).
__global__ void k_permute_gather(int n, const int* __restrict__ perm, AtomArrays a, AtomArrays st,
                                 const int* __restrict__ cell_old, int* __restrict__ cell_new,
                                 int* __restrict__ inv, const int* __restrict__ rep_of,
                                 const int* __restrict__ rflag) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || !rep_on(rflag, rep_of, k)) return;  // a replica's atoms stay in its index range
    int o = perm[k];
    cell_new[k] = cell_old[o];
    inv[a.id[o]] = k;
    st.x[k] = a.x[o];
    st.y[k] = a.y[o];
    st.z[k] = a.z[o];
    st.vx[k] = a.vx[o];
    st.vy[k] = a.vy[o];
    st.vz[k] = a.vz[o];
    st.type[k] = a.type[o];
    st.id[k] = a.id[o];
    st.flag[k] = a.flag[o];
    for (int q = 0; q < a.extra_n; q++) st.extra[(size_t)q * n + k] = a.extra[(size_t)q * n + o];
}

// The state a rebuild reorders, copied before the rebuild of a step (unless
// an earlier rebuild of the queued steps overflowed: then the copy of that
// rebuild's input is kept), with the step state.
// Only the first rebuild of the queued steps takes it (taken is cleared when
// a new batch of steps starts and set after the copy): a recovery restores
// that earlier state and replays from there, which reaches the same state.
__global__ void k_snapshot(int n, const int* __restrict__ halted, const int* __restrict__ taken, AtomArrays a,
                           AtomArrays snap, const unsigned char* __restrict__ st, unsigned char* __restrict__ st_snap,
                           int st_bytes) {
    if (*halted || *taken) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < st_bytes) st_snap[k] = st[k];
    if (k >= n) return;
    snap.x[k] = a.x[k];
    snap.y[k] = a.y[k];
    snap.z[k] = a.z[k];
    snap.vx[k] = a.vx[k];
    snap.vy[k] = a.vy[k];
    snap.vz[k] = a.vz[k];
    snap.type[k] = a.type[k];
    snap.id[k] = a.id[k];
    snap.flag[k] = a.flag[k];
}

__global__ void k_set_one(int* p) { *p = 1; }

// An overflowed build halts the queued steps' later rebuilds.
__global__ void k_halt_on_overflow(const unsigned* __restrict__ status, int* halted) {
    if (*status & ERR_NBR_OVERFLOW) *halted = 1;
}

__global__ void k_permute_copyback(int n, AtomArrays st, AtomArrays a, const int* __restrict__ rep_of,
                                   const int* __restrict__ rflag) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n || !rep_on(rflag, rep_of, k)) return;
    a.x[k] = st.x[k];
    a.y[k] = st.y[k];
    a.z[k] = st.z[k];
    a.vx[k] = st.vx[k];
    a.vy[k] = st.vy[k];
    a.vz[k] = st.vz[k];
    a.type[k] = st.type[k];
    a.id[k] = st.id[k];
    a.flag[k] = st.flag[k];
    for (int q = 0; q < a.extra_n; q++) a.extra[(size_t)q * n + k] = st.extra[(size_t)q * n + k];
}

__global__ void k_zero_ints(int m, int* __restrict__ a, int* __restrict__ b) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < m) {
        a[k] = 0;
        b[k] = 0;
    }
}

// The cell counters of the flagged replicas (and the sentinel past the last cell).
__global__ void k_zero_cells_rep(int m, int* __restrict__ count, int* __restrict__ fill,
                                 const int* __restrict__ cell_rep, const int* __restrict__ rflag) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > m || (k < m && !rep_on(rflag, cell_rep, k))) return;
    count[k] = 0;
    fill[k] = 0;
}

// After a build: count it for each replica rebuilt and clear the flags
// (all replicas after a full build).
__global__ void k_rep_build_done(int nrep, int full, int* __restrict__ rflag, int* __restrict__ builds) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrep; r += gridDim.x * blockDim.x) {
        if (full || rflag[r]) builds[r] += 1;
        rflag[r] = 0;
    }
}


// Cell of each sorted atom (cell[] is indexed by the previous order).

// Replica mode: every replica has its own periodic lengths and cell grid,
// and its cells occupy the global cell range [cell_base, cell_base + cells).
// base and hf are the replica's cell reference points in the pack frame
// (LocFrame below).
struct RepGeom {
    double lo[3], L[3], cell_org[3], cell_h[3], inv_h[3];
    int nc[3], periodic[3];
    int cell_base;
    ShiftF S;
    float base[3], hf[3];
};

// The pack coordinate is X = x + Q with Q = P - org, formed as FP32 hi + lo
// by pack_coord (the integrator refreshes the pack with the same function).
struct PackFrame {
    float Qh[3], Ql[3];
};

// The list screen works in a cell-local frame: each cell has an FP32
// reference point R(c) = fma(c, h, base) per axis (base = the pack-frame
// corner of cell 0), and an atom's local coordinate u = (X_hi - R) + X_lo is
// exact up to its final FP32 rounding (X_hi - R is Sterbenz-exact).  The
// build recomputes R(c) with the same expression.
struct LocFrame {
    int nc[3];
    float base[3], h[3];
};

__device__ __forceinline__ float cell_ref(int c, float h, float base) { return fmaf((float)c, h, base); }

__global__ void k_pack(int n, const double* __restrict__ x, const double* __restrict__ y,
                       const double* __restrict__ z, const int* __restrict__ type, PackFrame f,
                       PosPack* __restrict__ pack, float4* __restrict__ xref, const int* __restrict__ cell,
                       LocFrame lf, const int* __restrict__ rep_of, const RepGeom* __restrict__ rg,
                       const unsigned* __restrict__ aflag, float4* __restrict__ loc, unsigned* umax,
                       const int* __restrict__ rflag) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    float m = 0.f;
    if (i < n && (!rflag || rflag[rep_of[i]])) {
        PosPack p;
        pack_coord(x[i], f.Qh[0], f.Ql[0], p.hi.x, p.lo.x);
        pack_coord(y[i], f.Qh[1], f.Ql[1], p.hi.y, p.lo.y);
        pack_coord(z[i], f.Qh[2], f.Ql[2], p.hi.z, p.lo.z);
        p.hi.w = __int_as_float(type[i]);
        p.lo.w = 0.f;
        pack[i] = p;
        if (xref) xref[i] = make_float4(p.hi.x, p.hi.y, p.hi.z, 0.f);
        if (loc) {
            int c = cell[i];
            if (rep_of) {  // the replica's own grid and reference points
                const RepGeom& g = rg[rep_of[i]];
                c -= g.cell_base;
                for (int d = 0; d < 3; d++) {
                    lf.nc[d] = g.nc[d];
                    lf.h[d] = g.hf[d];
                    lf.base[d] = g.base[d];
                }
            }
            const int cx = c % lf.nc[0], cy = (c / lf.nc[0]) % lf.nc[1], cz = c / (lf.nc[0] * lf.nc[1]);
            const float ux = __fadd_rn(__fsub_rn(p.hi.x, cell_ref(cx, lf.h[0], lf.base[0])), p.lo.x);
            const float uy = __fadd_rn(__fsub_rn(p.hi.y, cell_ref(cy, lf.h[1], lf.base[1])), p.lo.y);
            const float uz = __fadd_rn(__fsub_rn(p.hi.z, cell_ref(cz, lf.h[2], lf.base[2])), p.lo.z);
            if (aflag && !(aflag[i] & 1u)) {
                // inactive (SetActive false): far from every centre, so no
                // list takes it, and outside the band's max |u|
                loc[i] = make_float4(3.0e38f, 3.0e38f, 3.0e38f, 0.f);
            } else {
                loc[i] = make_float4(ux, uy, uz, __int_as_float(type[i]));  // w: the type, for the row's type mask
                m = fmaxf(fabsf(ux), fmaxf(fabsf(uy), fabsf(uz)));
                if (!(m <= 3.0e38f)) m = 3.0e38f;  // non-finite: flagged by the cell assignment
            }
        }
    }
    if (loc) {
        // the largest |u| sets the width of the screening band
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(umax, __float_as_uint(m));
    }
}

// EAM cell tiles: besides the list entry, the build writes each entry's
// slot in the staged halo of its centre's tile (tile t, halo cell h:
// sb[t HC + h] + the candidate's offset in its cell).  Halo cells run z, y, x
// from the cell below the tile's first to the one above its last, the order
// the build visits a row's cells, so slots increase along a row.
struct TileOut {
    unsigned short* slot;  // null: no tile output
    const unsigned short* sb;
    const int* nst;
    int T[3], nt[3];
    int hx, hy;            // halo cells along x, y (T + 2)
    int HC, stride, cap;
};

struct BuildParams {
    TileOut to;
    int n, maxnb, hshift;
    int nc[3];
    int periodic[3];
    ShiftF L;
    double L64[3];
    double rsq;           // Rv*Rv in FP64 (VerletList.cpp:161)
    float rsq_lo, rsq_hi; // FP32 screening band around rsq
    float rv;             // Rv rounded to FP32
    float base[3], h[3];  // cell reference points (LocFrame)
    float hmax;           // largest cell size over all grids (screening band)
};

// Per axis, how many (cell, image) candidates a cell has and the idx-th one,
// in traversal order: cells c-1, c, c+1 (a periodic axis wraps them with
// image -1 / +1, a free axis drops the ones off the grid); a periodic axis
// of fewer than 3 cells takes every cell with images -1, 0, +1.
__device__ __forceinline__ int axis_count(int nc, int periodic) { return (periodic && nc < 3) ? 3 * nc : 3; }

__device__ __forceinline__ bool axis_cell(int c, int nc, int periodic, int idx, int& cell, int& shift) {
    if (periodic) {
        if (nc >= 3) {
            int k = c + idx - 1;
            shift = 0;
            if (k < 0) {
                k += nc;
                shift = -1;
            } else if (k >= nc) {
                k -= nc;
                shift = 1;
            }
            cell = k;
        } else {
            cell = idx / 3;
            shift = idx % 3 - 1;
        }
        return true;
    }
    const int k = c + idx - 1;
    cell = k;
    shift = 0;
    return k >= 0 && k < nc;
}

// The reference's FP64 test (dx = x_i - (x_j + s), r2 = (dx*dx + dy*dy) +
// dz*dz <= Rv^2) for the rare pairs inside the FP32 screening band.
__device__ __noinline__ bool exact_within(double Lx, double Ly, double Lz, double rsq, const double* __restrict__ x,
                                          const double* __restrict__ y, const double* __restrict__ z, int i, int k,
                                          unsigned code) {
    const int sx = nbr_sx(code), sy = nbr_sy(code), sz = nbr_sz(code);
    double gx = sx == 0 ? 0.0 : (sx > 0 ? Lx : -Lx);
    double gy = sy == 0 ? 0.0 : (sy > 0 ? Ly : -Ly);
    double gz = sz == 0 ? 0.0 : (sz > 0 ? Lz : -Lz);
    double dx = __dsub_rn(x[i], __dadd_rn(x[k], gx));
    double dy = __dsub_rn(y[i], __dadd_rn(y[k], gy));
    double dz = __dsub_rn(z[i], __dadd_rn(z[k], gz));
    double rr = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    return rr <= rsq && !(k == i && code == nbr_encode(0, 0, 0, 0));
}

// One thread per centre atom, screening in the cell-local frame: a
// candidate costs one 16-byte load of its local coordinate, the difference
// against the centre shifted by the (cell, image) offset R(c_i) - R(c_k) - sL
// (computed once per cell), and the squared length.  Every FP32 step is
// bounded by a few ulps of max(|u|, h); pairs within that band of Rv take
// the reference's FP64 test, so the list is the reference's exactly.  Rows
// come out in the traversal order of the other build variants.
//
// Grid accessors: the single box reads the kernel parameters, a replica its
// RepGeom entry (both inline to plain loads).
struct BoxGrid {
    const BuildParams& p;
    __device__ int nc(int d) const { return p.nc[d]; }
    __device__ int periodic(int d) const { return p.periodic[d]; }
    __device__ float base(int d) const { return p.base[d]; }
    __device__ float h(int d) const { return p.h[d]; }
    __device__ double L64(int d) const { return p.L64[d]; }
    __device__ const ShiftF& L() const { return p.L; }
    __device__ int cell_base() const { return 0; }
};

struct RepGrid {
    const RepGeom* r;
    __device__ int nc(int d) const { return r->nc[d]; }
    __device__ int periodic(int d) const { return r->periodic[d]; }
    __device__ float base(int d) const { return r->base[d]; }
    __device__ float h(int d) const { return r->hf[d]; }
    __device__ double L64(int d) const { return r->L[d]; }
    __device__ const ShiftF& L() const { return r->S; }
    __device__ int cell_base() const { return r->cell_base; }
};


template <bool TILES, class G>
__device__ __forceinline__ void build_row(const BuildParams& p, const G& g, int i, const float4* __restrict__ loc,
                                          const double* __restrict__ x, const double* __restrict__ y,
                                          const double* __restrict__ z, const int* __restrict__ cell,
                                          const int* __restrict__ start, const unsigned* __restrict__ umax,
                                          unsigned* __restrict__ nbr, int* __restrict__ nnb, unsigned* status,
                                          int* need, unsigned* __restrict__ nbmask) {
    // band: per component |error| <= 3 ulp(2 max(|u|, h)) (two operand
    // roundings, the offset, the difference); 2x margin, then sqrt(3) for
    // the length and 1e-6 relative for the squares
    const float U = fmaxf(__uint_as_float(*umax), p.hmax);
    const float dlt = 1.7320509f * (12.f * U * 2.3841858e-7f) + 1e-6f * p.rv;
    const float rl = fmaxf(p.rv - dlt, 0.f), rh = p.rv + dlt;
    const float rsq_lo = rl * rl * (1.f - 1e-6f), rsq_hi = rh * rh * (1.f + 1e-6f);
    const float4 ui = loc[i];
    if (ui.x == 3.0e38f) {  // inactive centre (k_pack): an empty row
        nnb[i] = 0;
        nbmask[i] = 0u;
        return;
    }
    unsigned tmask = 0u;  // types the row holds
    const int nx = g.nc(0), ny = g.nc(1), nz = g.nc(2);
    const int ci = cell[i] - g.cell_base();
    const int cx = ci % nx, cy = (ci / nx) % ny, cz = ci / (nx * ny);
    // tile slots (single box only): the centre's tile, where it is staged
    const unsigned short* tsb = nullptr;
    unsigned short* trow = nullptr;
    int tox = 0, toy = 0, toz = 0;
    if (TILES) {
        const int tx = cx / p.to.T[0], ty = cy / p.to.T[1], tz = cz / p.to.T[2];
        const int t = (tz * p.to.nt[1] + ty) * p.to.nt[0] + tx;
        if (p.to.nst[t] <= p.to.cap) {
            tsb = p.to.sb + (size_t)t * p.to.HC;
            trow = p.to.slot + (size_t)i * p.to.stride;
            tox = cx - tx * p.to.T[0];
            toy = cy - ty * p.to.T[1];
            toz = cz - tz * p.to.T[2];
        }
    }
    const float rx = cell_ref(cx, g.h(0), g.base(0)), ry = cell_ref(cy, g.h(1), g.base(1)),
                rz = cell_ref(cz, g.h(2), g.base(2));
    const int mx = axis_count(nx, g.periodic(0));
    const int my = axis_count(ny, g.periodic(1));
    const int mz = axis_count(nz, g.periodic(2));
    const unsigned self_code = nbr_encode(0, 0, 0, 0);
    int cnt = 0;
#pragma unroll 1
    for (int a = 0; a < mz; a++) {
        int kz, sz;
        if (!axis_cell(cz, nz, g.periodic(2), a, kz, sz)) continue;
        const float pz = ui.z + (((rz - cell_ref(kz, g.h(2), g.base(2))) - sel_shift(sz, g.L().hz)) -
                                 sel_shift(sz, g.L().lz));
#pragma unroll 1
        for (int b = 0; b < my; b++) {
            int ky, sy;
            if (!axis_cell(cy, ny, g.periodic(1), b, ky, sy)) continue;
            const float py = ui.y + (((ry - cell_ref(ky, g.h(1), g.base(1))) - sel_shift(sy, g.L().hy)) -
                                     sel_shift(sy, g.L().ly));
#pragma unroll 1
            for (int q = 0; q < mx; q++) {
                int kx, sx;
                if (!axis_cell(cx, nx, g.periodic(0), q, kx, sx)) continue;
                const float px = ui.x + (((rx - cell_ref(kx, g.h(0), g.base(0))) - sel_shift(sx, g.L().hx)) -
                                         sel_shift(sx, g.L().lx));
                const int c = g.cell_base() + (kz * ny + ky) * nx + kx;
                const unsigned code = nbr_encode(0, sx, sy, sz);
                const int e = start[c + 1];
                // slot of candidate k in the tile's staged halo: tb + k
                const int tb =
                    TILES && trow ? (int)tsb[((toz + a) * p.to.hy + (toy + b)) * p.to.hx + (tox + q)] - start[c] : 0;
                for (int k = start[c]; k < e; k++) {
                    const float4 uk = loc[k];
                    const float dx = px - uk.x, dy = py - uk.y, dz = pz - uk.z;
                    const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                    if (r2 > rsq_hi) continue;
                    if (k == i && code == self_code) continue;
                    // borderline pairs: the reference's FP64 arithmetic, out of line
                    if (!(r2 < rsq_lo) &&
                        !exact_within(g.L64(0), g.L64(1), g.L64(2), p.rsq, x, y, z, i, k, code))
                        continue;
                    if (r2 < 1e-6f) report_overlap(status, i, k);
                    tmask |= 1u << (__float_as_int(uk.w) & 31);
                    if (cnt < p.maxnb) {
                        nbr[nbr_at(i, cnt, p.hshift, p.maxnb)] = code | (unsigned)k;
                        if (TILES && trow) trow[cnt] = (unsigned short)(tb + k);
                    }
                    cnt++;
                }
            }
        }
    }
    if (cnt > p.maxnb) {
        atomicOr(status, ERR_NBR_OVERFLOW);
        atomicMax(need, cnt);
        cnt = p.maxnb;
    }
    nnb[i] = cnt;
    nbmask[i] = tmask;
}

// REP: the atom's replica supplies the grid, reference points and lengths.
// TILES: the rows also go out as EAM tile slots.
template <bool REP, bool TILES = false>
__global__ void __launch_bounds__(128, REP ? 7 : 8) k_build(BuildParams p, const RepGeom* __restrict__ rg,
                                               const int* __restrict__ rep_of, const float4* __restrict__ loc,
                                               const double* __restrict__ x, const double* __restrict__ y,
                                               const double* __restrict__ z, const int* __restrict__ cell,
                                               const int* __restrict__ start, const unsigned* __restrict__ umax,
                                               unsigned* __restrict__ nbr, int* __restrict__ nnb, unsigned* status,
                                               int* need, const int* __restrict__ rflag,
                                               unsigned* __restrict__ nbmask) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    if (REP && rflag && !rflag[rep_of[i]]) return;  // the replica keeps its list
    if (REP)
        build_row<false>(p, RepGrid{rg + rep_of[i]}, i, loc, x, y, z, cell, start, umax, nbr, nnb, status, need,
                         nbmask);
    else
        build_row<TILES>(p, BoxGrid{p}, i, loc, x, y, z, cell, start, umax, nbr, nnb, status, need, nbmask);
}

// ------------------------------------------------------------------ EAM cell tiles

struct TilePrep {
    int T[3], nt[3], nc[3], periodic[3];
    int hx, hy, HC;
    double corg[3], h[3];   // cell grid origin and widths
    double borg[3], P[3];   // pack frame: X = x - borg + P
};

// One CTA per tile: the atom count of each halo cell (z, y, x from the cell
// below the tile's first to the one above its last; a periodic axis wraps,
// a free axis has no cells beyond the grid), their exclusive scan as each
// cell's first staged slot (saturating at 65535; such a tile exceeds every
// capacity), the total, and the tile's lower corner in the pack frame.
constexpr int TILE_PREP_THREADS = 256;  // >= the 216 halo cells of a 4x4x4 tile

__global__ void __launch_bounds__(TILE_PREP_THREADS) k_tile_prep(TilePrep tp, const int* __restrict__ start,
                                                                 unsigned short* __restrict__ sb,
                                                                 int* __restrict__ nst, float4* __restrict__ org) {
    __shared__ int s_warp[TILE_PREP_THREADS / 32];
    const int t = blockIdx.x;
    const int tx = t % tp.nt[0], ty = (t / tp.nt[0]) % tp.nt[1], tz = t / (tp.nt[0] * tp.nt[1]);
    const int h = threadIdx.x;
    int cnt = 0;
    if (h < tp.HC) {
        const int l[3] = {h % tp.hx, (h / tp.hx) % tp.hy, h / (tp.hx * tp.hy)};
        const int t3[3] = {tx, ty, tz};
        int k[3];
        bool ok = true;
        for (int d = 0; d < 3; d++) {
            int gk = t3[d] * tp.T[d] - 1 + l[d];
            if (tp.periodic[d]) {
                if (gk < 0) gk += tp.nc[d];
                else if (gk >= tp.nc[d]) gk -= tp.nc[d];
            } else if (gk < 0 || gk >= tp.nc[d]) {
                ok = false;
            }
            k[d] = gk;
        }
        if (ok) {
            const int c = (k[2] * tp.nc[1] + k[1]) * tp.nc[0] + k[0];
            cnt = start[c + 1] - start[c];
        }
    }
    // block exclusive scan
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int incl = cnt;
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) s_warp[w] = incl;
    __syncthreads();
    if (w == 0) {
        int v = lane < TILE_PREP_THREADS / 32 ? s_warp[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += u;
        }
        if (lane < TILE_PREP_THREADS / 32) s_warp[lane] = v;
    }
    __syncthreads();
    const int excl = incl - cnt + (w > 0 ? s_warp[w - 1] : 0);
    if (h < tp.HC) sb[(size_t)t * tp.HC + h] = (unsigned short)min(excl, 65535);
    if (h == tp.HC - 1) nst[t] = excl + cnt;
    if (h == 0) {
        const int t3[3] = {tx, ty, tz};
        float o[3];
        for (int d = 0; d < 3; d++)
            o[d] = (float)(__dadd_rn(__dsub_rn(fma((double)(t3[d] * tp.T[d]), tp.h[d], tp.corg[d]), tp.borg[d]),
                                     tp.P[d]));
        org[t] = make_float4(o[0], o[1], o[2], 0.f);
    }
}

// ------------------------------------------------------------------ replicas

__global__ void k_cell_assign_rep(int n, double* __restrict__ x, double* __restrict__ y, double* __restrict__ z,
                                  const int* __restrict__ rep_of, const RepGeom* __restrict__ rg,
                                  int* __restrict__ cell, int* __restrict__ count, unsigned* status,
                                  const int* __restrict__ rflag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !rep_on(rflag, rep_of, i)) return;
    const RepGeom& g = rg[rep_of[i]];
    double p[3] = {x[i], y[i], z[i]};
    const int cx = axis_cell_of(p[0], g.periodic[0], g.lo[0], g.L[0], g.cell_org[0], g.inv_h[0], g.nc[0]);
    const int cy = axis_cell_of(p[1], g.periodic[1], g.lo[1], g.L[1], g.cell_org[1], g.inv_h[1], g.nc[1]);
    const int cz = axis_cell_of(p[2], g.periodic[2], g.lo[2], g.L[2], g.cell_org[2], g.inv_h[2], g.nc[2]);
    x[i] = p[0];
    y[i] = p[1];
    z[i] = p[2];
    int c = g.cell_base + (cz * g.nc[1] + cy) * g.nc[0] + cx;
    if (!(isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2]))) {
        atomicOr(status, ERR_NONFINITE);
        c = g.cell_base + i % (g.nc[0] * g.nc[1] * g.nc[2]);
    }
    cell[i] = c;
    atomicAdd(&count[c], 1);
}

// Same list as k_build with LANES threads per atom: the lanes test
// consecutive atoms of a cell together and append the accepted ones in lane
// order (ballot + prefix popcount), so each row keeps exactly the
// cell-traversal order of the one-thread build.
template <int LANES>
__global__ void __launch_bounds__(256) k_build_lanes(BuildParams p, const PosPack* __restrict__ pack,
                                                     const double* __restrict__ x, const double* __restrict__ y,
                                                     const double* __restrict__ z, const int* __restrict__ cell,
                                                     const int* __restrict__ start, unsigned* __restrict__ nbr,
                                                     int* __restrict__ nnb, unsigned* status, int* need) {
    const int lane = threadIdx.x & (LANES - 1);
    const int gbase = (threadIdx.x & 31) & ~(LANES - 1);
    const unsigned gmask = (LANES == 32 ? 0xffffffffu : ((1u << LANES) - 1u)) << gbase;
    const int i = blockIdx.x * (blockDim.x / LANES) + threadIdx.x / LANES;
    if (i >= p.n) return;  // whole groups leave together
    const PosPack pi = pack[i];
    const int ci = cell[i];
    const int cx = ci % p.nc[0], cy = (ci / p.nc[0]) % p.nc[1], cz = ci / (p.nc[0] * p.nc[1]);
    const int mx = axis_count(p.nc[0], p.periodic[0]);
    const int my = axis_count(p.nc[1], p.periodic[1]);
    const int mz = axis_count(p.nc[2], p.periodic[2]);
    int cnt = 0;
    for (int a = 0; a < mz; a++)
        for (int b = 0; b < my; b++)
            for (int q = 0; q < mx; q++) {
                int kz, sz, ky, sy, kx, sx;
                if (!axis_cell(cz, p.nc[2], p.periodic[2], a, kz, sz) ||
                    !axis_cell(cy, p.nc[1], p.periodic[1], b, ky, sy) ||
                    !axis_cell(cx, p.nc[0], p.periodic[0], q, kx, sx))
                    continue;
                const int c = (kz * p.nc[1] + ky) * p.nc[0] + kx;
                const unsigned code = nbr_encode(0, sx, sy, sz);
                const bool self_image = (sx == 0 && sy == 0 && sz == 0);
                const int e = start[c + 1];
                for (int k0 = start[c]; k0 < e; k0 += LANES) {
                    const int k = k0 + lane;
                    bool in = false;
                    if (k < e && !(self_image && k == i)) {
                        const PosPack pk = pack[k];
                        const float3 d = pair_delta(pi.hi, pi.lo, pk.hi, pk.lo, code, p.L);
                        const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
                        if (r2 <= p.rsq_hi) {
                            in = r2 < p.rsq_lo;
                            if (!in) {
                                // borderline: the reference's FP64 arithmetic decides
                                double gx = sx == 0 ? 0.0 : (sx > 0 ? p.L64[0] : -p.L64[0]);
                                double gy = sy == 0 ? 0.0 : (sy > 0 ? p.L64[1] : -p.L64[1]);
                                double gz = sz == 0 ? 0.0 : (sz > 0 ? p.L64[2] : -p.L64[2]);
                                double dx = __dsub_rn(x[i], __dadd_rn(x[k], gx));
                                double dy = __dsub_rn(y[i], __dadd_rn(y[k], gy));
                                double dz = __dsub_rn(z[i], __dadd_rn(z[k], gz));
                                double rr = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)),
                                                      __dmul_rn(dz, dz));
                                in = rr <= p.rsq;
                            }
                            if (in && r2 < 1e-6f) report_overlap(status, i, k);
                        }
                    }
                    const unsigned bal = __ballot_sync(gmask, in) >> gbase;
                    if (in) {
                        const int pos = cnt + __popc(bal & ((1u << lane) - 1u));
                        if (pos < p.maxnb) nbr[nbr_at(i, pos, p.hshift, p.maxnb)] = code | (unsigned)k;
                    }
                    cnt += __popc(bal);
                }
            }
    if (lane == 0) {
        if (cnt > p.maxnb) {
            atomicOr(status, ERR_NBR_OVERFLOW);
            atomicMax(need, cnt);
            cnt = p.maxnb;
        }
        nnb[i] = cnt;
    }
}

// Cell-centric build: one CTA per cell.  The CTA copies the packs of every
// (cell, image) of the cell's neighbourhood into shared memory in traversal
// order (chunks of `cap` candidates when the neighbourhood is larger), and
// groups of 8 lanes test one centre atom each against the staged candidates,
// appending in lane order.  Rows come out identical to k_build's.
constexpr int BUILD_CELL_THREADS = 128;
constexpr int BUILD_GROUP = 8;

__global__ void __launch_bounds__(BUILD_CELL_THREADS) k_build_cells(BuildParams p, const PosPack* __restrict__ pack,
                                                                    const double* __restrict__ x,
                                                                    const double* __restrict__ y,
                                                                    const double* __restrict__ z,
                                                                    const int* __restrict__ start, int cap,
                                                                    unsigned* __restrict__ nbr, int* __restrict__ nnb,
                                                                    unsigned* status, int* need) {
    extern __shared__ float4 s_cand[];  // 2 float4 per candidate: hi (w = atom index), lo (w = image code)
    __shared__ int s_cell[64], s_code[64], s_pref[65];
    __shared__ float4 s_sh[64], s_sl[64];  // split image shift by the entry's 6 image bits
    for (int k = threadIdx.x; k < 64; k += blockDim.x) {
        const float fx = (float)((k & 3) - 1), fy = (float)(((k >> 2) & 3) - 1), fz = (float)(((k >> 4) & 3) - 1);
        s_sh[k] = make_float4(fx * p.L.hx, fy * p.L.hy, fz * p.L.hz, 0.f);
        s_sl[k] = make_float4(fx * p.L.lx, fy * p.L.ly, fz * p.L.lz, 0.f);
    }
    const int c = blockIdx.x;
    const int cx = c % p.nc[0], cy = (c / p.nc[0]) % p.nc[1], cz = c / (p.nc[0] * p.nc[1]);
    const int mx = axis_count(p.nc[0], p.periodic[0]);
    const int my = axis_count(p.nc[1], p.periodic[1]);
    const int mz = axis_count(p.nc[2], p.periodic[2]);
    const int ncombo = mx * my * mz;  // <= 27 unless a periodic axis has fewer than 3 cells
    // enumerate (cell, image) combos in traversal order (combo t = (a, b, q)
    // with q fastest); the first two warps look up one combo each in parallel
    if (threadIdx.x < 64) {
        const int t = threadIdx.x;
        int cnt = 0, cc = 0;
        unsigned code = 0;
        if (t < ncombo) {
            const int q = t % mx, b = (t / mx) % my, a = t / (mx * my);
            int kz, sz, ky, sy, kx, sx;
            if (axis_cell(cz, p.nc[2], p.periodic[2], a, kz, sz) && axis_cell(cy, p.nc[1], p.periodic[1], b, ky, sy) &&
                axis_cell(cx, p.nc[0], p.periodic[0], q, kx, sx)) {
                cc = (kz * p.nc[1] + ky) * p.nc[0] + kx;
                cnt = start[cc + 1] - start[cc];
                code = nbr_encode(0, sx, sy, sz);
            }
        }
        s_cell[t] = cc;
        s_code[t] = (int)code;
        s_pref[t + 1] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        s_pref[0] = 0;
        for (int t = 0; t < 64; t++) s_pref[t + 1] += s_pref[t];
    }
    __syncthreads();
    const int nc_used = ncombo < 64 ? ncombo : 64;
    const int total = s_pref[nc_used];
    const int c_begin = start[c], c_end = start[c + 1];
    const int group = threadIdx.x / BUILD_GROUP, lane = threadIdx.x & (BUILD_GROUP - 1);
    const int gbase = (threadIdx.x & 31) & ~(BUILD_GROUP - 1);
    const unsigned gmask = ((1u << BUILD_GROUP) - 1u) << gbase;
    const unsigned self_code = nbr_encode(0, 0, 0, 0);
    for (int batch = c_begin; batch < c_end; batch += BUILD_CELL_THREADS / BUILD_GROUP) {
        const int i = batch + group;
        const bool active = i < c_end;
        PosPack pi;
        if (active) pi = pack[i];
        int cnt = 0;
        for (int c0 = 0; c0 < total; c0 += cap) {
            const int c1 = min(total, c0 + cap);
            __syncthreads();
            for (int t = c0 + threadIdx.x; t < c1; t += blockDim.x) {
                int lo = 0, hi = nc_used;  // combo holding candidate t
                while (hi - lo > 1) {
                    int mid = (lo + hi) >> 1;
                    if (s_pref[mid] <= t) lo = mid;
                    else hi = mid;
                }
                const int k = start[s_cell[lo]] + (t - s_pref[lo]);
                PosPack pk = pack[k];
                pk.hi.w = __int_as_float(k);
                pk.lo.w = __int_as_float(s_code[lo]);
                s_cand[2 * (t - c0)] = pk.hi;
                s_cand[2 * (t - c0) + 1] = pk.lo;
            }
            __syncthreads();
            if (active) {
                for (int k0 = c0; k0 < c1; k0 += BUILD_GROUP) {
                    const int t = k0 + lane;
                    bool in = false;
                    unsigned entry = 0;
                    if (t < c1) {
                        const float4 hk = s_cand[2 * (t - c0)], lk = s_cand[2 * (t - c0) + 1];
                        const unsigned code = __float_as_uint(lk.w);
                        entry = code | __float_as_uint(hk.w);
                        const float4 sh = s_sh[code >> 26], sl = s_sl[code >> 26];
                        const float dx = __fadd_rn(__fsub_rn(__fsub_rn(pi.hi.x, hk.x), sh.x),
                                                   __fsub_rn(__fsub_rn(pi.lo.x, lk.x), sl.x));
                        const float dy = __fadd_rn(__fsub_rn(__fsub_rn(pi.hi.y, hk.y), sh.y),
                                                   __fsub_rn(__fsub_rn(pi.lo.y, lk.y), sl.y));
                        const float dz = __fadd_rn(__fsub_rn(__fsub_rn(pi.hi.z, hk.z), sh.z),
                                                   __fsub_rn(__fsub_rn(pi.lo.z, lk.z), sl.z));
                        const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                        // the atom itself is the only candidate at exactly zero distance
                        in = r2 < p.rsq_lo && r2 > 0.f;
                        if (r2 >= p.rsq_lo && r2 <= p.rsq_hi)
                            in = exact_within(p.L64[0], p.L64[1], p.L64[2], p.rsq, x, y, z, i,
                                              (int)(entry & (unsigned)INDEX_MASK), code);
                        if (in && r2 < 1e-6f) report_overlap(status, i, (int)(entry & (unsigned)INDEX_MASK));
                    }
                    const unsigned bal = __ballot_sync(gmask, in) >> gbase;
                    if (in) {
                        const int pos = cnt + __popc(bal & ((1u << lane) - 1u));
                        if (pos < p.maxnb) nbr[nbr_at(i, pos, p.hshift, p.maxnb)] = entry;
                    }
                    cnt += __popc(bal);
                }
            }
        }
        if (active && lane == 0) {
            if (cnt > p.maxnb) {
                atomicOr(status, ERR_NBR_OVERFLOW);
                atomicMax(need, cnt);
                cnt = p.maxnb;
            }
            nnb[i] = cnt;
        }
    }
}

// rev at (i, s): the slot of (i, -image) in the row of j = nbr at (i, s).
// For every list entry (i, s) -> j, the slot of i in row j: REV_LANES
// threads per centre, each searching for every REV_LANES-th entry (the
// searches are independent chains of loads; lanes keep more of them in
// flight).
constexpr int REV_LANES = 4;

__global__ void k_reverse(int n, int hshift, int maxnb, const unsigned* __restrict__ nbr,
                          const int* __restrict__ nnb, int* __restrict__ rev, unsigned* status,
                          const int* __restrict__ rep_of, const int* __restrict__ rflag) {
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    const int i = (int)(t / REV_LANES), lane = (int)(t % REV_LANES);
    if (i >= n) return;
    if (rflag && !rflag[rep_of[i]]) return;  // the replica kept its rows, and so their reverse slots
    int m = nnb[i];
    for (int s = lane; s < m; s += REV_LANES) {
        unsigned e = nbr[nbr_at(i, s, hshift, maxnb)];
        int j = nbr_index(e);
        unsigned want = nbr_encode(i, -nbr_sx(e), -nbr_sy(e), -nbr_sz(e));
        int mj = nnb[j], found = -1;
        for (int u = 0; u < mj; u++)
            if (nbr[nbr_at(j, u, hshift, maxnb)] == want) {
                found = u;
                break;
            }
        if (found < 0) atomicOr(status, ERR_NBR_OVERFLOW);
        rev[nbr_at(i, s, hshift, maxnb)] = found < 0 ? 0 : found;
    }
}

// ---------------------------------------------------------------- host side

// Cells along an axis of extent ext: as many as fit with each at least
// Rv (1 + 1e-12) wide (the margin absorbs cell_coord's rounding).
static int cells_along(double ext, double rv) {
    const int nc = (int)(ext / (rv * (1.0 + 1e-12)));
    return nc < 1 ? 1 : nc;
}

void nlist_prepare_geometry(Context* c) {
    double rv = c->rc_max + c->skin;
    BoxGeom& b = c->box;
    for (int d = 0; d < 3; d++) {
        if (b.periodic[d]) {
            b.cell_org[d] = b.lo[d];
            b.nc[d] = cells_along(b.L[d], rv);
            b.cell_h[d] = b.L[d] / b.nc[d];
        } else {
            // free axis: a fixed grid over the box with a margin; atoms
            // beyond it are clamped into the edge cells, which keeps the
            // 27-cell search complete.
            double margin = 2.0 * rv;
            b.cell_org[d] = b.lo[d] - margin;
            double ext = b.L[d] + 2.0 * margin;
            b.nc[d] = cells_along(ext, rv);
            b.cell_h[d] = ext / b.nc[d];
        }
    }
}

// Cell grids of the replicas (same rules as nlist_prepare_geometry, per
// replica) and the replica of every atom; uploads both.
int replica_prepare(Context* c) {
    const double rv = c->rc_max + c->skin;
    std::vector<RepGeom> rg(c->nrep);
    std::vector<ShiftF> sh(c->nrep);
    int base = 0;
    double hmax = 0.0;
    for (int r = 0; r < c->nrep; r++) {
        RepGeom& g = rg[r];
        for (int d = 0; d < 3; d++) {
            g.lo[d] = c->rep_lo[3 * r + d];
            g.L[d] = c->rep_hi[3 * r + d] - c->rep_lo[3 * r + d];
            g.periodic[d] = c->rep_periodic[d];
            if (g.periodic[d]) {
                g.cell_org[d] = g.lo[d];
                g.nc[d] = cells_along(g.L[d], rv);
                g.cell_h[d] = g.L[d] / g.nc[d];
            } else {
                const double margin = 2.0 * rv;
                g.cell_org[d] = g.lo[d] - margin;
                const double ext = g.L[d] + 2.0 * margin;
                g.nc[d] = cells_along(ext, rv);
                g.cell_h[d] = ext / g.nc[d];
            }
            g.inv_h[d] = 1.0 / g.cell_h[d];
            g.base[d] = (float)(g.cell_org[d] - c->box.org[d] + c->box.P[d]);
            g.hf[d] = (float)g.cell_h[d];
            hmax = std::max(hmax, g.cell_h[d]);
        }
        const float lh[3] = {(float)g.L[0], (float)g.L[1], (float)g.L[2]};
        g.S.hx = lh[0];
        g.S.hy = lh[1];
        g.S.hz = lh[2];
        g.S.lx = (float)(g.L[0] - (double)lh[0]);
        g.S.ly = (float)(g.L[1] - (double)lh[1]);
        g.S.lz = (float)(g.L[2] - (double)lh[2]);
        sh[r] = g.S;
        g.cell_base = base;
        base += g.nc[0] * g.nc[1] * g.nc[2];
    }
    c->rep_cells = base;
    c->rep_hmax = hmax;
    // The step graph holds these pointers: allocate once (omdg_set_replicas
    // frees them) and reallocate only for a larger atom capacity, dropping
    // the graph then.  Contents are rewritten in place.
    cudaError_t e = cudaSuccess;
    if (!c->d_rep_geom) e = cudaMalloc(&c->d_rep_geom, sizeof(RepGeom) * c->nrep);
    if (e == cudaSuccess && !c->d_rep_shift) e = cudaMalloc(&c->d_rep_shift, sizeof(ShiftF) * c->nrep);
    if (e == cudaSuccess && !c->d_rep_start) e = cudaMalloc(&c->d_rep_start, sizeof(int) * (c->nrep + 1));
    if (e == cudaSuccess && !c->d_rep_sums) e = cudaMalloc(&c->d_rep_sums, sizeof(double) * 2 * c->nrep);
    if (e == cudaSuccess && !c->d_rep_flag) {
        e = cudaMalloc(&c->d_rep_flag, sizeof(int) * c->nrep);
        if (e == cudaSuccess) e = cudaMemsetAsync(c->d_rep_flag, 0, sizeof(int) * c->nrep, c->stream);
    }
    if (e == cudaSuccess && !c->d_rep_builds) {
        e = cudaMalloc(&c->d_rep_builds, sizeof(int) * c->nrep);
        if (e == cudaSuccess) e = cudaMemsetAsync(c->d_rep_builds, 0, sizeof(int) * c->nrep, c->stream);
    }
    if (e == cudaSuccess && !c->d_cell_rep) e = cudaMalloc(&c->d_cell_rep, sizeof(int) * std::max(1, base));
    if (e == cudaSuccess && (!c->d_rep_of || c->rep_of_cap < c->cap)) {
        cudaFree(c->d_rep_of);
        c->d_rep_of = nullptr;
        e = cudaMalloc(&c->d_rep_of, sizeof(int) * std::max(1, c->cap));
        c->rep_of_cap = c->cap;
        invalidate_graph(c);
    }
    if (e != cudaSuccess) return set_error(c, OMDG_ENOMEM, "replica tables");
    std::vector<int> of(c->n), cell_rep(std::max(1, base));
    for (int r = 0; r < c->nrep; r++)
        for (int i = c->rep_start[r]; i < c->rep_start[r + 1]; i++) of[i] = r;
    for (int r = 0; r < c->nrep; r++)
        for (int k = rg[r].cell_base; k < (r + 1 < c->nrep ? rg[r + 1].cell_base : base); k++) cell_rep[k] = r;
    cudaMemcpyAsync(c->d_cell_rep, cell_rep.data(), sizeof(int) * cell_rep.size(), cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(c->d_rep_geom, rg.data(), sizeof(RepGeom) * c->nrep, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(c->d_rep_shift, sh.data(), sizeof(ShiftF) * c->nrep, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(c->d_rep_of, of.data(), sizeof(int) * c->n, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(c->d_rep_start, c->rep_start.data(), sizeof(int) * (c->nrep + 1), cudaMemcpyHostToDevice,
                    c->stream);
    return check_cuda(c, cudaStreamSynchronize(c->stream), "replica tables");
}

// The tiled EAM passes apply to one box (no replicas) whose periodic axes
// have at least three cells (the build's 27-cell stencil), with tiles of at
// most 4 cells a side.
int tile_prepare(Context* c) {
    c->tile_want = false;
    c->tile_valid = false;
    if (!tiles_apply(c)) return OMDG_OK;
    const BoxGeom& b = c->box;
    for (int d = 0; d < 3; d++) {
        if (b.periodic[d] && b.nc[d] < 3) return OMDG_OK;
        if (c->tile_dim[d] < 1 || c->tile_dim[d] > 4) return OMDG_OK;
    }
    int nt[3], hc = 1;
    for (int d = 0; d < 3; d++) {
        nt[d] = (b.nc[d] + c->tile_dim[d] - 1) / c->tile_dim[d];
        hc *= c->tile_dim[d] + 2;
    }
    const int ntiles = nt[0] * nt[1] * nt[2];
    if ((long long)ntiles * hc > c->tile_alloc || !c->tile_sb) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(c->stream, &cs);
        if (cs != cudaStreamCaptureStatusNone) return set_error(c, OMDG_ESTATE, "tile grid grew inside a capture");
        invalidate_graph(c);
        cudaFree(c->tile_sb);
        cudaFree(c->tile_nst);
        cudaFree(c->tile_org);
        c->tile_sb = nullptr;
        c->tile_nst = nullptr;
        c->tile_org = nullptr;
        c->tile_alloc = 0;
        if (cudaMalloc(&c->tile_sb, sizeof(unsigned short) * (size_t)ntiles * hc) != cudaSuccess ||
            cudaMalloc(&c->tile_nst, sizeof(int) * ntiles) != cudaSuccess ||
            cudaMalloc(&c->tile_org, sizeof(float4) * ntiles) != cudaSuccess)
            return set_error(c, OMDG_ENOMEM, "tile tables");
        c->tile_alloc = ntiles * hc;
    }
    for (int d = 0; d < 3; d++) c->tile_nt[d] = nt[d];
    c->tile_count = ntiles;
    c->tile_hc = hc;
    c->tile_want = true;
    return tile_reserve_slots(c);
}

// The slot rows: one per atom of the capacity, maxnb rounded up to 8 slots.
int tile_reserve_slots(Context* c) {
    if (!c->tile_want || c->maxnb <= 0) return OMDG_OK;
    const int stride = (c->maxnb + 7) & ~7;
    const size_t need = (size_t)c->cap * stride;
    if (need > c->tslot_alloc || !c->tslot) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(c->stream, &cs);
        if (cs != cudaStreamCaptureStatusNone) return set_error(c, OMDG_ESTATE, "tile slots grew inside a capture");
        invalidate_graph(c);
        cudaFree(c->tslot);
        c->tslot = nullptr;
        c->tslot_alloc = 0;
        if (cudaMalloc(&c->tslot, need * sizeof(unsigned short)) != cudaSuccess)
            return set_error(c, OMDG_ENOMEM, "tile slot rows");
        c->tslot_alloc = need;
    }
    if (stride != c->tile_stride) invalidate_graph(c);
    c->tile_stride = stride;
    return OMDG_OK;
}

void tile_release(Context* c) {
    cudaFree(c->tile_sb);
    cudaFree(c->tile_nst);
    cudaFree(c->tile_org);
    cudaFree(c->tslot);
    c->tile_sb = nullptr;
    c->tile_nst = nullptr;
    c->tile_org = nullptr;
    c->tslot = nullptr;
    c->tile_alloc = 0;
    c->tslot_alloc = 0;
    c->tile_want = false;
    c->tile_valid = false;
}

size_t nlist_slots(const Context* c, int maxnb) {
    size_t H = (size_t)1 << c->nbr_hshift;
    size_t slices = ((size_t)c->cap + H - 1) / H;
    return slices * H * (size_t)maxnb;
}

int nlist_reserve(Context* c, int maxnb) {
    size_t need = nlist_slots(c, maxnb) * sizeof(unsigned);
    if (maxnb <= c->maxnb && c->nbr) return OMDG_OK;
    cudaFree(c->nbr);
    cudaFree(c->rev);
    cudaFree(c->slot_buf);
    c->nbr = nullptr;
    c->rev = nullptr;
    c->slot_buf = nullptr;
    if (cudaMalloc(&c->nbr, need) != cudaSuccess) return set_error(c, OMDG_ENOMEM, "neighbour list allocation");
    if (c->need_rev) {
        if (cudaMalloc(&c->rev, need) != cudaSuccess) return set_error(c, OMDG_ENOMEM, "reverse slot allocation");
        if (cudaMalloc(&c->slot_buf, nlist_slots(c, maxnb) * sizeof(float4)) != cudaSuccess)
            return set_error(c, OMDG_ENOMEM, "slot buffer allocation");
    }
    c->maxnb = maxnb;
    c->nbr_bytes = (long)need;
    return tile_reserve_slots(c);
}

static int ensure_cells(Context* c, int m) {
    if (m + 1 <= c->ncell_cap) return OMDG_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(c->stream, &cs);
    if (cs != cudaStreamCaptureStatusNone) return set_error(c, OMDG_ESTATE, "cell grid grew inside a captured step");
    invalidate_graph(c);  // a captured step holds the old cell arrays
    cudaFree(c->cell_count);
    cudaFree(c->cell_start);
    cudaFree(c->cell_fill);
    cudaFree(c->cell_tile_sum);
    int cap = m + 1;
    if (cudaMalloc(&c->cell_count, cap * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&c->cell_start, (cap + 1) * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&c->cell_fill, cap * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&c->cell_tile_sum, (cap / SCAN_TILE + 2) * sizeof(int)) != cudaSuccess)
        return set_error(c, OMDG_ENOMEM, "cell arrays");
    c->ncell_cap = cap;
    return OMDG_OK;
}

PackFrame pack_frame(const Context* c) {
    PackFrame f;
    for (int d = 0; d < 3; d++) {
        const double Q = c->box.P[d] - c->box.org[d];
        f.Qh[d] = (float)Q;
        f.Ql[d] = (float)(Q - (double)f.Qh[d]);
    }
    return f;
}

int integrate_pack(Context* c) {
    if (c->n == 0) return OMDG_OK;
    // xref keeps the positions of the last build (the displacement reference)
    k_pack<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->x, c->y, c->z, c->type, pack_frame(c), c->pack,
                                                       nullptr, nullptr, LocFrame{}, nullptr, nullptr,
                                                       nullptr, nullptr, nullptr, nullptr);
    c->launches++;
    return check_cuda(c, cudaGetLastError(), "pack");
}

int nlist_build(Context* c) {
    int n = c->n;
    if (n == 0) return OMDG_OK;
    CellGeom g = cell_geom(c);
    const bool reps = c->nrep > 0;
    int m = reps ? c->rep_cells : g.nc[0] * g.nc[1] * g.nc[2];
    int rc = ensure_cells(c, m);
    if (rc) return rc;
    cudaStream_t s = c->stream;
    prof_begin(c, "cell_sort");
    if (c->build_in_step && c->snap_d) {
        AtomArrays cur0{c->x, c->y, c->z, c->vx, c->vy, c->vz, c->type, c->id, c->aflag, nullptr, 0};
        AtomArrays snap{c->snap_d, c->snap_d + c->cap, c->snap_d + 2 * (size_t)c->cap, c->snap_d + 3 * (size_t)c->cap,
                        c->snap_d + 4 * (size_t)c->cap, c->snap_d + 5 * (size_t)c->cap, c->snap_i,
                        c->snap_i + c->cap, reinterpret_cast<unsigned*>(c->snap_i + 2 * (size_t)c->cap), nullptr, 0};
        const int sb = (int)step_state_bytes();
        int* taken = c->d_flags + 6;
        k_snapshot<<<grid_for(std::max(n, sb), 256), 256, 0, s>>>(
            n, step_state_halted(c), taken, cur0, snap, static_cast<const unsigned char*>(c->d_state),
            static_cast<unsigned char*>(c->snap_state), sb);
        k_set_one<<<1, 1, 0, s>>>(taken);
        c->launches += 2;
    }
    // a partial build (replica mode, inside a step): only the replicas whose
    // atoms moved past skin/2 are re-sorted and re-listed; every replica keeps
    // its index range and cell range, so the others' arrays stay valid
    const int* rflag = (reps && c->build_partial) ? c->d_rep_flag : nullptr;
    if (rflag)
        k_zero_cells_rep<<<grid_for(m + 1, 256), 256, 0, s>>>(m, c->cell_count, c->cell_fill, c->d_cell_rep, rflag);
    else
        k_zero_ints<<<grid_for(m + 1, 256), 256, 0, s>>>(m + 1, c->cell_count, c->cell_fill);
    if (reps)
        k_cell_assign_rep<<<grid_for(n, 256), 256, 0, s>>>(n, c->x, c->y, c->z, c->d_rep_of,
                                                             static_cast<const RepGeom*>(c->d_rep_geom), c->cell,
                                                             c->cell_count, c->d_status, rflag);
    else
        k_cell_assign<<<grid_for(n, 256), 256, 0, s>>>(n, c->x, c->y, c->z, g, c->cell, c->cell_count,
                                                         c->d_status);
    const int ntiles = (m + SCAN_TILE - 1) / SCAN_TILE;
    k_scan_tiles<<<ntiles, SCAN_THREADS, 0, s>>>(m, c->cell_count, c->cell_start, c->cell_tile_sum);
    k_scan_totals<<<1, 1024, 0, s>>>(ntiles, m, c->cell_tile_sum, c->cell_start);
    k_scan_add<<<grid_for(m, 256), 256, 0, s>>>(m, c->cell_start, c->cell_tile_sum);
    k_scatter<<<grid_for(n, 256), 256, 0, s>>>(n, c->cell, c->cell_start, c->cell_fill, c->perm, c->d_rep_of, rflag);
    // most cells of a sparse grid (replica margins, vacuum) hold 0 or 1 atoms:
    // a bounded grid of warps strides over the cells instead of one warp each
    // sparse grids (a few atoms per cell) sort most cells a thread each;
    // dense ones (EAM: ~20 atoms per cell) leave every cell to the warps
    const bool sparse = n < 8 * m;
    int* big = nullptr;  // the queue of cells for the warps: the cell_fill array, free again after the scatter
    if (sparse) {
        big = c->cell_fill;
        k_zero_ints<<<1, 32, 0, s>>>(1, big, big);
        k_cell_sort_small<<<grid_for(m, 256), 256, 0, s>>>(m, c->cell_start, c->perm, c->d_cell_rep, rflag, big);
        c->launches += 2;
    }
    k_cell_sort_warp<<<std::min(grid_for(m, 8), 16 * c->num_sms), 256, 0, s>>>(
        m, c->cell_start, c->perm, sparse ? CELL_SORT_SMALL : 1, c->d_cell_rep, rflag, big);
    c->launches += 7;
    AtomArrays cur{c->x, c->y, c->z, c->vx, c->vy, c->vz, c->type, c->id, c->aflag, c->extra, c->extra_n};
    AtomArrays stg{c->stage_d, c->stage_d + c->cap, c->stage_d + 2 * (size_t)c->cap, c->stage_d + 3 * (size_t)c->cap,
                   c->stage_d + 4 * (size_t)c->cap, c->stage_d + 5 * (size_t)c->cap, c->stage_i,
                   c->stage_i + c->cap, reinterpret_cast<unsigned*>(c->stage_i + 2 * (size_t)c->cap),
                   c->stage_extra, c->extra_n};
    int* cell_sorted = c->cell_sorted;
    k_permute_gather<<<grid_for(n, 256), 256, 0, s>>>(n, c->perm, cur, stg, c->cell, cell_sorted, c->inv,
                                                      c->d_rep_of, rflag);
    k_permute_copyback<<<grid_for(n, 256), 256, 0, s>>>(n, stg, cur, c->d_rep_of, rflag);
    c->launches += 2;
    prof_end(c);
    prof_begin(c, "pack");
    LocFrame lf;
    for (int d = 0; d < 3; d++) {
        lf.nc[d] = g.nc[d];
        lf.h[d] = (float)g.h[d];
        lf.base[d] = (float)(g.org[d] - c->box.org[d] + c->box.P[d]);
    }
    unsigned* umax = reinterpret_cast<unsigned*>(c->d_flags + 3);
    k_zero_ints<<<1, 32, 0, s>>>(1, c->d_flags + 3, c->d_flags + 3);
    const RepGeom* rg = reps ? static_cast<const RepGeom*>(c->d_rep_geom) : nullptr;
    k_pack<<<grid_for(n, 256), 256, 0, s>>>(n, c->x, c->y, c->z, c->type, pack_frame(c), c->pack, c->xref,
                                            cell_sorted, lf, reps ? c->d_rep_of : nullptr, rg,
                                            c->flags_used ? c->aflag : nullptr, c->loc, umax, rflag);
    c->launches += 2;
    prof_end(c);

    BuildParams bp;
    bp.to = TileOut{};
    // tile slots: prepared per tile after the scan, written by the cell-local build
    const bool tiles = c->tile_want && !reps && c->tslot && c->tile_stride >= c->maxnb;
    if (tiles) {
        TilePrep tp;
        for (int d = 0; d < 3; d++) {
            tp.T[d] = c->tile_dim[d];
            tp.nt[d] = c->tile_nt[d];
            tp.nc[d] = g.nc[d];
            tp.periodic[d] = g.periodic[d];
            tp.corg[d] = g.org[d];
            tp.h[d] = g.h[d];
            tp.borg[d] = c->box.org[d];
            tp.P[d] = c->box.P[d];
        }
        tp.hx = tp.T[0] + 2;
        tp.hy = tp.T[1] + 2;
        tp.HC = c->tile_hc;
        k_tile_prep<<<c->tile_count, TILE_PREP_THREADS, 0, s>>>(tp, c->cell_start, c->tile_sb, c->tile_nst,
                                                                c->tile_org);
        c->launches++;
        bp.to.slot = c->tslot;
        bp.to.sb = c->tile_sb;
        bp.to.nst = c->tile_nst;
        for (int d = 0; d < 3; d++) {
            bp.to.T[d] = tp.T[d];
            bp.to.nt[d] = tp.nt[d];
        }
        bp.to.hx = tp.hx;
        bp.to.hy = tp.hy;
        bp.to.HC = tp.HC;
        bp.to.stride = c->tile_stride;
        bp.to.cap = c->tile_cap;
    }
    c->tile_valid = tiles;
    bp.n = n;
    bp.maxnb = c->maxnb;
    bp.hshift = c->nbr_hshift;
    for (int d = 0; d < 3; d++) {
        bp.nc[d] = g.nc[d];
        bp.periodic[d] = g.periodic[d];
        bp.L64[d] = g.L[d];
    }
    bp.L = make_shift(c->box);
    double rv = c->rc_max + c->skin;
    bp.rsq = rv * rv;
    bp.rsq_lo = (float)(bp.rsq * (1.0 - 2e-5));
    bp.rsq_hi = (float)(bp.rsq * (1.0 + 2e-5));
    bp.rv = (float)rv;
    bp.hmax = 0.f;
    for (int d = 0; d < 3; d++) {
        bp.base[d] = lf.base[d];
        bp.h[d] = lf.h[d];
        bp.hmax = fmaxf(bp.hmax, lf.h[d]);
    }
    if (reps) bp.hmax = (float)c->rep_hmax;
    prof_begin(c, "nlist_build");
    int combos = 1;
    for (int d = 0; d < 3; d++) combos *= (g.periodic[d] && g.nc[d] < 3) ? 3 * g.nc[d] : 3;
    // the cell-local builds also write each row's type mask
    c->nbmask_valid = reps || c->flags_used || tiles || !(c->build_lanes == 0 && combos <= 64 && !sparse) &&
                                                   c->build_lanes != 8 && c->build_lanes != 4;
    if (reps) {
        k_build<true><<<grid_for(n, 128), 128, 0, s>>>(bp, rg, c->d_rep_of, c->loc, c->x, c->y, c->z, cell_sorted,
                                                       c->cell_start, umax, reinterpret_cast<unsigned*>(c->nbr),
                                                       c->nnb, c->d_status, c->d_flags + 1, rflag, c->nbmask);
    } else if (tiles) {  // only the cell-local build writes tile slots
        k_build<false, true><<<grid_for(n, 128), 128, 0, s>>>(bp, nullptr, nullptr, c->loc, c->x, c->y, c->z,
                                                              cell_sorted, c->cell_start, umax,
                                                              reinterpret_cast<unsigned*>(c->nbr), c->nnb,
                                                              c->d_status, c->d_flags + 1, nullptr, c->nbmask);
    } else if (c->flags_used) {  // only the cell-local build skips inactive atoms
        k_build<false><<<grid_for(n, 128), 128, 0, s>>>(bp, nullptr, nullptr, c->loc, c->x, c->y, c->z,
                                                        cell_sorted, c->cell_start, umax,
                                                        reinterpret_cast<unsigned*>(c->nbr), c->nnb, c->d_status,
                                                        c->d_flags + 1, nullptr, c->nbmask);
    } else if (c->build_lanes == 0 && combos <= 64 && !sparse) {  // a cell CTA wants >= 8 atoms per cell
        const int cap = 1024;  // staged candidates per chunk (32 bytes each)
        k_build_cells<<<m, BUILD_CELL_THREADS, cap * 2 * sizeof(float4), s>>>(
            bp, c->pack, c->x, c->y, c->z, c->cell_start, cap, reinterpret_cast<unsigned*>(c->nbr), c->nnb,
            c->d_status, c->d_flags + 1);
    } else if (c->build_lanes == 8) {
        k_build_lanes<8><<<grid_for(n, 256 / 8), 256, 0, s>>>(bp, c->pack, c->x, c->y, c->z, cell_sorted,
                                                               c->cell_start, reinterpret_cast<unsigned*>(c->nbr),
                                                               c->nnb, c->d_status, c->d_flags + 1);
    } else if (c->build_lanes == 4) {
        k_build_lanes<4><<<grid_for(n, 256 / 4), 256, 0, s>>>(bp, c->pack, c->x, c->y, c->z, cell_sorted,
                                                               c->cell_start, reinterpret_cast<unsigned*>(c->nbr),
                                                               c->nnb, c->d_status, c->d_flags + 1);
    } else {
        k_build<false><<<grid_for(n, 128), 128, 0, s>>>(bp, nullptr, nullptr, c->loc, c->x, c->y, c->z,
                                                        cell_sorted, c->cell_start, umax,
                                                        reinterpret_cast<unsigned*>(c->nbr), c->nnb, c->d_status,
                                                        c->d_flags + 1, nullptr, c->nbmask);
    }
    c->launches++;
    if (c->build_in_step) {
        k_halt_on_overflow<<<1, 1, 0, s>>>(c->d_status, step_state_halted(c));
        c->launches++;
    }

    prof_end(c);
    if (c->need_rev) {
        prof_begin(c, "nlist_reverse");
        k_reverse<<<grid_for(n, 128 / REV_LANES), 128, 0, s>>>(n, c->nbr_hshift, c->maxnb,
                                                   reinterpret_cast<const unsigned*>(c->nbr), c->nnb, c->rev,
                                                   c->d_status, c->d_rep_of, rflag);
        c->launches++;
        prof_end(c);
    }
    if (reps) {
        k_rep_build_done<<<grid_for(c->nrep, 256), 256, 0, s>>>(c->nrep, rflag ? 0 : 1, c->d_rep_flag,
                                                                 c->d_rep_builds);
        c->launches++;
    }
    c->rebuilds++;
    c->list_valid = true;
    c->steps_since_build = 0;
    return check_cuda(c, cudaGetLastError(), "neighbour build");
}

}  // namespace omdg
