// omdg_count_neighbors_static: per-atom neighbour counts within a cutoff for
// positions that live in the caller's device memory, with no device
// allocation of any kind.
//
// It is the linked-cell counting sort of the neighbour-list build (cell
// assignment, exclusive scan of the cell counts, scatter into cell order)
// followed by a 27-cell count, but every scratch array (cell counts, fill
// counters, cell starts, per-atom cell index, cell-ordered atom index) sits in
// one file-scope __device__ array of fixed size.  Its address is looked up
// once per device with cudaGetSymbolAddress, the first time the entry point
// runs on that device.  Distances follow the list build exactly: the image of
// j is x_j + s L in FP64, r^2 = (dx dx + dy dy) + dz dz, and a pair counts when
// r^2 <= rcut^2 (VerletList.cpp:161), so the counts equal the per-atom
// neighbour counts of the list omdg_build_neighbors makes with Rv = rcut.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <mutex>

#include "../../include/omdg.h"

namespace {

constexpr int SC_MAX_ATOMS = OMDG_STATIC_MAX_ATOMS;
constexpr int SC_MAX_CELLS = OMDG_STATIC_MAX_CELLS;
constexpr int SC_MAX_DEVICES = 64;
constexpr int SC_SCAN_THREADS = 1024;
constexpr int SC_SCAN_PER_THREAD = SC_MAX_CELLS / SC_SCAN_THREADS;
static_assert(SC_MAX_CELLS % SC_SCAN_THREADS == 0, "scan covers the cell limit exactly");

// Scratch layout, in ints:
//   [0, C)             cell counts     (zeroed by every call before use)
//   [C, 2C)            fill counters   (zeroed by every call before use)
//   [2C, 3C+1)         cell starts     (written by the scan)
//   [3C+1, 3C+1+N)     cell of each atom
//   [3C+1+N, 3C+1+2N)  atoms in cell order
// with C = SC_MAX_CELLS and N = SC_MAX_ATOMS: 1,441,796 bytes.
constexpr size_t SC_COUNT = 0;
constexpr size_t SC_FILL = SC_MAX_CELLS;
constexpr size_t SC_START = 2 * (size_t)SC_MAX_CELLS;
constexpr size_t SC_CELL_OF = 3 * (size_t)SC_MAX_CELLS + 1;
constexpr size_t SC_SORTED = SC_CELL_OF + SC_MAX_ATOMS;
constexpr size_t SC_INTS = SC_SORTED + SC_MAX_ATOMS;

__device__ __align__(256) int g_scratch[SC_INTS];

int* g_scratch_addr[SC_MAX_DEVICES];
std::mutex g_scratch_mu;

struct SCGeom {
    int n;
    int nc[3];
    int periodic[3];
    double lo[3], L[3];
    double scale[3];  // nc / L
    double rsq;
};

__device__ __forceinline__ double sc_wrap(double x, double lo, double L, int periodic) {
    if (!periodic) return x;
    return __dsub_rn(x, __dmul_rn(floor(__ddiv_rn(__dsub_rn(x, lo), L)), L));
}

__device__ __forceinline__ int sc_cell_axis(double w, double lo, double scale, int nc) {
    int c = (int)floor(__dmul_rn(__dsub_rn(w, lo), scale));
    return min(max(c, 0), nc - 1);
}

__global__ void k_sc_clear(int ncells, int* __restrict__ scratch) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ncells; k += gridDim.x * blockDim.x) {
        scratch[SC_COUNT + k] = 0;
        scratch[SC_FILL + k] = 0;
    }
}

__global__ void k_sc_assign(SCGeom g, const double* __restrict__ x, int* __restrict__ scratch) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    int c[3];
    for (int d = 0; d < 3; d++) {
        const double w = sc_wrap(x[3 * (size_t)i + d], g.lo[d], g.L[d], g.periodic[d]);
        c[d] = sc_cell_axis(w, g.lo[d], g.scale[d], g.nc[d]);
    }
    const int cell = (c[2] * g.nc[1] + c[1]) * g.nc[0] + c[0];
    scratch[SC_CELL_OF + i] = cell;
    atomicAdd(&scratch[SC_COUNT + cell], 1);
}

// One block: exclusive scan of the cell counts into the cell starts.
__global__ void __launch_bounds__(SC_SCAN_THREADS) k_sc_scan(int ncells, int* __restrict__ scratch) {
    __shared__ int warp_sum[SC_SCAN_THREADS / 32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int b0 = t * SC_SCAN_PER_THREAD;
    int local = 0;
    for (int k = 0; k < SC_SCAN_PER_THREAD; k++)
        if (b0 + k < ncells) local += scratch[SC_COUNT + b0 + k];
    int incl = local;
    for (int off = 1; off < 32; off <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, off);
        if (lane >= off) incl += v;
    }
    if (lane == 31) warp_sum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int w = warp_sum[lane];
        for (int off = 1; off < 32; off <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += v;
        }
        warp_sum[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    int run = incl - local + (warp > 0 ? warp_sum[warp - 1] : 0);
    for (int k = 0; k < SC_SCAN_PER_THREAD; k++) {
        if (b0 + k < ncells) {
            scratch[SC_START + b0 + k] = run;
            run += scratch[SC_COUNT + b0 + k];
        }
    }
    if (t == SC_SCAN_THREADS - 1) scratch[SC_START + ncells] = warp_sum[31];
}

__global__ void k_sc_scatter(int n, int* __restrict__ scratch) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int cell = scratch[SC_CELL_OF + i];
    const int slot = scratch[SC_START + cell] + atomicAdd(&scratch[SC_FILL + cell], 1);
    scratch[SC_SORTED + slot] = i;
}

// One thread per atom, taken in cell order so that a warp reads the same
// stencil cells.  With at least 3 cells on each periodic axis the 27 stencil
// cells are distinct, so every image pair is seen once.
__global__ void __launch_bounds__(128) k_sc_count(SCGeom g, const double* __restrict__ x,
                                                  const int* __restrict__ scratch, int* __restrict__ count) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n) return;
    const int i = scratch[SC_SORTED + t];
    const int cell = scratch[SC_CELL_OF + i];
    const int c0 = cell % g.nc[0], c1 = (cell / g.nc[0]) % g.nc[1], c2 = cell / (g.nc[0] * g.nc[1]);
    const double xi = sc_wrap(x[3 * (size_t)i], g.lo[0], g.L[0], g.periodic[0]);
    const double yi = sc_wrap(x[3 * (size_t)i + 1], g.lo[1], g.L[1], g.periodic[1]);
    const double zi = sc_wrap(x[3 * (size_t)i + 2], g.lo[2], g.L[2], g.periodic[2]);
    int found = 0;
    for (int dz = -1; dz <= 1; dz++) {
        int cz = c2 + dz, sz = 0;
        if (cz < 0 || cz >= g.nc[2]) {
            if (!g.periodic[2]) continue;
            sz = cz < 0 ? -1 : 1;
            cz -= sz * g.nc[2];
        }
        const double gz = sz == 0 ? 0.0 : (sz > 0 ? g.L[2] : -g.L[2]);
        for (int dy = -1; dy <= 1; dy++) {
            int cy = c1 + dy, sy = 0;
            if (cy < 0 || cy >= g.nc[1]) {
                if (!g.periodic[1]) continue;
                sy = cy < 0 ? -1 : 1;
                cy -= sy * g.nc[1];
            }
            const double gy = sy == 0 ? 0.0 : (sy > 0 ? g.L[1] : -g.L[1]);
            for (int dx = -1; dx <= 1; dx++) {
                int cx = c0 + dx, sx = 0;
                if (cx < 0 || cx >= g.nc[0]) {
                    if (!g.periodic[0]) continue;
                    sx = cx < 0 ? -1 : 1;
                    cx -= sx * g.nc[0];
                }
                const double gx = sx == 0 ? 0.0 : (sx > 0 ? g.L[0] : -g.L[0]);
                const int nb = (cz * g.nc[1] + cy) * g.nc[0] + cx;
                const bool home = sx == 0 && sy == 0 && sz == 0;
                const int k0 = scratch[SC_START + nb], k1 = scratch[SC_START + nb + 1];
                for (int k = k0; k < k1; k++) {
                    const int j = scratch[SC_SORTED + k];
                    if (home && j == i) continue;
                    const double xj = sc_wrap(x[3 * (size_t)j], g.lo[0], g.L[0], g.periodic[0]);
                    const double yj = sc_wrap(x[3 * (size_t)j + 1], g.lo[1], g.L[1], g.periodic[1]);
                    const double zj = sc_wrap(x[3 * (size_t)j + 2], g.lo[2], g.L[2], g.periodic[2]);
                    const double ex = __dsub_rn(xi, __dadd_rn(xj, gx));
                    const double ey = __dsub_rn(yi, __dadd_rn(yj, gy));
                    const double ez = __dsub_rn(zi, __dadd_rn(zj, gz));
                    const double rr =
                        __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
                    found += rr <= g.rsq;
                }
            }
        }
    }
    count[i] = found;
}

int sc_fail(char* err, int err_len, int code, const char* fmt, ...) {
    if (err && err_len > 0) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(err, (size_t)err_len, fmt, ap);
        va_end(ap);
    }
    return code;
}

}  // namespace

extern "C" int omdg_count_neighbors_static(const double* x, int n, const double lo[3], const double hi[3],
                                           const int periodic[3], double rcut, int* count, void* stream, char* err,
                                           int err_len) {
    if (err && err_len > 0) err[0] = '\0';
    if (n < 0 || !lo || !hi || !periodic) return sc_fail(err, err_len, OMDG_EINVAL, "invalid arguments");
    if (n > SC_MAX_ATOMS)
        return sc_fail(err, err_len, OMDG_ERANGE, "%d atoms exceed the static scratch limit of %d atoms", n,
                       SC_MAX_ATOMS);
    if (n > 0 && (!x || !count)) return sc_fail(err, err_len, OMDG_EINVAL, "null position or count pointer");
    if (!(rcut > 0.0) || !std::isfinite(rcut)) return sc_fail(err, err_len, OMDG_EINVAL, "rcut must be positive");
    SCGeom g;
    g.n = n;
    for (int d = 0; d < 3; d++) {
        g.lo[d] = lo[d];
        g.L[d] = hi[d] - lo[d];
        g.periodic[d] = periodic[d] ? 1 : 0;
        if (!(g.L[d] > 0.0) || !std::isfinite(g.L[d]))
            return sc_fail(err, err_len, OMDG_EINVAL, "box axis %d has no positive length", d);
        // cells no narrower than rcut, with a margin for the rounding of (x - lo) nc / L
        const double fit = std::floor(g.L[d] / (rcut * (1.0 + 1e-12)));
        g.nc[d] = (int)std::min(fit, 1024.0);
        if (g.periodic[d] && g.nc[d] < 3)
            return sc_fail(err, err_len, OMDG_EINVAL,
                           "periodic axis %d is not longer than 3 rcut (%.17g vs %.17g): too small for the static path",
                           d, g.L[d], 3.0 * rcut);
        if (g.nc[d] < 1) g.nc[d] = 1;
    }
    // coarsen the widest axis until the grid fits the scratch (wider cells stay correct)
    while ((long long)g.nc[0] * g.nc[1] * g.nc[2] > SC_MAX_CELLS) {
        int d = 0;
        for (int e = 1; e < 3; e++)
            if (g.nc[e] > g.nc[d]) d = e;
        g.nc[d] = std::max(g.periodic[d] ? 3 : 1, g.nc[d] * 3 / 4);
    }
    for (int d = 0; d < 3; d++) g.scale[d] = g.nc[d] / g.L[d];
    g.rsq = rcut * rcut;
    const int ncells = g.nc[0] * g.nc[1] * g.nc[2];
    if (n == 0) return OMDG_OK;

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return sc_fail(err, err_len, OMDG_ECUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= SC_MAX_DEVICES)
        return sc_fail(err, err_len, OMDG_EINVAL, "device %d is beyond the %d devices the static path tracks", dev,
                       SC_MAX_DEVICES);
    int* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mu);
        if (!g_scratch_addr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_scratch);
            if (e != cudaSuccess)
                return sc_fail(err, err_len, OMDG_ECUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
            g_scratch_addr[dev] = static_cast<int*>(p);
        }
        scratch = g_scratch_addr[dev];
    }

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int blocks = (n + 255) / 256;
    k_sc_clear<<<(ncells + 255) / 256, 256, 0, s>>>(ncells, scratch);
    k_sc_assign<<<blocks, 256, 0, s>>>(g, x, scratch);
    k_sc_scan<<<1, SC_SCAN_THREADS, 0, s>>>(ncells, scratch);
    k_sc_scatter<<<blocks, 256, 0, s>>>(n, scratch);
    k_sc_count<<<(n + 127) / 128, 128, 0, s>>>(g, x, scratch, count);
    e = cudaGetLastError();
    if (e != cudaSuccess) return sc_fail(err, err_len, OMDG_ECUDA, "launch: %s", cudaGetErrorString(e));
    return OMDG_OK;
}
