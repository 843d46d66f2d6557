// Local thermodynamics (ThermoDetector, include/detect/ThermoDetector.h) and
// the homogeneous scaling-corrected two-temperature model (TTM_Homogen,
// include/misc/TTM_Homogen_SCNA.h) on the device.
//
// Detector, after every step (ExtractTemperature, ThermoDetector.h:176-237),
// over each atom and its list neighbours within ercut:
//   k_thermo_cm     v_cm_i = sum m_j v_j / sum m_j, n_i = 1 + neighbours
//   k_thermo_temp   T_i = 2/(3 k_B) 1/2 sum m_j |v_j - v_cm_j|^2 / n_i,
//                   density n_i / (4/3 pi ercut^3); block partials of the
//                   averages (atoms with n_i >= 2), kinetic energy, max v^2
//   k_thermo_final  one block, fixed order
// TTM, before the kick-drift of every step (PreIntegration, :337-376):
//   k_ttm_fd        one thread: electron temperature step (fd_main_loop, :232-263)
//   k_ttm_scale     rescaling about the local centre of mass (velocity_scalling, :272-330)
//   k_ttm_sum       one block: integrated lattice energy
// Distances as CalcDistance: an FP32 screen from the position packs, and
// sqrt((dx dx + dy dy) + dz dz) <= ercut in FP64 near the edge.
#include <cfloat>
#include <cmath>
#include <string>

#include "device_common.cuh"
#include "fdtd_internal.h"

namespace omdg {

constexpr int TH_BLOCK = 128;

struct TTMState {
    double te, int_een, int_aen, n_zero, coup;
    double t_avg, d_avg, kin, vmax2, elapsed;
    int firstfd, active, navg, pad;
};

struct ThermoParams {
    int n, hshift, maxnb;
    ShiftF L;
    double L64[3];
    double rc, rc2;
    float rc2_lo, rc2_hi;
    double volcut, fac;
};

struct TTMCtx {
    bool ttm = false;
    HostTable g, ce;
    DevTable dg{}, dce{};
    double4_32a* coef64[2] = {nullptr, nullptr};
    double g0 = 0, c0 = 0, vol = 0, te0 = -1, offset = 0;
    double ercut = -1;                  // <= 0: the largest cutoff of the force kernels
    double *vcm = nullptr, *temp = nullptr, *dens = nullptr;  // 3n, n, n
    int* nneig = nullptr;
    double* partial = nullptr;          // per block: T, dens, count, kinetic, max v^2; + scale partials
    TTMState* st = nullptr;
    int cap = 0, nblocks = 0;
    // diffusing electron temperature: the cells of a finite-difference grid
    omdg_fdtd* grid = nullptr;
    double org[3] = {0, 0, 0};
    unsigned long long* cell_sum = nullptr;  // per cell: lattice temperatures x 2^20
    int* cell_cnt = nullptr;                 // per cell: atoms counted
    int* dev_ctr = nullptr;                  // [0] solves done, [1] the model active in this step
};

// Within ercut: the FP32 screen, and the reference's FP64 distance in the band.
__device__ __forceinline__ bool th_within(const ThermoParams& p, const PosPack& pi, const PosPack& pj, unsigned e,
                                          int i, int j, const double* __restrict__ x, const double* __restrict__ y,
                                          const double* __restrict__ z) {
    const float3 d = pair_delta(pi.hi, pi.lo, pj.hi, pj.lo, e, p.L);
    const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
    if (r2 > p.rc2_hi) return false;
    if (r2 < p.rc2_lo) return true;
    const int sx = nbr_sx(e), sy = nbr_sy(e), sz = nbr_sz(e);
    const double gx = sx == 0 ? 0.0 : (sx > 0 ? p.L64[0] : -p.L64[0]);
    const double gy = sy == 0 ? 0.0 : (sy > 0 ? p.L64[1] : -p.L64[1]);
    const double gz = sz == 0 ? 0.0 : (sz > 0 ? p.L64[2] : -p.L64[2]);
    const double dx = __dsub_rn(x[i], __dadd_rn(x[j], gx));
    const double dy = __dsub_rn(y[i], __dadd_rn(y[j], gy));
    const double dz = __dsub_rn(z[i], __dadd_rn(z[j], gz));
    return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz))) <= p.rc;
}

__global__ void __launch_bounds__(TH_BLOCK) k_thermo_cm(ThermoParams p, const PosPack* __restrict__ pack,
                                                        const unsigned* __restrict__ nbr,
                                                        const int* __restrict__ nnb, const double* __restrict__ x,
                                                        const double* __restrict__ y, const double* __restrict__ z,
                                                        const double* __restrict__ vx, const double* __restrict__ vy,
                                                        const double* __restrict__ vz, const int* __restrict__ type,
                                                        const double* __restrict__ mass, double* __restrict__ vcm,
                                                        int* __restrict__ nneig) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const PosPack pi = pack[i];
    double ms = mass[type[i]];
    double px = ms * vx[i], py = ms * vy[i], pz = ms * vz[i];
    int cnt = 1;
    const int m = nnb[i];
    for (int s = 0; s < m; s++) {
        const unsigned e = nbr[nbr_at(i, s, p.hshift, p.maxnb)];
        const int j = nbr_index(e);
        if (!th_within(p, pi, pack[j], e, i, j, x, y, z)) continue;
        const double mj = mass[type[j]];
        ms += mj;
        px = fma(mj, vx[j], px);
        py = fma(mj, vy[j], py);
        pz = fma(mj, vz[j], pz);
        cnt++;
    }
    vcm[i] = px / ms;
    vcm[p.n + i] = py / ms;
    vcm[2 * (size_t)p.n + i] = pz / ms;
    nneig[i] = cnt;
}

__device__ __forceinline__ double th_ek(int j, const double* __restrict__ vx, const double* __restrict__ vy,
                                        const double* __restrict__ vz, const double* __restrict__ vcm, int n,
                                        double mj) {
    const double cx = vx[j] - vcm[j], cy = vy[j] - vcm[n + j], cz = vz[j] - vcm[2 * (size_t)n + j];
    return mj * (cx * cx + cy * cy + cz * cz);
}

// Block partials of the detector, per block TH_Q doubles: 0 sum T_i, 1 sum
// n_i, 2 count (atoms with n_i >= 2), 3 sum m v^2 (every atom), 4 max v^2
// (the two-temperature model's); over active atoms (MeasureSystemTempPres,
// ExtractPressure): 5-7 sum m v, 8 sum m, 9 sum m v^2, 10 sum virial, 11 sum
// local pressure, 12 count, 13-15 min x y z, 16-18 max x y z.
constexpr int TH_Q = 19;
constexpr double TH_GPA = 160.22;  // MD_GIGAPASCAL (conversion.h:39)

__device__ __forceinline__ bool th_is_max(int q) { return q == 4 || q >= 16; }
__device__ __forceinline__ bool th_is_min(int q) { return q >= 13 && q < 16; }

__device__ __forceinline__ double th_combine(int q, double a, double b) {
    return th_is_max(q) ? fmax(a, b) : (th_is_min(q) ? fmin(a, b) : a + b);
}

__global__ void __launch_bounds__(TH_BLOCK) k_thermo_temp(
    ThermoParams p, const PosPack* __restrict__ pack, const unsigned* __restrict__ nbr, const int* __restrict__ nnb,
    const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
    const double* __restrict__ vx, const double* __restrict__ vy, const double* __restrict__ vz,
    const int* __restrict__ type, const double* __restrict__ mass, const double* __restrict__ vcm,
    const int* __restrict__ nneig, const float* __restrict__ vir, const unsigned* __restrict__ aflag,
    double* __restrict__ temp, double* __restrict__ dens, double* __restrict__ partial) {
    __shared__ double st[TH_Q][TH_BLOCK];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double q[TH_Q];
    for (int k = 0; k < TH_Q; k++) q[k] = th_is_max(k) && k != 4 ? -DBL_MAX : (th_is_min(k) ? DBL_MAX : 0.0);
    if (i < p.n) {
        const PosPack pi = pack[i];
        const double mi = mass[type[i]];
        double sum = th_ek(i, vx, vy, vz, vcm, p.n, mi);
        const int m = nnb[i];
        for (int s = 0; s < m; s++) {
            const unsigned e = nbr[nbr_at(i, s, p.hshift, p.maxnb)];
            const int j = nbr_index(e);
            if (!th_within(p, pi, pack[j], e, i, j, x, y, z)) continue;
            sum += th_ek(j, vx, vy, vz, vcm, p.n, mass[type[j]]);
        }
        const int nn = nneig[i];
        const double t = p.fac * (0.5 * sum / (double)nn);
        const double dn = (double)nn / p.volcut;
        temp[i] = t;
        dens[i] = dn;
        const bool active = !aflag || (aflag[i] & 1u);
        if (nn >= 2 && active) {
            q[0] = t;
            q[1] = dn;
            q[2] = 1.0;
        }
        const double v2 = vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i];
        q[3] = mi * v2;
        q[4] = v2;
        if (active) {
            q[5] = mi * vx[i];
            q[6] = mi * vy[i];
            q[7] = mi * vz[i];
            q[8] = mi;
            q[9] = mi * v2;
            q[10] = (double)vir[i];
            // a_i = Unit->Pressure(n_i virial_i / 6 + sumek_i / (3 V)), sumek_i = 2 T_i n_i / fac
            q[11] = TH_GPA * dn * ((double)vir[i] / 6.0 + 2.0 * t / (3.0 * p.fac));
            q[12] = 1.0;
            q[13] = q[16] = x[i];
            q[14] = q[17] = y[i];
            q[15] = q[18] = z[i];
        }
    }
    for (int k = 0; k < TH_Q; k++) st[k][threadIdx.x] = q[k];
    __syncthreads();
    for (int off = TH_BLOCK / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off)
            for (int k = 0; k < TH_Q; k++)
                st[k][threadIdx.x] = th_combine(k, st[k][threadIdx.x], st[k][threadIdx.x + off]);
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < TH_Q; k++) partial[TH_Q * (size_t)blockIdx.x + k] = st[k][0];
}

// The detector's totals (one block, fixed order).  With a ledger row, its
// columns 8-11 take SysMonitor's temp:, avtemp:, pres:, avpres: slots
// (ThermoDetector.h:118-127): the system temperature about the
// centre-of-mass velocity and pressure over the active atoms' bounding box
// (MeasureSystemTempPres, :329-420), the average local temperature and
// pressure.
__global__ void k_thermo_final(int nblocks, const double* __restrict__ partial, TTMState* st, double fac,
                               double* ledger, int ledger_cap, const int* row, int shift) {
    __shared__ double red[TH_Q][256];
    double a[TH_Q];
    for (int k = 0; k < TH_Q; k++) a[k] = th_is_max(k) && k != 4 ? -DBL_MAX : (th_is_min(k) ? DBL_MAX : 0.0);
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
        for (int k = 0; k < TH_Q; k++) a[k] = th_combine(k, a[k], partial[TH_Q * (size_t)b + k]);
    for (int k = 0; k < TH_Q; k++) red[k][threadIdx.x] = a[k];
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off)
            for (int k = 0; k < TH_Q; k++) red[k][threadIdx.x] = th_combine(k, red[k][threadIdx.x], red[k][threadIdx.x + off]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double cnt = red[2][0];
        st->t_avg = cnt > 0.0 ? red[0][0] / cnt : 0.0;
        st->d_avg = cnt > 0.0 ? red[1][0] / cnt : 0.0;
        st->navg = (int)cnt;
        st->kin = 0.5 * red[3][0];
        st->vmax2 = red[4][0];
        if (ledger) {
            // the row of the step just completed (shift 1), or of the
            // measurement that does not advance the step (shift 0)
            double* ledger_row = ledger + LEDGER_W * (size_t)(((*row - shift) % ledger_cap + ledger_cap) % ledger_cap);
            const double msum = red[8][0], nact = red[12][0];
            double twoek = red[9][0];  // sum m |v - v_cm|^2 = sum m v^2 - |sum m v|^2 / M
            if (msum > 0.0)
                twoek -= (red[5][0] * red[5][0] + red[6][0] * red[6][0] + red[7][0] * red[7][0]) / msum;
            double vol = 1.0;
            for (int d = 0; d < 3; d++) {
                const double ext = red[16 + d][0] - red[13 + d][0];
                vol *= ext > 0.0 ? ext : 1.0;
            }
            ledger_row[8] = nact > 0.0 ? fac * 0.5 * twoek / nact : 0.0;
            ledger_row[9] = st->t_avg;
            ledger_row[10] = TH_GPA * (0.5 * red[10][0] + twoek) / (3.0 * vol);
            ledger_row[11] = nact > 0.0 ? red[11][0] / nact : 0.0;
        }
    }
}

struct TTMParams {
    DevTable g, ce;
    double g0, c0, vol, te0, offset, dt;
    int natoms;
};

__global__ void k_ttm_fd(TTMParams p, TTMState* st, unsigned* status) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const bool active = st->elapsed > p.offset;
    st->active = active ? 1 : 0;
    st->elapsed += p.dt;
    if (!active) return;
    const double ta = st->t_avg;
    double v, dv;
    if (st->firstfd) {
        if (st->te < 0.0) st->te = ta;
        tab_read64(p.ce, st->te, v, dv, status);
        st->int_een = 0.5 * st->te * p.c0 * v * p.vol;
        st->int_aen = 2.0 * st->kin / p.natoms;
        st->n_zero = st->d_avg;
        st->firstfd = 0;
    }
    tab_read64(p.g, st->te, v, dv, status);
    const double de = -p.g0 * v * (st->te - ta) * p.dt;
    st->int_een += de * p.vol;
    tab_read64(p.ce, st->te, v, dv, status);
    st->te += de / (p.c0 * v);
    tab_read64(p.g, st->te, v, dv, status);
    st->coup = p.g0 * v;
}

// The rescaling of one atom about its local centre-of-mass velocity, given
// the energy e it receives (velocity_scalling, TTM_Homogen_SCNA.h:294-320).
// Returns true when the velocity changed.
__device__ __forceinline__ bool ttm_rescale(int i, int n, double e, double m, double small,
                                            double* __restrict__ vx, double* __restrict__ vy,
                                            double* __restrict__ vz, const double* __restrict__ vcm) {
    const double cmx = vcm[i], cmy = vcm[n + i], cmz = vcm[2 * (size_t)n + i];
    const double ux = vx[i], uy = vy[i], uz = vz[i];
    const double cx = ux - cmx, cy = uy - cmy, cz = uz - cmz;
    const double c2 = cx * cx + cy * cy + cz * cz;
    if (c2 < small) return false;
    const double cmc = cmx * cx + cmy * cy + cmz * cz;
    const double cm2 = cmx * cmx + cmy * cmy + cmz * cmz;
    const double v2 = ux * ux + uy * uy + uz * uz;
    const double rr = cmc * cmc + c2 * (2.0 * e / m + v2 - cm2);
    if (rr < 0.0) return false;
    const double sa = (-cmc + sqrt(rr)) / c2;
    vx[i] = cmx + sa * cx;
    vy[i] = cmy + sa * cy;
    vz[i] = cmz + sa * cz;
    return true;
}

__device__ __forceinline__ void ttm_block_partial(double de, double cnt, double* __restrict__ partial) {
    __shared__ double se[TH_BLOCK], sc[TH_BLOCK];
    se[threadIdx.x] = de;
    sc[threadIdx.x] = cnt;
    __syncthreads();
    for (int off = TH_BLOCK / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) {
            se[threadIdx.x] += se[threadIdx.x + off];
            sc[threadIdx.x] += sc[threadIdx.x + off];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[2 * (size_t)blockIdx.x] = se[0];
        partial[2 * (size_t)blockIdx.x + 1] = sc[0];
    }
}

__global__ void __launch_bounds__(TH_BLOCK) k_ttm_scale(TTMParams p, int n, double volcut,
                                                        const TTMState* __restrict__ st, double* __restrict__ vx,
                                                        double* __restrict__ vy, double* __restrict__ vz,
                                                        const int* __restrict__ type, const double* __restrict__ mass,
                                                        const double* __restrict__ vcm,
                                                        const double* __restrict__ temp,
                                                        const double* __restrict__ dens,
                                                        const unsigned* __restrict__ aflag,
                                                        double* __restrict__ partial) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double de = 0.0, cnt = 0.0;
    // inactive atoms are skipped (TTM_Homogen_SCNA.h:288)
    if (st->active && i < n && (!aflag || (aflag[i] & 1u)) && dens[i] * volcut > 3.0) {
        const double m = mass[type[i]];
        const double e = st->coup * (st->te - temp[i]) * p.vol * p.dt;
        if (ttm_rescale(i, n, e, m, st->vmax2 * 1e-12, vx, vy, vz, vcm)) {
            de = e;
            cnt = 1.0;
        }
    }
    ttm_block_partial(de, cnt, partial);
}

// ------------------------------------------------------------------ diffusing electron temperature
// The electron temperature lives on the cells of a finite-difference grid
// (FDTDSolver): per step, before the kick-drift,
//   k_ttm_grid_lattice  per atom: its detector temperature into its cell's
//                       sum (atoms counted as in the detector's average:
//                       active, at least two within ercut), as fixed-point
//                       integers so that the sums do not depend on order
//   k_ttm_grid_fd       per cell: Te (a negative Te at the first active step
//                       takes the cell's lattice temperature, as
//                       fd_main_loop does for the scalar, :238-241), the
//                       external vector E = -G0 G(Te) (Te - Ta) where the cell
//                       holds atoms, the capacity C0 Ce(Te), and the copy the
//                       solve reads
//   k_fd_solve          the grid's explicit step (csrc/fdtd.cu)
//   k_ttm_grid_scale    per atom: the rescaling with its cell's new Te and
//                       G0 G(Te), as velocity_scalling does with the scalar
//   k_ttm_sum           the integrated lattice energy
// With one periodic cell and no source this is the scalar model: the face
// terms are K (T - T) = 0, so A = Te + (E dt) / cap is fd_main_loop's
// Te + de / (C0 Ce(Te)), term for term.
constexpr double TTM_CELL_SCALE = 1048576.0;  // 2^20: lattice temperature fixed point

struct GridTTM {
    FDDev fd;
    double* A;   // cell vector (the solve writes it)
    double* T;   // the copy the solve reads
    double* cap;
    double org[3], h;
    int nx, ny, nz;
    int periodic[3];
    double lo[3], L[3];
    unsigned long long* sum;
    int* cnt;
    int* ctr;    // [0] solves done, [1] active in this step
};

// The grid cell of a position (periodic axes wrapped into the box first);
// -1 outside the grid.  A 2D grid (nz = 1) spans every z.
__device__ __forceinline__ int ttm_cell(const GridTTM& q, double x, double y, double z) {
    const double r[3] = {x, y, z};
    int c[3];
    for (int d = 0; d < 3; d++) {
        double w = r[d];
        if (q.periodic[d]) w -= floor((w - q.lo[d]) / q.L[d]) * q.L[d];
        c[d] = (int)floor((w - q.org[d]) / q.h);
    }
    if (q.nz == 1) c[2] = 0;
    if (c[0] < 0 || c[0] >= q.nx || c[1] < 0 || c[1] >= q.ny || c[2] < 0 || c[2] >= q.nz) return -1;
    return c[2] * q.nx * q.ny + c[0] + c[1] * q.nx;
}

__global__ void __launch_bounds__(TH_BLOCK) k_ttm_grid_lattice(GridTTM q, int n, const double* __restrict__ x,
                                                               const double* __restrict__ y,
                                                               const double* __restrict__ z,
                                                               const double* __restrict__ temp,
                                                               const int* __restrict__ nneig,
                                                               const unsigned* __restrict__ aflag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || nneig[i] < 2 || (aflag && !(aflag[i] & 1u))) return;
    const int c = ttm_cell(q, x[i], y[i], z[i]);
    if (c < 0) return;
    const double t = temp[i] > 0.0 ? temp[i] : 0.0;
    atomicAdd(&q.sum[c], (unsigned long long)llrint(t * TTM_CELL_SCALE));
    atomicAdd(&q.cnt[c], 1);
}

__global__ void __launch_bounds__(TH_BLOCK) k_ttm_grid_fd(TTMParams p, GridTTM q, TTMState* st, unsigned* status) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = st->elapsed > p.offset;
    if (c == 0) {
        q.ctr[1] = active ? 1 : 0;
        st->active = active ? 1 : 0;
        if (active && st->firstfd) {
            st->int_aen = 2.0 * st->kin / p.natoms;
            st->n_zero = st->d_avg;
        }
    }
    if (c >= q.fd.dim) return;
    const int cnt = q.cnt[c];
    const double ta = cnt > 0 ? ((double)q.sum[c] / TTM_CELL_SCALE) / (double)cnt : 0.0;
    q.sum[c] = 0ull;  // ready for the next step's sums
    q.cnt[c] = 0;
    if (!active) return;
    double te = q.A[c];
    if (st->firstfd && te < 0.0) te = ta;
    double v, dv;
    tab_read64(p.g, te, v, dv, status);
    q.fd.E[c] = cnt > 0 ? -p.g0 * v * (te - ta) : 0.0;
    tab_read64(p.ce, te, v, dv, status);
    q.cap[c] = p.c0 * v;
    q.T[c] = te;
}

__global__ void __launch_bounds__(TH_BLOCK) k_ttm_grid_scale(TTMParams p, GridTTM q, int n, double volcut,
                                                             TTMState* st, const double* __restrict__ x,
                                                             const double* __restrict__ y,
                                                             const double* __restrict__ z, double* __restrict__ vx,
                                                             double* __restrict__ vy, double* __restrict__ vz,
                                                             const int* __restrict__ type,
                                                             const double* __restrict__ mass,
                                                             const double* __restrict__ vcm,
                                                             const double* __restrict__ temp,
                                                             const double* __restrict__ dens,
                                                             const unsigned* __restrict__ aflag,
                                                             double* __restrict__ partial, unsigned* status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = q.ctr[1] != 0;
    double de = 0.0, cnt = 0.0;
    if (active && i < n && (!aflag || (aflag[i] & 1u)) && dens[i] * volcut > 3.0) {
        const int c = ttm_cell(q, x[i], y[i], z[i]);
        if (c >= 0) {
            const double te = q.A[c];
            double v, dv;
            tab_read64(p.g, te, v, dv, status);
            const double e = p.g0 * v * (te - temp[i]) * p.vol * p.dt;
            if (ttm_rescale(i, n, e, mass[type[i]], st->vmax2 * 1e-12, vx, vy, vz, vcm)) {
                de = e;
                cnt = 1.0;
            }
        }
    }
    ttm_block_partial(de, cnt, partial);
    if (i == 0) {  // the step's bookkeeping, after every reader of it
        st->elapsed += p.dt;
        if (active) {
            st->firstfd = 0;
            q.ctr[0] += 1;
        }
    }
}

__global__ void k_ttm_sum(int nblocks, const double* __restrict__ partial, TTMState* st) {
    __shared__ double se[256], sc[256];
    double e = 0.0, c = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
        e += partial[2 * (size_t)b];
        c += partial[2 * (size_t)b + 1];
    }
    se[threadIdx.x] = e;
    sc[threadIdx.x] = c;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) {
            se[threadIdx.x] += se[threadIdx.x + off];
            sc[threadIdx.x] += sc[threadIdx.x + off];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0 && st->active && sc[0] > 0.0) st->int_aen += se[0] / sc[0];
}

// ------------------------------------------------------------------ host
static int th_ensure(Context* c, TTMCtx& t) {
    if (t.cap >= c->n && t.st) return OMDG_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(c->stream, &cs);
    if (cs != cudaStreamCaptureStatusNone) return set_error(c, OMDG_ESTATE, "detector buffers missing in capture");
    cudaFree(t.vcm);
    cudaFree(t.temp);
    cudaFree(t.dens);
    cudaFree(t.nneig);
    cudaFree(t.partial);
    const size_t n = (size_t)std::max(c->cap, c->n);
    t.nblocks = grid_for((int)n, TH_BLOCK);
    cudaError_t e = cudaMalloc(&t.vcm, sizeof(double) * 3 * n);
    if (e == cudaSuccess) e = cudaMalloc(&t.temp, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMalloc(&t.dens, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMalloc(&t.nneig, sizeof(int) * n);
    if (e == cudaSuccess) e = cudaMalloc(&t.partial, sizeof(double) * TH_Q * t.nblocks);
    if (e == cudaSuccess && !t.st) {
        e = cudaMalloc(&t.st, sizeof(TTMState));
        TTMState h{};
        h.te = t.te0;
        h.firstfd = 1;
        if (e == cudaSuccess) e = cudaMemcpy(t.st, &h, sizeof(h), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) return set_error(c, OMDG_ENOMEM, "detector buffers");
    t.cap = (int)n;
    invalidate_graph(c);
    return OMDG_OK;
}

static ThermoParams th_params(const Context* c, const TTMCtx& t) {
    ThermoParams p;
    p.n = c->n;
    p.hshift = c->nbr_hshift;
    p.maxnb = c->maxnb;
    p.L = make_shift(c->box);
    for (int d = 0; d < 3; d++) p.L64[d] = c->box.periodic[d] ? c->box.L[d] : 0.0;
    p.rc = t.ercut > 0 ? t.ercut : c->rc_ref;
    p.rc2 = p.rc * p.rc;
    p.rc2_lo = (float)(p.rc2 * (1.0 - 2e-5));
    p.rc2_hi = (float)(p.rc2 * (1.0 + 2e-5));
    p.volcut = 4.0 * M_PI * p.rc * p.rc * p.rc / 3.0;
    p.fac = 2.0 / 3.0 / 8.61734279e-05;
    return p;
}

double thermo_ercut(const Context* c) {
    if (!c->ttm) return -1.0;
    return c->ttm->ercut > 0 ? c->ttm->ercut : c->rc_ref;
}

int thermo_detect(Context* c, bool after_step) {
    TTMCtx& t = *c->ttm;
    int rc = th_ensure(c, t);
    if (rc) return rc;
    const ThermoParams p = th_params(c, t);
    if (p.rc > c->rc_max + c->skin) return set_error(c, OMDG_EINVAL, "detector cutoff beyond the neighbour list");
    const unsigned* nbr = reinterpret_cast<const unsigned*>(c->nbr);
    const int g = grid_for(c->n, TH_BLOCK);
    prof_begin(c, "thermo_detector");
    k_thermo_cm<<<g, TH_BLOCK, 0, c->stream>>>(p, c->pack, nbr, c->nnb, c->x, c->y, c->z, c->vx, c->vy, c->vz,
                                                c->type, c->d_mass, t.vcm, t.nneig);
    k_thermo_temp<<<g, TH_BLOCK, 0, c->stream>>>(p, c->pack, nbr, c->nnb, c->x, c->y, c->z, c->vx, c->vy, c->vz,
                                                  c->type, c->d_mass, t.vcm, t.nneig, c->vir,
                                                  c->flags_used ? c->aflag : nullptr, t.temp, t.dens, t.partial);
    k_thermo_final<<<1, 256, 0, c->stream>>>(g, t.partial, t.st, p.fac, c->d_ledger, c->ledger_cap,
                                             step_state_row(c), after_step ? 1 : 0);
    prof_end(c);
    c->launches += 3;
    return check_cuda(c, cudaGetLastError(), "thermo detector");
}

int ttm_pre(Context* c) {
    TTMCtx& t = *c->ttm;
    int rc = th_ensure(c, t);
    if (rc) return rc;
    TTMParams p;
    p.g = t.dg;
    p.ce = t.dce;
    p.g0 = t.g0;
    p.c0 = t.c0;
    p.vol = t.vol;
    p.te0 = t.te0;
    p.offset = t.offset;
    p.dt = c->dt;
    p.natoms = c->n;
    const ThermoParams tp = th_params(c, t);
    const int g = grid_for(c->n, TH_BLOCK);
    const unsigned* aflag = c->flags_used ? c->aflag : nullptr;
    prof_begin(c, "ttm");
    if (t.grid) {
        FDGrid* fg = t.grid;
        GridTTM q;
        q.fd = fd_dev(fg);
        q.fd.dt = c->dt;  // the grid steps with the MD time step (fd_time_step, TTM_Homogen_SCNA.h:175)
        q.fd.mask_first = fg->dmask[0];
        q.fd.mask_later = fg->dmask[1];
        q.fd.solves = t.dev_ctr;
        q.fd.active = t.dev_ctr + 1;
        q.fd.keep_S = 1;  // the unranged source tokens would assign the same pattern every step
        q.A = fg->dA[0];
        q.T = fg->dA[1];
        q.cap = fg->dcap;
        q.h = fg->spacestep;
        q.nx = fg->nx;
        q.ny = fg->ny;
        q.nz = fg->nz;
        for (int d = 0; d < 3; d++) {
            q.org[d] = t.org[d];
            q.periodic[d] = c->box.periodic[d];
            q.lo[d] = c->box.lo[d];
            q.L[d] = c->box.L[d];
        }
        q.sum = t.cell_sum;
        q.cnt = t.cell_cnt;
        q.ctr = t.dev_ctr;
        const int gc = grid_for(fg->dim, TH_BLOCK);
        k_ttm_grid_lattice<<<g, TH_BLOCK, 0, c->stream>>>(q, c->n, c->x, c->y, c->z, t.temp, t.nneig, aflag);
        k_ttm_grid_fd<<<gc, TH_BLOCK, 0, c->stream>>>(p, q, t.st, c->d_status);
        cudaError_t e = fd_solve_coupled(q.fd, q.T, q.A, c->stream);
        if (e != cudaSuccess) return check_cuda(c, e, "ttm grid solve");
        k_ttm_grid_scale<<<g, TH_BLOCK, 0, c->stream>>>(p, q, c->n, tp.volcut, t.st, c->x, c->y, c->z, c->vx, c->vy,
                                                        c->vz, c->type, c->d_mass, t.vcm, t.temp, t.dens, aflag,
                                                        t.partial, c->d_status);
        k_ttm_sum<<<1, 256, 0, c->stream>>>(g, t.partial, t.st);
        prof_end(c);
        c->launches += 5;
        return check_cuda(c, cudaGetLastError(), "ttm grid");
    }
    k_ttm_fd<<<1, 32, 0, c->stream>>>(p, t.st, c->d_status);
    k_ttm_scale<<<g, TH_BLOCK, 0, c->stream>>>(p, c->n, tp.volcut, t.st, c->vx, c->vy, c->vz, c->type, c->d_mass,
                                                t.vcm, t.temp, t.dens, aflag, t.partial);
    k_ttm_sum<<<1, 256, 0, c->stream>>>(g, t.partial, t.st);
    prof_end(c);
    c->launches += 3;
    return check_cuda(c, cudaGetLastError(), "ttm");
}

bool ttm_active(const Context* c) { return c->ttm && c->ttm->ttm; }

// Ends the grid coupling: the grid's solve count and cell vector (dA[0])
// come back to its host-driven state.
static void ttm_grid_detach(Context* c, TTMCtx& t) {
    if (!t.grid) return;
    int ctr[2] = {0, 0};
    if (t.dev_ctr && cudaMemcpyAsync(ctr, t.dev_ctr, sizeof(ctr), cudaMemcpyDeviceToHost, c->stream) == cudaSuccess &&
        cudaStreamSynchronize(c->stream) == cudaSuccess)
        t.grid->solves = ctr[0];
    t.grid->cur = 0;
    t.grid->coupled = false;
    t.grid = nullptr;
    cudaFree(t.cell_sum);
    cudaFree(t.cell_cnt);
    cudaFree(t.dev_ctr);
    t.cell_sum = nullptr;
    t.cell_cnt = nullptr;
    t.dev_ctr = nullptr;
}

void ttm_release(Context* c) {
    if (!c->ttm) return;
    TTMCtx& t = *c->ttm;
    ttm_grid_detach(c, t);
    cudaFree(t.vcm);
    cudaFree(t.temp);
    cudaFree(t.dens);
    cudaFree(t.nneig);
    cudaFree(t.partial);
    cudaFree(t.st);
    cudaFree(t.coef64[0]);
    cudaFree(t.coef64[1]);
    delete c->ttm;
    c->ttm = nullptr;
}

static int upload64(Context* c, HostTable& h, DevTable& d, double4_32a*& buf) {
    std::vector<double4_32a> v(h.n);
    for (int k = 0; k < h.n; k++) v[k] = make_double4_32a(h.a[k], h.b[k], h.c[k], h.d[k]);
    if (cudaMalloc(&buf, sizeof(double4_32a) * h.n) != cudaSuccess) return set_error(c, OMDG_ENOMEM, "ttm tables");
    cudaMemcpy(buf, v.data(), sizeof(double4_32a) * h.n, cudaMemcpyHostToDevice);
    d = DevTable{};
    d.coef = nullptr;
    d.coef64 = buf;
    d.n = h.n;
    d.dr64 = h.dr;
    d.off64 = h.off;
    d.rmult = h.rmult ? 1 : 0;
    d.allow_hi = h.allow_hi ? 1 : 0;
    d.allow_lo = h.allow_lo ? 1 : 0;
    d.out_hi = h.out_hi;
    d.out_lo = h.out_lo;
    return OMDG_OK;
}

}  // namespace omdg

using namespace omdg;

extern "C" {

int omdg_set_thermo_detector(omdg_ctx* c, int on, double ercut) {
    if (!c) return OMDG_EINVAL;
    if (c->nrep > 0) return set_error(c, OMDG_EINVAL, "the detector runs on single boxes");
    if (!on) {
        if (c->ttm && c->ttm->ttm) return set_error(c, OMDG_ESTATE, "the two-temperature model needs the detector");
        ttm_release(c);
        update_rc(c);
        return OMDG_OK;
    }
    if (!c->ttm) c->ttm = new TTMCtx();
    c->ttm->ercut = ercut;
    update_rc(c);  // the list must reach the detector's cutoff
    return OMDG_OK;
}

int omdg_set_ttm(omdg_ctx* c, const char* table_file, double atom_volume, double electron_temperature,
                 double pulse_offset) {
    if (!c || !table_file || !(atom_volume > 0)) return c ? set_error(c, OMDG_EINVAL, "atom_volume must be > 0")
                                                          : OMDG_EINVAL;
    if (c->thermo_tau > 0.0)
        return set_error(c, OMDG_EINVAL, "the two-temperature model and the Berendsen thermostat exclude each other");
    cudaSetDevice(c->device);
    int rc = omdg_set_thermo_detector(c, 1, c->ttm ? c->ttm->ercut : -1.0);
    if (rc) return rc;
    TTMCtx& t = *c->ttm;
    std::string err;
    if ((rc = table_load(table_file, "ELECTRON_PHONON_COUPLING", t.g, err)) ||
        (rc = table_load(table_file, "ELECTRON_HEAT_CAPACITY", t.ce, err)))
        return set_error(c, rc, err);
    if (!t.g.has_constant || !t.ce.has_constant) return set_error(c, OMDG_EFILE, "TTM tables need a Constant");
    table_coef(t.g);
    table_coef(t.ce);
    cudaFree(t.coef64[0]);
    cudaFree(t.coef64[1]);
    t.coef64[0] = t.coef64[1] = nullptr;
    if ((rc = upload64(c, t.g, t.dg, t.coef64[0])) || (rc = upload64(c, t.ce, t.dce, t.coef64[1]))) return rc;
    t.g0 = t.g.constant;
    t.c0 = t.ce.constant;
    t.vol = atom_volume;
    t.te0 = electron_temperature;
    t.offset = pulse_offset;
    t.ttm = true;
    if (t.st) {  // restart the model
        TTMState h{};
        h.te = t.te0;
        h.firstfd = 1;
        cudaMemcpy(t.st, &h, sizeof(h), cudaMemcpyHostToDevice);
    }
    invalidate_graph(c);
    return OMDG_OK;
}

int omdg_set_ttm_grid(omdg_ctx* c, omdg_fdtd* grid, const double* origin) {
    if (!c) return OMDG_EINVAL;
    cudaSetDevice(c->device);
    if (!grid) {
        if (c->ttm) ttm_grid_detach(c, *c->ttm);
        invalidate_graph(c);
        return OMDG_OK;
    }
    if (!origin) return set_error(c, OMDG_EINVAL, "the grid needs an origin");
    if (!c->ttm || !c->ttm->ttm) return set_error(c, OMDG_ESTATE, "set the two-temperature model first");
    if (grid->device != c->device) return set_error(c, OMDG_EINVAL, "the grid lives on another device");
    if (grid->coupled && c->ttm->grid != grid) return set_error(c, OMDG_ESTATE, "the grid is coupled to another context");
    for (const std::string* k : {&grid->str_src, &grid->str_con, &grid->str_cap})
        if (k->find(':') != std::string::npos || k->find('{') != std::string::npos)
            return set_error(c, OMDG_EINVAL, "time-ranged assignments need host steps of the grid");
    TTMCtx& t = *c->ttm;
    ttm_grid_detach(c, t);
    // the kept strings once more (they are unranged: every later step would
    // apply the same values), then their images on the device
    int rc = fd_sync_data(grid);
    if (!rc) rc = fd_upload(grid, grid->stream);
    if (rc) return set_error(c, rc, grid->err);
    cudaError_t e = cudaSuccess;
    if (grid->cur == 1) {
        e = cudaMemcpyAsync(grid->dA[0], grid->dA[1], sizeof(double) * grid->dim, cudaMemcpyDeviceToDevice,
                            grid->stream);
        grid->cur = 0;
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(grid->stream);
    if (e == cudaSuccess) e = cudaMalloc(&t.cell_sum, sizeof(unsigned long long) * grid->dim);
    if (e == cudaSuccess) e = cudaMalloc(&t.cell_cnt, sizeof(int) * grid->dim);
    if (e == cudaSuccess) e = cudaMalloc(&t.dev_ctr, 2 * sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(t.cell_sum, 0, sizeof(unsigned long long) * grid->dim);
    if (e == cudaSuccess) e = cudaMemset(t.cell_cnt, 0, sizeof(int) * grid->dim);
    const int ctr[2] = {grid->solves, 0};
    if (e == cudaSuccess) e = cudaMemcpy(t.dev_ctr, ctr, sizeof(ctr), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(t.cell_sum);
        cudaFree(t.cell_cnt);
        cudaFree(t.dev_ctr);
        t.cell_sum = nullptr;
        t.cell_cnt = nullptr;
        t.dev_ctr = nullptr;
        return check_cuda(c, e, "ttm grid");
    }
    for (int d = 0; d < 3; d++) t.org[d] = origin[d];
    t.grid = grid;
    grid->coupled = true;
    invalidate_graph(c);
    return OMDG_OK;
}

int omdg_ttm_state(omdg_ctx* c, double* electron_temperature, double* int_een, double* int_aen,
                   double* lattice_temperature) {
    if (!c) return OMDG_EINVAL;
    if (!c->ttm || !c->ttm->st) return set_error(c, OMDG_ESTATE, "no detector state yet");
    cudaSetDevice(c->device);
    TTMState h;
    cudaError_t e = cudaMemcpyAsync(&h, c->ttm->st, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return check_cuda(c, e, "ttm state");
    if (electron_temperature) *electron_temperature = h.te;
    if (int_een) *int_een = h.int_een;
    if (int_aen) *int_aen = h.int_aen;
    if (lattice_temperature) *lattice_temperature = h.t_avg;
    return OMDG_OK;
}

int omdg_local_thermo(omdg_ctx* c, double* temperature, double* density, double* vcm) {
    if (!c) return OMDG_EINVAL;
    if (!c->ttm || !c->ttm->temp) return set_error(c, OMDG_ESTATE, "no detector state yet");
    cudaSetDevice(c->device);
    const int n = c->n;
    std::vector<double> t(n), d(n), v(3 * (size_t)n);
    std::vector<int> id(n);
    cudaMemcpyAsync(t.data(), c->ttm->temp, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(d.data(), c->ttm->dens, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(v.data(), c->ttm->vcm, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(id.data(), c->id, sizeof(int) * n, cudaMemcpyDeviceToHost, c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return check_cuda(c, e, "local thermo");
    for (int i = 0; i < n; i++) {
        const int k = id[i];  // caller index of sorted atom i
        if (temperature) temperature[k] = t[i];
        if (density) density[k] = d[i];
        if (vcm)
            for (int q = 0; q < 3; q++) vcm[3 * (size_t)k + q] = v[(size_t)q * n + i];
    }
    return OMDG_OK;
}

}  // extern "C"
