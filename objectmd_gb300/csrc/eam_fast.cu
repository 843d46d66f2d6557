// Specialised EAM kernels for the common case: one atom type, PAIR and
// EDENS tables on the same knot grid, no OutOfRange values (a read outside
// the table is an error, as in the reference).  Same arithmetic as eam.cu
// (team.cpp:81-92, :116-145, :224-237), arranged for the GB300 memory system:
//   - each lane loads all of its neighbour-list entries up front (one DRAM
//     round trip per atom instead of one per neighbour) and gathers the next
//     neighbour's pack while it evaluates the current one,
//   - a neighbour's position pack (with F'(rho) in its spare word) and an
//     interleaved (phi, rho) knot are one 256-bit load each,
//   - the periodic image comes from a 64-entry shared table of split shift
//     vectors indexed by the entry's 6 image bits,
//   - the knot index is clamped instead of branched (r <= rc keeps it below
//     n-1; the reference's x == n-1 rule selects the same segment),
//   - forces use Kahan sums, the per-pair energy and virial plain FP32 sums.
//
// Cell tiles (k_eamt_*): the gathers above cost one L1 wavefront-limited
// 32-byte sector per neighbour pack.  A tiled pass gives each CTA a block of
// cells; it stages the packs of those cells and their one-cell halo into
// shared memory once (coalesced runs of each cell's atoms), as coordinates
// relative to the tile's corner with the periodic image already applied,
// and walks each owned atom's row of 16-bit slots into that staged halo
// (written by the list build).  The relative vector keeps the gather
// path's precision: hi - O is exact (one binade), adding the image's hi
// length is exact (Sterbenz: the wrapped atom sits about one box length
// from the tile), so hi'_i - hi'_j is the exact hi difference and the lo
// parts add the remainder with one rounding.
#include "integrate_dev.cuh"

namespace omdg {

struct EAMFast {
    int n, hshift, maxnb;
    float Lh[3], Ll[3];
    const float4* coef2;   // (phi, rho) knot pairs
    const float4* emb;     // EMBED knots
    float off, dr, inv_dr;
    int nknot;
    float rc_phi, rc_rho, rc2;
    int rmult_phi, rmult_rho;
    float e_off, e_dr, e_inv_dr;
    int e_n, e_rmult;
    int stage_k0, stage_n;
    int first;
    int src_phi, src_rho, src_emb;  // table ids for error reports (DevTable::src)
};

__device__ __forceinline__ void build_shift_table(const EAMFast& p, float4* s_hi, float4* s_lo) {
    for (int k = threadIdx.x; k < 64; k += blockDim.x) {
        int bx = k & 3, by = (k >> 2) & 3, bz = (k >> 4) & 3;
        float fx = (float)(bx - 1), fy = (float)(by - 1), fz = (float)(bz - 1);
        s_hi[k] = make_float4(fx * p.Lh[0], fy * p.Lh[1], fz * p.Lh[2], 0.f);
        s_lo[k] = make_float4(fx * p.Ll[0], fy * p.Ll[1], fz * p.Ll[2], 0.f);
    }
}

// d = x_i - (x_j + s L) with the shift from the table (exact hi differences,
// see pair_delta in device_common.cuh).
__device__ __forceinline__ float3 delta_tab(const float4& hi, const float4& lo, const float4& hj, const float4& lj,
                                            const float4& sh, const float4& sl) {
    float3 d;
    d.x = __fadd_rn(__fsub_rn(__fsub_rn(hi.x, hj.x), sh.x), __fsub_rn(__fsub_rn(lo.x, lj.x), sl.x));
    d.y = __fadd_rn(__fsub_rn(__fsub_rn(hi.y, hj.y), sh.y), __fsub_rn(__fsub_rn(lo.y, lj.y), sl.y));
    d.z = __fadd_rn(__fsub_rn(__fsub_rn(hi.z, hj.z), sh.z), __fsub_rn(__fsub_rn(lo.z, lj.z), sl.z));
    return d;
}

template <int LANES>
__device__ __forceinline__ void twosum_reduce(float& s, float& c) {
#pragma unroll
    for (int off = LANES / 2; off > 0; off >>= 1) {
        float s2 = __shfl_xor_sync(0xffffffffu, s, off);
        float c2 = __shfl_xor_sync(0xffffffffu, c, off);
        float t = __fadd_rn(s, s2);
        float bp = __fsub_rn(t, s);
        float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(s2, bp));
        c = __fsub_rn(__fadd_rn(c, c2), e);
        s = t;
    }
}

template <int LANES>
__device__ __forceinline__ float plain_reduce(float v) {
#pragma unroll
    for (int off = LANES / 2; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// Entries a lane prefetches into registers per pass over its row.
template <int LANES>
struct Prefetch {
    static constexpr int N = LANES >= 4 ? 64 / LANES : 16;
};

// Staged variants hold the knot window in shared memory (up to ~110 KB) and
// run two 512-thread CTAs per SM, so 32 warps hide the gathers' latency.
#define EAMF_BOUNDS(STAGED) __launch_bounds__((STAGED) ? 512 : 256, (STAGED) ? 2 : 4)

// Index of the rho knot below r, or -1 when r is closer than the first knot
// (outside every tabulated range here).
__device__ __forceinline__ int knot_of(const EAMFast& p, float r, float offdr, float& dx) {
    int x = __float2int_rz(fmaf(r, p.inv_dr, -offdr));
    if (x < 0) return -1;
    x = min(x, p.nknot - 2);
    dx = fmaf(-(float)x, p.dr, r - p.off);
    return x;
}

// One lane's share of rho_i over the gathered row of atom ii (entries lane,
// lane + LANES, ...).
template <int LANES, bool STAGED>
__device__ __forceinline__ void gather_density_sum(const EAMFast& p, const PosPack* pack,
                                                   const unsigned* __restrict__ nbr, int ii, int m, int lane,
                                                   const float4* s_hi, const float4* s_lo, const float4* s_rho,
                                                   Kahan& acc, unsigned* status) {
    constexpr int PF = Prefetch<LANES>::N;
    const int step = LANES << p.hshift;
    const float rc2 = p.rc_rho * p.rc_rho * 1.0001f;
    const float offdr = p.off * p.inv_dr;
    const float4 hi = pack[ii].hi, lo = pack[ii].lo;
    const unsigned* rp = nbr + nbr_at(ii, lane, p.hshift, p.maxnb);
    bool bad = false;
    for (int s0 = lane; s0 < m; s0 += PF * LANES, rp += PF * step) {
        unsigned ent[PF];
#pragma unroll
        for (int k = 0; k < PF; k++) ent[k] = (s0 + k * LANES < m) ? __ldg(rp + k * step) : 0u;
        float4 hj, lj;
        ld256(pack + (ent[0] & (unsigned)INDEX_MASK), hj, lj);
#pragma unroll
        for (int k = 0; k < PF; k++) {
            if (s0 + k * LANES >= m) break;
            float4 hn, ln;
            if (k + 1 < PF && s0 + (k + 1) * LANES < m) ld256(pack + (ent[k + 1] & (unsigned)INDEX_MASK), hn, ln);
            const int code = (int)(ent[k] >> 26);
            const float3 d = delta_tab(hi, lo, hj, lj, s_hi[code], s_lo[code]);
            hj = hn;
            lj = ln;
            const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
            if (r2 > rc2) continue;
            const float r = r2 * rsqrtf(r2);
            if (!(r <= p.rc_rho)) continue;
            float dx;
            const int x = knot_of(p, r, offdr, dx);
            if (x < 0) {
                if (!bad) report_range(status, r, p.src_rho);
                bad = true;
                continue;
            }
            float4 cf;
            if (STAGED && (unsigned)(x - p.stage_k0) < (unsigned)p.stage_n) cf = s_rho[x - p.stage_k0];
            else cf = __ldg(&p.coef2[2 * (size_t)x + 1]);
            float v = fmaf(dx, fmaf(dx, fmaf(dx, cf.x, cf.y), cf.z), cf.w);
            if (p.rmult_rho) v = v / r;
            acc.add(v);
        }
    }
}

// F(rho), F'(rho) for atom i (TableReader::read on the EMBED section); F'
// also travels with the position for the force pass.
__device__ __forceinline__ void density_finish(const EAMFast& p, int i, float rho, PosPack* pack, float* fp,
                                               float* femb, unsigned* status) {
    const float rval = rho - p.e_off;
    int x = __float2int_rz(rval * p.e_inv_dr);
    float F = 0.f, dF = 0.f;
    if (x < -1 || x > p.e_n - 1) {
        report_range(status, rho, p.src_emb);
    } else {
        float dx = fmaf(-(float)x, p.e_dr, rval);
        if (x == p.e_n - 1) {
            dx += p.e_dr;
            x--;
        }
        if (x == -1) x = 0;
        const float4 cf = __ldg(&p.emb[x]);
        F = fmaf(dx, fmaf(dx, fmaf(dx, cf.x, cf.y), cf.z), cf.w);
        dF = fmaf(dx, fmaf(3.0f * dx, cf.x, 2.0f * cf.y), cf.z);
        if (p.e_rmult) {
            F = F / rho;
            dF = (dF - F) / rho;
        }
    }
    fp[i] = dF;
    femb[i] = F;
    pack[i].lo.w = dF;
}

template <int LANES, bool STAGED>
__global__ void EAMF_BOUNDS(STAGED) k_eamf_density(EAMFast p, PosPack* pack, const unsigned* __restrict__ nbr,
                                                   const int* __restrict__ nnb, float* __restrict__ fp,
                                                   float* __restrict__ femb, unsigned* status) {
    __shared__ float4 s_hi[64], s_lo[64];
    extern __shared__ float4 s_rho[];
    build_shift_table(p, s_hi, s_lo);
    if (STAGED)
        for (int k = threadIdx.x; k < p.stage_n; k += blockDim.x) s_rho[k] = p.coef2[2 * (size_t)(p.stage_k0 + k) + 1];
    __syncthreads();
    const int lane = threadIdx.x & (LANES - 1);
    const int per_block = blockDim.x / LANES;
    for (int base = blockIdx.x * per_block; base < p.n; base += gridDim.x * per_block) {
        const int i = base + threadIdx.x / LANES;
        const bool valid = i < p.n;
        const int ii = valid ? i : p.n - 1;
        const int m = valid ? nnb[ii] : 0;
        Kahan acc;
        gather_density_sum<LANES, STAGED>(p, pack, nbr, ii, m, lane, s_hi, s_lo, s_rho, acc, status);
        float sum = acc.s, comp = acc.c;
        twosum_reduce<LANES>(sum, comp);
        if (lane == 0 && valid) density_finish(p, i, __fsub_rn(sum, comp), pack, fp, femb, status);
    }
}

// The pair terms of one neighbour: force factor fr (f_i += d fr), half the
// pair energy and the virial term.
__device__ __forceinline__ void eam_pair_terms(const EAMFast& p, float r2, float fpij, const float4& cp,
                                               const float4& cr, float dx, float r, float rinv, float& fr,
                                               float& eh) {
    float ph = fmaf(dx, fmaf(dx, fmaf(dx, cp.x, cp.y), cp.z), cp.w);
    float dph = fmaf(dx, fmaf(3.0f * dx, cp.x, 2.0f * cp.y), cp.z);
    if (p.rmult_phi) {
        ph = ph * rinv;
        dph = (dph - ph) * rinv;
    }
    float drho = fmaf(dx, fmaf(3.0f * dx, cr.x, 2.0f * cr.y), cr.z);
    if (p.rmult_rho) {
        const float rv = fmaf(dx, fmaf(dx, fmaf(dx, cr.x, cr.y), cr.z), cr.w);
        drho = (drho - rv * rinv) * rinv;
    }
    if (r > p.rc_rho) drho = 0.f;
    fr = -fmaf(fpij, drho, dph) * rinv;
    eh = 0.5f * ph;
}

// One lane's share of the force, energy and virial of atom ii over its
// gathered row.
template <int LANES, bool STAGED>
__device__ __forceinline__ void gather_force_sum(const EAMFast& p, const PosPack* __restrict__ pack,
                                                 const unsigned* __restrict__ nbr, int ii, int m, int lane,
                                                 const float4* s_hi, const float4* s_lo, const float4* s_tab,
                                                 Kahan& ax, Kahan& ay, Kahan& az, float& ae, float& av,
                                                 unsigned* status) {
    constexpr int PF = Prefetch<LANES>::N;
    const int step = LANES << p.hshift;
    const float offdr = p.off * p.inv_dr;
    const float4 hi = pack[ii].hi, lo = pack[ii].lo;
    const float fpi = lo.w;
    const unsigned* rp = nbr + nbr_at(ii, lane, p.hshift, p.maxnb);
    bool bad = false;
    for (int s0 = lane; s0 < m; s0 += PF * LANES, rp += PF * step) {
        unsigned ent[PF];
#pragma unroll
        for (int k = 0; k < PF; k++) ent[k] = (s0 + k * LANES < m) ? __ldg(rp + k * step) : 0u;
        float4 hj, lj;
        ldg256(pack + (ent[0] & (unsigned)INDEX_MASK), hj, lj);
#pragma unroll
        for (int k = 0; k < PF; k++) {
            if (s0 + k * LANES >= m) break;
            float4 hn, ln;
            if (k + 1 < PF && s0 + (k + 1) * LANES < m) ldg256(pack + (ent[k + 1] & (unsigned)INDEX_MASK), hn, ln);
            const int code = (int)(ent[k] >> 26);
            const float3 d = delta_tab(hi, lo, hj, lj, s_hi[code], s_lo[code]);
            const float fpj = lj.w;  // F'(rho_j) from the density pass
            hj = hn;
            lj = ln;
            const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
            if (r2 > p.rc2) continue;
            const float rinv = rsqrtf(r2);
            const float r = r2 * rinv;
            if (!(r <= p.rc_phi)) continue;
            float dx;
            const int x = knot_of(p, r, offdr, dx);
            if (x < 0) {
                if (!bad) report_range(status, r, p.src_phi);
                bad = true;
                continue;
            }
            float4 cp, cr;
            if (STAGED && (unsigned)(x - p.stage_k0) < (unsigned)p.stage_n) {
                cp = s_tab[x - p.stage_k0];
                cr = s_tab[p.stage_n + x - p.stage_k0];
            } else {
                ldg256(&p.coef2[2 * (size_t)x], cp, cr);
            }
            float fr, eh;
            eam_pair_terms(p, r2, fpi + fpj, cp, cr, dx, r, rinv, fr, eh);
            ax.add(d.x * fr);
            ay.add(d.y * fr);
            az.add(d.z * fr);
            ae += eh;
            av = fmaf(fr, r2, av);
        }
    }
}

// Lane reductions of one atom's force sums (every lane holds the totals).
template <int LANES>
__device__ __forceinline__ void force_reduce(Kahan& ax, Kahan& ay, Kahan& az, float& ae, float& av) {
    twosum_reduce<LANES>(ax.s, ax.c);
    twosum_reduce<LANES>(ay.s, ay.c);
    twosum_reduce<LANES>(az.s, az.c);
    ae = plain_reduce<LANES>(ae);
    av = plain_reduce<LANES>(av);
}

__device__ __forceinline__ void force_store(const EAMFast& p, int i, float vfx, float vfy, float vfz, float ve,
                                            float av, float* fx, float* fy, float* fz, float* pe, float* vir) {
    if (p.first) {
        fx[i] = vfx;
        fy[i] = vfy;
        fz[i] = vfz;
        pe[i] = ve;
        vir[i] = av;
    } else {
        fx[i] += vfx;
        fy[i] += vfy;
        fz[i] += vfz;
        pe[i] += ve;
        vir[i] += av;
    }
}

// KICK: the step's second half-kick and its ledger terms in the epilogue (the
// force is final here: one potential, no force modifies), as k_kick does
// them, one ledger partial per warp.
template <int LANES, bool STAGED, bool KICK>
__global__ void EAMF_BOUNDS(STAGED) k_eamf_force(EAMFast p, const PosPack* __restrict__ pack,
                                                       const unsigned* __restrict__ nbr, const int* __restrict__ nnb,
                                                       const float* __restrict__ femb, float* __restrict__ fx,
                                                       float* __restrict__ fy, float* __restrict__ fz,
                                                       float* __restrict__ pe, float* __restrict__ vir,
                                                       unsigned* status, KickArgs ka, double* __restrict__ vx,
                                                       double* __restrict__ vy, double* __restrict__ vz,
                                                       const unsigned* __restrict__ aflag, double* __restrict__ ledger) {
    // the kick's ledger terms of each thread wait in shared memory, not in
    // registers held across the neighbour loop
    // (one slot per atom of the block: lane 0 of each atom's lanes)
    constexpr int KS = KICK ? (STAGED ? 512 : 256) / LANES : 1;
    __shared__ F2 s_kk[KS], s_ke[KS], s_kw[KS];
    __shared__ unsigned long long s_kv[KS];
    const int kslot = threadIdx.x / LANES;
    if (KICK && (threadIdx.x & (LANES - 1)) == 0) {
        s_kk[kslot] = s_ke[kslot] = s_kw[kslot] = F2{0.f, 0.f};
        s_kv[kslot] = 0ull;
    }
    __shared__ float4 s_hi[64], s_lo[64];
    extern __shared__ float4 s_tab[];  // phi knots [k0, k0+ns), then rho knots (separate arrays: a warp's
                                       // random knots spread over all eight 16-byte bank groups)
    build_shift_table(p, s_hi, s_lo);
    if (STAGED)
        for (int k = threadIdx.x; k < 2 * p.stage_n; k += blockDim.x) {
            const int kk = k < p.stage_n ? k : k - p.stage_n;
            s_tab[k] = p.coef2[2 * (size_t)(p.stage_k0 + kk) + (k < p.stage_n ? 0 : 1)];
        }
    __syncthreads();
    const int lane = threadIdx.x & (LANES - 1);
    const int per_block = blockDim.x / LANES;
    for (int base = blockIdx.x * per_block; base < p.n; base += gridDim.x * per_block) {
        const int i = base + threadIdx.x / LANES;
        const bool valid = i < p.n;
        const int ii = valid ? i : p.n - 1;
        const int m = valid ? nnb[ii] : 0;
        Kahan ax, ay, az;
        float ae = 0.f, av = 0.f;
        gather_force_sum<LANES, STAGED>(p, pack, nbr, ii, m, lane, s_hi, s_lo, s_tab, ax, ay, az, ae, av, status);
        force_reduce<LANES>(ax, ay, az, ae, av);
        if (lane == 0 && valid) {
            const float vfx = __fsub_rn(ax.s, ax.c), vfy = __fsub_rn(ay.s, ay.c), vfz = __fsub_rn(az.s, az.c);
            const float ve = ae + femb[i];
            force_store(p, i, vfx, vfy, vfz, ve, av, fx, fy, fz, pe, vir);
            // inactive atoms: not integrated, not measured (system.cpp:1067, :1085)
            if (KICK && (!aflag || (aflag[i] & 1u))) {
                F2 kk = s_kk[kslot], ke = s_ke[kslot], kw = s_kw[kslot];
                unsigned long long kv = s_kv[kslot];
                // one type on this path; the finalising block changes hdtm only after every block read it
                kick_atom_terms(ka.p, i, 0, vfx, vfy, vfz, ve, av, ka.st->hdtm[0], vx, vy, vz, kk, ke, kw, kv);
                s_kk[kslot] = kk;
                s_ke[kslot] = ke;
                s_kw[kslot] = kw;
                s_kv[kslot] = kv;
            }
        }
    }
    if (KICK) {
        // one partial per warp, no block barrier (a barrier here would hold
        // every warp's slot until the block's slowest warp is done); a
        // one-block kernel sums them and writes the ledger row
        const bool own = (threadIdx.x & (LANES - 1)) == 0;
        const F2 z = {0.f, 0.f};
        warp_partial(ka.p, own ? s_kk[kslot] : z, own ? s_ke[kslot] : z, own ? s_kw[kslot] : z,
                     own ? s_kv[kslot] : 0ull, ka.partial + (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5));
    }
}

// ------------------------------------------------------------------ cell tiles

struct EAMTileArgs {
    int T[3], nt[3], nc[3], periodic[3];
    int hx, hy, HC, cap, stride;
    const unsigned short* __restrict__ sb;
    const int* __restrict__ nst;
    const float4* __restrict__ org;
    const unsigned short* __restrict__ tslot;
    const int* __restrict__ start;
};

constexpr int TILE_HC_MAX = 216;   // (4 + 2)^3 halo cells
constexpr int TILE_OWN_MAX = 64;   // 4^3 owned cells
constexpr int TILE_THREADS = 256;

// A tile's cells in shared memory: for each halo cell its first atom (the
// cell's start), its first staged slot and its periodic image; for each
// owned cell its halo index and the owned atoms before it.
struct TileSmem {
    int hj0[TILE_HC_MAX];
    int hsb[TILE_HC_MAX + 1];  // [HC]: atoms staged
    unsigned char hcode[TILE_HC_MAX];
    int own_h[TILE_OWN_MAX];
    int own_pre[TILE_OWN_MAX + 1];
    int nown;                  // owned cells
};

__device__ __forceinline__ void tile_setup(const EAMTileArgs& a, int t, TileSmem& ts) {
    const int t3[3] = {t % a.nt[0], (t / a.nt[0]) % a.nt[1], t / (a.nt[0] * a.nt[1])};
    for (int h = threadIdx.x; h < a.HC; h += blockDim.x) {
        const int l[3] = {h % a.hx, (h / a.hx) % a.hy, h / (a.hx * a.hy)};
        int k[3], code = 0, mul = 1;
        bool ok = true;
        for (int d = 0; d < 3; d++) {
            int gk = t3[d] * a.T[d] - 1 + l[d], s = 0;
            if (a.periodic[d]) {
                if (gk < 0) {
                    gk += a.nc[d];
                    s = -1;
                } else if (gk >= a.nc[d]) {
                    gk -= a.nc[d];
                    s = 1;
                }
            } else if (gk < 0 || gk >= a.nc[d]) {
                ok = false;
            }
            k[d] = gk;
            code += (s + 1) * mul;
            mul *= 3;
        }
        ts.hj0[h] = ok ? a.start[(k[2] * a.nc[1] + k[1]) * a.nc[0] + k[0]] : 0;
        ts.hsb[h] = a.sb[(size_t)t * a.HC + h];
        ts.hcode[h] = (unsigned char)code;
    }
    if (threadIdx.x == 0) {
        ts.hsb[a.HC] = a.nst[t];
        int no = 0, pre = 0;
        for (int lz = 1; lz <= a.T[2]; lz++)
            for (int ly = 1; ly <= a.T[1]; ly++)
                for (int lx = 1; lx <= a.T[0]; lx++) {
                    const int gx = t3[0] * a.T[0] + lx - 1, gy = t3[1] * a.T[1] + ly - 1, gz = t3[2] * a.T[2] + lz - 1;
                    if (gx >= a.nc[0] || gy >= a.nc[1] || gz >= a.nc[2]) continue;
                    const int c = (gz * a.nc[1] + gy) * a.nc[0] + gx;
                    ts.own_h[no] = (lz * a.hy + ly) * a.hx + lx;
                    ts.own_pre[no] = pre;
                    pre += a.start[c + 1] - a.start[c];
                    no++;
                }
        ts.own_pre[no] = pre;
        ts.nown = no;
    }
    __syncthreads();
}

// The tile's halo into shared memory: hi' = (hi - O) + s Lh (exact), lo' =
// lo + s Ll; w of hi' carries F'(rho_j) for the force pass.
template <bool COHERENT>
__device__ __forceinline__ void tile_stage(const EAMFast& p, const EAMTileArgs& a, int t, const TileSmem& ts,
                                           const PosPack* pack, float4* s_h, float4* s_l) {
    const float4 O = a.org[t];
    const int nst = ts.hsb[a.HC];
    for (int k = threadIdx.x; k < nst; k += blockDim.x) {
        int lo = 0, hi = a.HC - 1;  // the last halo cell starting at or before k
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (ts.hsb[mid] <= k) lo = mid;
            else hi = mid - 1;
        }
        const int j = ts.hj0[lo] + (k - ts.hsb[lo]);
        float4 hj, lj;
        if (COHERENT) ld256(pack + j, hj, lj);
        else ldg256(pack + j, hj, lj);
        const int code = ts.hcode[lo];
        const int sx = code % 3 - 1, sy = (code / 3) % 3 - 1, sz = code / 9 - 1;
        float4 H, L;
        H.x = __fadd_rn(__fsub_rn(hj.x, O.x), sel_shift(sx, p.Lh[0]));
        H.y = __fadd_rn(__fsub_rn(hj.y, O.y), sel_shift(sy, p.Lh[1]));
        H.z = __fadd_rn(__fsub_rn(hj.z, O.z), sel_shift(sz, p.Lh[2]));
        H.w = lj.w;
        L.x = __fadd_rn(lj.x, sel_shift(sx, p.Ll[0]));
        L.y = __fadd_rn(lj.y, sel_shift(sy, p.Ll[1]));
        L.z = __fadd_rn(lj.z, sel_shift(sz, p.Ll[2]));
        L.w = 0.f;
        s_h[k] = H;
        s_l[k] = L;
    }
}

// Owned atom q of the tile: its owned cell, its index and its staged slot.
__device__ __forceinline__ void tile_owned(const TileSmem& ts, int q, int& i, int& slot) {
    int lo = 0, hi = ts.nown - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (ts.own_pre[mid] <= q) lo = mid;
        else hi = mid - 1;
    }
    const int off = q - ts.own_pre[lo];
    const int h = ts.own_h[lo];
    i = ts.hj0[h] + off;
    slot = ts.hsb[h] + off;
}

__device__ __forceinline__ float3 tile_delta(const float4& hi, const float4& lo, const float4& hj, const float4& lj) {
    float3 d;
    d.x = __fadd_rn(__fsub_rn(hi.x, hj.x), __fsub_rn(lo.x, lj.x));
    d.y = __fadd_rn(__fsub_rn(hi.y, hj.y), __fsub_rn(lo.y, lj.y));
    d.z = __fadd_rn(__fsub_rn(hi.z, hj.z), __fsub_rn(lo.z, lj.z));
    return d;
}

// Slots a lane loads ahead from its row.
template <int LANES>
struct TilePrefetch {
    static constexpr int N = LANES >= 8 ? 64 / LANES : 8;
};

template <int LANES>
__global__ void __launch_bounds__(TILE_THREADS, 4) k_eamt_density(EAMFast p, EAMTileArgs a, PosPack* pack,
                                                                  const unsigned* __restrict__ nbr,
                                                                  const int* __restrict__ nnb, float* __restrict__ fp,
                                                                  float* __restrict__ femb, unsigned* status) {
    extern __shared__ float4 s_stage[];  // hi' [cap], then lo' [cap]
    __shared__ TileSmem ts;
    __shared__ float4 s_shi[64], s_slo[64];  // image shifts of the gather path
    const int t = blockIdx.x;
    tile_setup(a, t, ts);
    const bool staged = ts.hsb[a.HC] <= a.cap;
    float4* s_h = s_stage;
    float4* s_l = s_stage + a.cap;
    if (staged) tile_stage<true>(p, a, t, ts, pack, s_h, s_l);
    else build_shift_table(p, s_shi, s_slo);
    __syncthreads();
    constexpr int PF = TilePrefetch<LANES>::N;
    const float rc2 = p.rc_rho * p.rc_rho * 1.0001f;
    const float offdr = p.off * p.inv_dr;
    const int lane = threadIdx.x & (LANES - 1);
    const int per = blockDim.x / LANES;
    const int nown = ts.own_pre[ts.nown];
    for (int q0 = 0; q0 < nown; q0 += per) {
        const int q = q0 + threadIdx.x / LANES;
        const bool valid = q < nown;
        int i, si;
        tile_owned(ts, valid ? q : nown - 1, i, si);
        const int m = valid ? nnb[i] : 0;
        Kahan acc;
        if (staged) {
            const float4 hi = s_h[si], lo = s_l[si];
            const unsigned short* row = a.tslot + (size_t)i * a.stride;
            bool bad = false;
            for (int s0 = lane; s0 < m; s0 += PF * LANES) {
                int ent[PF];
#pragma unroll
                for (int k = 0; k < PF; k++) ent[k] = (s0 + k * LANES < m) ? (int)__ldg(row + s0 + k * LANES) : 0;
#pragma unroll
                for (int k = 0; k < PF; k++) {
                    if (s0 + k * LANES >= m) break;
                    const float3 d = tile_delta(hi, lo, s_h[ent[k]], s_l[ent[k]]);
                    const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
                    if (r2 > rc2) continue;
                    const float r = r2 * rsqrtf(r2);
                    if (!(r <= p.rc_rho)) continue;
                    float dx;
                    const int x = knot_of(p, r, offdr, dx);
                    if (x < 0) {
                        if (!bad) report_range(status, r, p.src_rho);
                        bad = true;
                        continue;
                    }
                    const float4 cf = __ldg(&p.coef2[2 * (size_t)x + 1]);
                    float v = fmaf(dx, fmaf(dx, fmaf(dx, cf.x, cf.y), cf.z), cf.w);
                    if (p.rmult_rho) v = v / r;
                    acc.add(v);
                }
            }
        } else {
            gather_density_sum<LANES, false>(p, pack, nbr, i, m, lane, s_shi, s_slo, nullptr, acc, status);
        }
        float sum = acc.s, comp = acc.c;
        twosum_reduce<LANES>(sum, comp);
        if (lane == 0 && valid) density_finish(p, i, __fsub_rn(sum, comp), pack, fp, femb, status);
    }
}

template <int LANES>
__global__ void __launch_bounds__(TILE_THREADS, 4) k_eamt_force(EAMFast p, EAMTileArgs a,
                                                                const PosPack* __restrict__ pack,
                                                                const unsigned* __restrict__ nbr,
                                                                const int* __restrict__ nnb,
                                                                const float* __restrict__ femb, float* __restrict__ fx,
                                                                float* __restrict__ fy, float* __restrict__ fz,
                                                                float* __restrict__ pe, float* __restrict__ vir,
                                                                unsigned* status) {
    extern __shared__ float4 s_stage[];
    __shared__ TileSmem ts;
    __shared__ float4 s_shi[64], s_slo[64];
    const int t = blockIdx.x;
    tile_setup(a, t, ts);
    const bool staged = ts.hsb[a.HC] <= a.cap;
    float4* s_h = s_stage;
    float4* s_l = s_stage + a.cap;
    if (staged) tile_stage<false>(p, a, t, ts, pack, s_h, s_l);
    else build_shift_table(p, s_shi, s_slo);
    __syncthreads();
    constexpr int PF = TilePrefetch<LANES>::N;
    const float offdr = p.off * p.inv_dr;
    const int lane = threadIdx.x & (LANES - 1);
    const int per = blockDim.x / LANES;
    const int nown = ts.own_pre[ts.nown];
    for (int q0 = 0; q0 < nown; q0 += per) {
        const int q = q0 + threadIdx.x / LANES;
        const bool valid = q < nown;
        int i, si;
        tile_owned(ts, valid ? q : nown - 1, i, si);
        const int m = valid ? nnb[i] : 0;
        Kahan ax, ay, az;
        float ae = 0.f, av = 0.f;
        if (staged) {
            const float4 hi = s_h[si], lo = s_l[si];
            const float fpi = hi.w;
            const unsigned short* row = a.tslot + (size_t)i * a.stride;
            bool bad = false;
            for (int s0 = lane; s0 < m; s0 += PF * LANES) {
                int ent[PF];
#pragma unroll
                for (int k = 0; k < PF; k++) ent[k] = (s0 + k * LANES < m) ? (int)__ldg(row + s0 + k * LANES) : 0;
#pragma unroll
                for (int k = 0; k < PF; k++) {
                    if (s0 + k * LANES >= m) break;
                    const float4 hj = s_h[ent[k]];
                    const float3 d = tile_delta(hi, lo, hj, s_l[ent[k]]);
                    const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
                    if (r2 > p.rc2) continue;
                    const float rinv = rsqrtf(r2);
                    const float r = r2 * rinv;
                    if (!(r <= p.rc_phi)) continue;
                    float dx;
                    const int x = knot_of(p, r, offdr, dx);
                    if (x < 0) {
                        if (!bad) report_range(status, r, p.src_phi);
                        bad = true;
                        continue;
                    }
                    float4 cp, cr;
                    ldg256(&p.coef2[2 * (size_t)x], cp, cr);
                    float fr, eh;
                    eam_pair_terms(p, r2, fpi + hj.w, cp, cr, dx, r, rinv, fr, eh);
                    ax.add(d.x * fr);
                    ay.add(d.y * fr);
                    az.add(d.z * fr);
                    ae += eh;
                    av = fmaf(fr, r2, av);
                }
            }
        } else {
            gather_force_sum<LANES, false>(p, pack, nbr, i, m, lane, s_shi, s_slo, nullptr, ax, ay, az, ae, av,
                                           status);
        }
        force_reduce<LANES>(ax, ay, az, ae, av);
        if (lane == 0 && valid) {
            const float vfx = __fsub_rn(ax.s, ax.c), vfy = __fsub_rn(ay.s, ay.c), vfz = __fsub_rn(az.s, az.c);
            force_store(p, i, vfx, vfy, vfz, ae + femb[i], av, fx, fy, fz, pe, vir);
        }
    }
}

template <int LANES>
static void launch_tiles(Context* c, const EAMFast& p, const EAMTileArgs& a) {
    static bool attr = false;
    const size_t smem = 2 * (size_t)a.cap * sizeof(float4);
    if (!attr) {
        cudaFuncSetAttribute(k_eamt_density<LANES>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
        cudaFuncSetAttribute(k_eamt_force<LANES>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
        attr = true;
    }
    const int grid = c->tile_count;
    prof_begin(c, "eam_density");
    k_eamt_density<LANES><<<grid, TILE_THREADS, smem, c->stream>>>(
        p, a, c->pack, reinterpret_cast<const unsigned*>(c->nbr), c->nnb, c->fp, c->femb, c->d_status);
    prof_end(c);
    prof_begin(c, "eam_force");
    k_eamt_force<LANES><<<grid, TILE_THREADS, smem, c->stream>>>(
        p, a, c->pack, reinterpret_cast<const unsigned*>(c->nbr), c->nnb, c->femb, c->fx, c->fy, c->fz, c->pe,
        c->vir, c->d_status);
    prof_end(c);
}

template <int LANES, bool STAGED>
static void launch_fast(Context* c, const EAMFast& p, int grid, int block, size_t smem1, size_t smem2,
                        const KickArgs* ka) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_eamf_density<LANES, STAGED>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(k_eamf_force<LANES, STAGED, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             200 * 1024);
        cudaFuncSetAttribute(k_eamf_force<LANES, STAGED, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             200 * 1024);
        attr = true;
    }
    prof_begin(c, "eam_density");
    k_eamf_density<LANES, STAGED><<<grid, block, smem1, c->stream>>>(
        p, c->pack, reinterpret_cast<const unsigned*>(c->nbr), c->nnb, c->fp, c->femb, c->d_status);
    prof_end(c);
    const unsigned* aflag = c->flags_used ? c->aflag : nullptr;
    if (ka) {
        prof_begin(c, "eam_force_kick");
        k_eamf_force<LANES, STAGED, true><<<grid, block, smem2, c->stream>>>(
            p, c->pack, reinterpret_cast<const unsigned*>(c->nbr), c->nnb, c->femb, c->fx, c->fy, c->fz, c->pe,
            c->vir, c->d_status, *ka, c->vx, c->vy, c->vz, aflag, c->d_ledger);
        launch_ledger_finalize(c, *ka, grid * (block >> 5));
    } else {
        prof_begin(c, "eam_force");
        k_eamf_force<LANES, STAGED, false><<<grid, block, smem2, c->stream>>>(
            p, c->pack, reinterpret_cast<const unsigned*>(c->nbr), c->nnb, c->femb, c->fx, c->fy, c->fz, c->pe,
            c->vir, c->d_status, KickArgs{}, nullptr, nullptr, nullptr, nullptr, nullptr);
    }
    prof_end(c);
}

// The fast path's shape: one type, PAIR and EDENS on one knot grid (their
// knots interleave in d_coef2, made by the first launch), no OutOfRange.
static bool eam_fast_shape(const Context* c, const Potential& pot) {
    const HostTable &a = pot.t0, &b = pot.t1;
    const bool same = a.n == b.n && a.dr == b.dr && a.off == b.off;
    return c->ntypes == 1 && same && !a.allow_lo && !a.allow_hi && !b.allow_lo && !b.allow_hi &&
           !pot.t2.allow_lo && !pot.t2.allow_hi && a.n >= 4;
}

bool tiles_apply(const Context* c) {
    if (!c->eam_tile || c->nrep > 0 || c->pots.size() != 1) return false;
    const Potential& p = c->pots[0];
    return p.kind == POT_EAM && eam_fast_shape(c, p);
}

bool eam_fast_ok(const Context* c, const Potential& pot) { return pot.d_coef2 && eam_fast_shape(c, pot); }

int eam_fast_launch(Context* c, Potential& pot, bool first) {
    EAMFast p;
    p.n = c->n;
    p.hshift = c->nbr_hshift;
    p.maxnb = c->maxnb;
    for (int d = 0; d < 3; d++) {
        p.Lh[d] = c->box.Lh[d];
        p.Ll[d] = c->box.Ll[d];
    }
    p.coef2 = pot.d_coef2;
    p.emb = pot.dt[2].coef;
    p.off = (float)pot.t0.off;
    p.dr = (float)pot.t0.dr;
    p.inv_dr = (float)(1.0 / pot.t0.dr);
    p.nknot = pot.t0.n;
    p.rc_phi = (float)pot.t0.max_range();
    p.rc_rho = (float)pot.t1.max_range();
    float rcm = p.rc_phi > p.rc_rho ? p.rc_phi : p.rc_rho;
    p.rc2 = rcm * rcm * 1.0001f;
    p.rmult_phi = pot.t0.rmult ? 1 : 0;
    p.rmult_rho = pot.t1.rmult ? 1 : 0;
    p.e_off = (float)pot.t2.off;
    p.e_dr = (float)pot.t2.dr;
    p.e_inv_dr = (float)(1.0 / pot.t2.dr);
    p.e_n = pot.t2.n;
    p.e_rmult = pot.t2.rmult ? 1 : 0;
    p.first = first ? 1 : 0;
    p.src_phi = pot.dt[0].src;
    p.src_rho = pot.dt[1].src;
    p.src_emb = pot.dt[2].src;
    int k0 = 0, ns = 0;
    if (c->eam_stage) {
        k0 = (int)((c->eam_stage_frac * pot.t1.max_range() - pot.t1.off) / pot.t1.dr);
        if (k0 < 0) k0 = 0;
        ns = pot.t1.n - k0;
        // two CTAs per SM: each holds at most 108 KB of (phi, rho) knots
        int max_stage = (108 * 1024) / (2 * (int)sizeof(float4));
        if (ns > max_stage) {
            k0 = pot.t1.n - max_stage;
            ns = max_stage;
        }
    }
    p.stage_k0 = k0;
    p.stage_n = ns;
    int block = c->eam_block > 256 ? 256 : c->eam_block, lanes = c->eam_lanes;
    int per_block = block / lanes;
    int grid = grid_for(c->n, per_block);
    if (ns > 0) {
        // staged: 512-thread CTAs, two resident per SM, striding over the atoms
        block = 512;
        per_block = block / lanes;
        grid = grid_for(c->n, per_block);
        int cap = 2 * c->num_sms;
        grid = grid < cap ? grid : cap;
    }
    size_t smem1 = (size_t)ns * sizeof(float4), smem2 = 2 * smem1;
    bool st = ns > 0;
    // the step's second half-kick in the force epilogue: one potential, the
    // first, and a block of whole warps (the ledger's block tree)
    KickArgs ka;
    const KickArgs* kap = nullptr;
    if (c->fuse_kick && c->fuse_kick_on && first && c->pots.size() == 1 && kick_fusable(c) && block % 32 == 0 &&
        (block & (block - 1)) == 0) {
        kick_args(c, ka);
        if (grid * (block >> 5) <= ka.partial_cap) {  // one partial per warp
            kap = &ka;
            c->kick_fused = true;
        }
    }
    // the tiled passes, where the last build wrote tile slots (staging keeps
    // the knots in global memory there; the kick stays a kernel of its own)
    if (c->tile_valid && c->eam_tile && c->tslot && !kap && c->tile_cap <= 5000) {
        EAMTileArgs a;
        for (int d = 0; d < 3; d++) {
            a.T[d] = c->tile_dim[d];
            a.nt[d] = c->tile_nt[d];
            a.nc[d] = c->box.nc[d];
            a.periodic[d] = c->box.periodic[d];
        }
        a.hx = a.T[0] + 2;
        a.hy = a.T[1] + 2;
        a.HC = c->tile_hc;
        a.cap = c->tile_cap;
        a.stride = c->tile_stride;
        a.sb = c->tile_sb;
        a.nst = c->tile_nst;
        a.org = c->tile_org;
        a.tslot = c->tslot;
        a.start = c->cell_start;
        switch (lanes) {
            case 4: launch_tiles<4>(c, p, a); break;
            case 16: launch_tiles<16>(c, p, a); break;
            default: launch_tiles<8>(c, p, a); break;
        }
        c->launches += 2;
        return check_cuda(c, cudaGetLastError(), "eam tiles");
    }
#define OMDG_EAMF(L)                                                 \
    (st ? launch_fast<L, true>(c, p, grid, block, smem1, smem2, kap) \
        : launch_fast<L, false>(c, p, grid, block, smem1, smem2, kap))
    switch (lanes) {
        case 1: OMDG_EAMF(1); break;
        case 2: OMDG_EAMF(2); break;
        case 4: OMDG_EAMF(4); break;
        case 8: OMDG_EAMF(8); break;
        case 16: OMDG_EAMF(16); break;
        default: OMDG_EAMF(32); break;
    }
#undef OMDG_EAMF
    c->launches += 2;
    return check_cuda(c, cudaGetLastError(), "eam");
}

}  // namespace omdg
