// Device side of the integrator shared by the kick kernel (integrate.cu) and
// the force kernels that take the second half-kick into their epilogue
// (eam_fast.cu): the step state, the kick parameters, and the energy ledger's
// block partials and last-block finalisation.
#pragma once

#include "device_common.cuh"

namespace omdg {

struct StepState {
    long long step;      // RunKernel Step (system.cpp:979)
    int row;             // ledger row within the current omdg_step call
    int rebuild;         // rebuild request for the next list build
    double lambda;       // velocity factor to apply before the next kick
    int rebuild_every;   // >0: rebuild when step % rebuild_every == 0
    int nrebuild;        // list builds taken by the graph's conditional node
    double dt;               // TimeStep (DynamicTimeStep changes it here, between steps)
    double hdtm[MAX_TYPES];  // (dt/2) / m per type, refreshed with dt
    double elapsed;          // ElapsedTime (system.cpp:979)
    double sqrmaxv;          // SqrMaxVelocity of the last measurement (system.cpp:1075-1094)
    int src_first;           // EnergySource: the first call inside the window only arms it
    int src_scale;           // EnergySource: scale velocities at the next PreIntegration
    int halted;              // a rebuild overflowed its rows: later rebuilds are skipped until omdg_sync recovers
    int rebuild_all;         // replica mode: the request covers every replica (periodic rebuild, state upload)
};

struct IntParams {
    int n;
    double org[3], P[3];
    float half_skin2;       // (skin/2)^2
    int use_f64;
    double Q[3];            // P - org: the pack coordinate is X = x + Q
    float Qh[3], Ql[3];     // Q as an FP32 pair (pack_coord)
    float mh[MAX_TYPES], ml[MAX_TYPES];  // mass per type as an FP32 pair
    int range_on;                        // RangeLimiter (RangeLimiter.h:33-54)
    unsigned range_group;                // group bits it acts on
    double range_lo[3], range_hi[3];     // box -/+ border
    int need_vmax;                       // measure SqrMaxVelocity (DynamicTimeStep)
};

struct FinParams {
    int natoms;
    int ledger_cap;
    int count_step;       // 1: this is a RunKernel step (advance Step)
    const int* ghosts;    // reference compatibility: periodic images added to the atom count (or null)
    unsigned* status;     // ERR_NONFINITE when a total is NaN or infinite
    unsigned* ticket;     // blocks done (the last one resets it)
    double tau, tset;     // thermostat (tau <= 0: off)
    double temp_factor;   // 2/3/k_B (unit.h:66-104)
    int need_vmax;        // SqrMaxVelocity from the block partials
    int dyn_update;       // DynamicTimeStep period (0: off; DynamicTimeStep.h:58-70)
    int dyn_apply;        // this measurement precedes a step's PreIntegration
    double dyn_maxpath, dyn_maxdt;
    double mass[MAX_TYPES];
    int src_on;                 // EnergySource (EnergySource.h:103-133)
    double src_start, src_stop;
};

// Block partials: sum m v^2, sum potential, sum virial as FP32 pairs, and
// the block's largest squared speed as the bit pattern of a non-negative
// double (integer order is value order): two float4 per block.
struct BlockPartial {
    float4 ke, wv;  // (k.hi, k.lo, e.hi, e.lo), (w.hi, w.lo, vmax bits low, high)
};

__device__ __forceinline__ unsigned long long vmax_bits(const float4& wv) {
    return ((unsigned long long)__float_as_uint(wv.w) << 32) | __float_as_uint(wv.z);
}

// Ledger row, thermostat factor and step counter from the block partials
// (one block; each thread sums a contiguous run of partials, then a fixed
// xor tree per warp and over the warps, all on FP32 pairs; FP64 only for
// the totals).  Partials are read through L2: other blocks wrote them.
static __device__ __noinline__ void finalize_block(const FinParams& p, int nblocks, const BlockPartial* partial, double* ledger,
                               StepState* st) {
    __shared__ F2 sk[32], se[32], sw[32];
    __shared__ unsigned long long sv[32];
    const int nwarps = blockDim.x >> 5;  // a power of two
    F2 kf = {0.f, 0.f}, ef = {0.f, 0.f}, wf = {0.f, 0.f};
    unsigned long long vb = 0ull;
    const int per = (nblocks + (int)blockDim.x - 1) / (int)blockDim.x;
    const int b0 = threadIdx.x * per, b1 = min(nblocks, b0 + per);
#pragma unroll 4
    for (int b = b0; b < b1; b++) {
        const float4 ke = __ldcg(&partial[b].ke), wv = __ldcg(&partial[b].wv);
        kf = f2_add(kf, F2{ke.x, ke.y});
        ef = f2_add(ef, F2{ke.z, ke.w});
        wf = f2_add(wf, F2{wv.x, wv.y});
        if (p.need_vmax) vb = max(vb, vmax_bits(wv));
    }
    // fixed xor tree within each warp, then over the warps in warp 0
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int o = 16; o > 0; o >>= 1) {
        kf = f2_add(kf, f2_shfl_xor(kf, o));
        ef = f2_add(ef, f2_shfl_xor(ef, o));
        wf = f2_add(wf, f2_shfl_xor(wf, o));
        if (p.need_vmax) vb = max(vb, __shfl_xor_sync(0xffffffffu, vb, o));
    }
    if (lane == 0) {
        sk[warp] = kf;
        se[warp] = ef;
        sw[warp] = wf;
        sv[warp] = vb;
    }
    __syncthreads();
    if (warp != 0) return;
    const F2 z = {0.f, 0.f};
    kf = lane < nwarps ? sk[lane] : z;
    ef = lane < nwarps ? se[lane] : z;
    wf = lane < nwarps ? sw[lane] : z;
    vb = lane < nwarps ? sv[lane] : 0ull;
    for (int o = nwarps / 2; o > 0; o >>= 1) {
        kf = f2_add(kf, f2_shfl_xor(kf, o));
        ef = f2_add(ef, f2_shfl_xor(ef, o));
        wf = f2_add(wf, f2_shfl_xor(wf, o));
        if (p.need_vmax) vb = max(vb, __shfl_xor_sync(0xffffffffu, vb, o));
    }
    const double k = f2_to_double(kf), e = f2_to_double(ef), w = f2_to_double(wf);
    const double vm = __longlong_as_double((long long)vb);
    if (threadIdx.x == 0) {
        double kinetic = 0.5 * k;
        if (!(isfinite(kinetic) && isfinite(e))) atomicOr(p.status, ERR_NONFINITE);
        int row = st->row;
        int slot = row % p.ledger_cap;  // ring buffer between host reads
        double* row_out = ledger + LEDGER_W * (size_t)slot;
        row_out[0] = kinetic;
        row_out[1] = e;
        row_out[2] = 0.5 * w;
        row_out[4] = (double)st->step;  // SysMonitor's Step, ElapsedTime and TimeStep of this step
        row_out[5] = st->elapsed;
        row_out[6] = st->dt;
        row_out[7] = 0.0;
        double lam = 1.0;
        if (p.count_step && p.tau > 0.0 && st->step != 0) {
            // TempController::PostIntegration: T from the system kinetic energy
            const double count = (double)p.natoms + (p.ghosts ? (double)*p.ghosts : 0.0);
            double T = p.temp_factor * kinetic / count;
            if (T > 0.0) lam = sqrt(1. + st->dt / p.tau * (p.tset / T - 1.));
        }
        row_out[3] = lam;
        if (p.need_vmax) st->sqrmaxv = vm;
        if (p.count_step) {
            st->lambda = lam;
            st->elapsed += st->dt;  // ElapsedTime += TimeStep; Step++ (system.cpp:979-980)
            st->step += 1;
            st->row = row + 1;
            if (st->rebuild_every > 0 && (st->step % st->rebuild_every) == 0) {
                st->rebuild = 1;
                st->rebuild_all = 1;
            }
            if (p.src_on) {  // EnergySource::PreIntegration of the next step
                int scale = 0;
                if (st->elapsed >= p.src_start) {
                    if (st->src_first) st->src_first = 0;  // firstcall: return
                    else scale = st->elapsed < p.src_stop ? 1 : 0;
                }
                st->src_scale = scale;
            }
        }
        if (p.dyn_update > 0 && p.dyn_apply && (st->step % p.dyn_update) == 0) {
            // DynamicTimeStep::PreIntegration of the next step
            double ndt;
            if (st->sqrmaxv > 0.0) {
                ndt = p.dyn_maxpath / (sqrt(st->sqrmaxv) * 1.10);
                if (ndt > p.dyn_maxdt) ndt = p.dyn_maxdt;
            } else {
                ndt = p.dyn_maxdt;
            }
            st->dt = ndt;
            for (int t = 0; t < MAX_TYPES; t++) st->hdtm[t] = p.mass[t] > 0 ? (0.5 * ndt) / p.mass[t] : 0.0;
        }
        *p.ticket = 0u;
    }
}

// One atom's second half-kick v += dt/2 f/m (velocity written back) and
// its ledger terms: m v^2 and the potential and virial as FP32 pairs, the
// squared speed's bits for DynamicTimeStep.  f is FP32 (the FP64 force path
// does not fuse).
__device__ __forceinline__ void kick_atom_terms(const IntParams& p, int i, int t, float fxi, float fyi, float fzi,
                                                float pei, float viri, double h, double* __restrict__ vx,
                                                double* __restrict__ vy, double* __restrict__ vz, F2& k, F2& e,
                                                F2& w, unsigned long long& vmax) {
    double ux = fma(f2d_exact(fxi), h, vx[i]);
    double uy = fma(f2d_exact(fyi), h, vy[i]);
    double uz = fma(f2d_exact(fzi), h, vz[i]);
    vx[i] = ux;
    vy[i] = uy;
    vz[i] = uz;
    const F2 sx = f2_from(ux), sy = f2_from(uy), sz = f2_from(uz);
    const F2 v2 = f2_add(f2_add(f2_mul(sx, sx), f2_mul(sy, sy)), f2_mul(sz, sz));
    k = f2_add(k, f2_mul(v2, F2{p.mh[t], p.ml[t]}));
    e = f2_add(e, F2{pei, 0.f});
    w = f2_add(w, F2{viri, 0.f});
    if (p.need_vmax)  // sqrv = vx*vx + vy*vy + vz*vz (system.cpp:1086)
        vmax = max(vmax, (unsigned long long)__double_as_longlong(
                             __dadd_rn(__dadd_rn(__dmul_rn(ux, ux), __dmul_rn(uy, uy)), __dmul_rn(uz, uz))));
}

// The block's ledger partial from every thread's terms (a fixed xor tree per
// warp and over the warps); the last block to finish sums the partials in
// block order and writes the ledger row (finalize_block).  Every thread of
// the block calls it.
__device__ __forceinline__ void ledger_block(const IntParams& p, const FinParams& f, F2 k, F2 e, F2 w,
                                             unsigned long long vmax, BlockPartial* __restrict__ partial,
                                             double* __restrict__ ledger, StepState* st) {
    if (p.need_vmax)
        for (int o = 16; o > 0; o >>= 1) vmax = max(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    for (int o = 16; o > 0; o >>= 1) {
        k = f2_add(k, f2_shfl_xor(k, o));
        e = f2_add(e, f2_shfl_xor(e, o));
        w = f2_add(w, f2_shfl_xor(w, o));
    }
    __shared__ F2 wk[32], we[32], ww[32];
    __shared__ unsigned long long wv[32];
    __shared__ bool last;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    if (lane == 0) {
        wk[warp] = k;
        we[warp] = e;
        ww[warp] = w;
        wv[warp] = vmax;
    }
    __syncthreads();
    if (warp == 0) {
        const F2 z = {0.f, 0.f};
        k = lane < nwarps ? wk[lane] : z;
        e = lane < nwarps ? we[lane] : z;
        w = lane < nwarps ? ww[lane] : z;
        for (int o = nwarps / 2; o > 0; o >>= 1) {
            k = f2_add(k, f2_shfl_xor(k, o));
            e = f2_add(e, f2_shfl_xor(e, o));
            w = f2_add(w, f2_shfl_xor(w, o));
        }
        if (lane == 0) {
            unsigned long long bv = 0ull;
            if (p.need_vmax)
                for (int q = 0; q < nwarps; q++) bv = max(bv, wv[q]);
            partial[blockIdx.x].ke = make_float4(k.hi, k.lo, e.hi, e.lo);
            partial[blockIdx.x].wv = make_float4(w.hi, w.lo, __uint_as_float((unsigned)bv),
                                                 __uint_as_float((unsigned)(bv >> 32)));
            __threadfence();
            last = atomicAdd(f.ticket, 1u) == gridDim.x - 1;
        }
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    finalize_block(f, gridDim.x, partial, ledger, st);
}

// One warp's ledger partial (the per-warp half of ledger_block): lane 0
// writes it.
__device__ __forceinline__ void warp_partial(const IntParams& p, F2 k, F2 e, F2 w, unsigned long long vmax,
                                             BlockPartial* __restrict__ out) {
    if (p.need_vmax)
        for (int o = 16; o > 0; o >>= 1) vmax = max(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    for (int o = 16; o > 0; o >>= 1) {
        k = f2_add(k, f2_shfl_xor(k, o));
        e = f2_add(e, f2_shfl_xor(e, o));
        w = f2_add(w, f2_shfl_xor(w, o));
    }
    if ((threadIdx.x & 31) == 0) {
        out->ke = make_float4(k.hi, k.lo, e.hi, e.lo);
        out->wv = make_float4(w.hi, w.lo, __uint_as_float((unsigned)vmax), __uint_as_float((unsigned)(vmax >> 32)));
    }
}

// Host: the kick's parameters for a context (integrate.cu).
struct KickArgs {
    IntParams p;
    FinParams f;
    BlockPartial* partial;  // one per block of the launch
    int partial_cap;
    StepState* st;
};

bool kick_fusable(const Context* c);
void kick_args(Context* c, KickArgs& ka);
// One block sums nparts warp partials in order and writes the step's ledger row.
void launch_ledger_finalize(Context* c, const KickArgs& ka, int nparts);

}  // namespace omdg
