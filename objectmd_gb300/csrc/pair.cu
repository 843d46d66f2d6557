// Tabulated pair potential (TForcePair, tpair.h:38-71): fr = -phi'(r)/r for
// r < rc (strict), ReturnForce on the owner side (forcekernel.h:92-110).
// Two precisions: FP32 on the mixed-precision relative vector (LANES threads
// per atom, Kahan partials combined by a TwoSum shuffle tree), and an FP64
// path (positions, table and accumulation in FP64) for the plain FP64
// Lennard-Jones configuration.
#include "device_common.cuh"

namespace omdg {

struct PairParams {
    int n;
    int hshift, maxnb;
    ShiftF L;
    double L64[3];
    DevTable phi;
    float rc, rc2;
    double rc64;
    int ta, tb, all_types;
    int first;
    const ShiftF* rep_L;  // replica mode: periodic lengths of each replica (else null)
    const int* rep_of;
};

__device__ __forceinline__ bool types_match(int a, int b, int ta, int tb) {
    return (a == ta && b == tb) || (a == tb && b == ta);
}

template <int LANES>
__device__ __forceinline__ void lanes_twosum(float& s, float& c) {
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
__global__ void __launch_bounds__(512) k_pair32(PairParams p, const PosPack* __restrict__ pack,
                                                const unsigned* __restrict__ nbr, const int* __restrict__ nnb,
                                                float* __restrict__ fx, float* __restrict__ fy,
                                                float* __restrict__ fz, float* __restrict__ pe,
                                                float* __restrict__ vir, unsigned* status,
                                                const unsigned* __restrict__ nbmask) {
    const int lane = threadIdx.x & (LANES - 1);
    const int per_block = blockDim.x / LANES;
    // a typed pair: the partner type(s) a centre of each type looks for
    const unsigned want_a = 1u << (p.tb & 31), want_b = 1u << (p.ta & 31);
    for (int base = blockIdx.x * per_block; base < p.n; base += gridDim.x * per_block) {
        int i = base + threadIdx.x / LANES;
        bool valid = i < p.n;
        int ii = valid ? i : p.n - 1;
        PosPack pi = pack[ii];
        int ti = pack_type(pi.hi);
        const ShiftF L = p.rep_L ? p.rep_L[p.rep_of[ii]] : p.L;
        bool any = valid && (p.all_types || ti == p.ta || ti == p.tb);
        // with the rows' type masks, a row without the partner type is skipped
        // whole (most rows of a mixed system: a Si atom with no Ar near)
        if (any && !p.all_types && nbmask)
            any = (nbmask[ii] & ((ti == p.ta ? want_a : 0u) | (ti == p.tb ? want_b : 0u))) != 0u;
        int m = any ? nnb[ii] : 0;
        Kahan ax, ay, az, ae;
        float av = 0.f;
        for (int s = lane; s < m; s += LANES) {
            unsigned e = __ldg(&nbr[nbr_at(ii, s, p.hshift, p.maxnb)]);
            int j = nbr_index(e);
            const float4* pj = reinterpret_cast<const float4*>(pack + j);
            const float4 hj = __ldg(pj);  // the type word first: most rows of a mixed system skip here
            if (!p.all_types && !types_match(ti, pack_type(hj), p.ta, p.tb)) continue;
            const float4 lj = __ldg(pj + 1);
            float3 d = pair_delta(pi.hi, pi.lo, hj, lj, e, L);
            float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
            if (r2 >= p.rc2) continue;
            float rinv = rsqrtf(r2);
            float r = r2 * rinv;
            if (!(r < p.rc)) continue;
            float ph, dph;
            tab_read(p.phi, p.phi.coef, r, rinv, ph, dph, status);
            float fr = -dph * rinv;
            ax.add(d.x * fr);
            ay.add(d.y * fr);
            az.add(d.z * fr);
            ae.add(0.5f * ph);
            av = fmaf(fr, r2, av);
        }
        lanes_twosum<LANES>(ax.s, ax.c);
        lanes_twosum<LANES>(ay.s, ay.c);
        lanes_twosum<LANES>(az.s, az.c);
        lanes_twosum<LANES>(ae.s, ae.c);
#pragma unroll
        for (int off = LANES / 2; off > 0; off >>= 1) av += __shfl_xor_sync(0xffffffffu, av, off);
        if (lane == 0 && valid) {
            float vfx = __fsub_rn(ax.s, ax.c), vfy = __fsub_rn(ay.s, ay.c), vfz = __fsub_rn(az.s, az.c);
            float ve = __fsub_rn(ae.s, ae.c);
            if (p.first) {
                fx[i] = vfx;
                fy[i] = vfy;
                fz[i] = vfz;
                pe[i] = ve;
                vir[i] = av;
            } else if (m) {
                fx[i] += vfx;
                fy[i] += vfy;
                fz[i] += vfz;
                pe[i] += ve;
                vir[i] += av;
            }
        }
    }
}

// FP64 end to end: dx = x_i - (x_j + s), r = sqrt(r2), TableReader in FP64.
// PAIR64_LANES lanes per atom take every PAIR64_LANES-th row entry, and the
// lanes' FP64 sums meet in a fixed xor tree, so the FP64 work of a small box
// spreads over the whole chip (one thread per atom left most SMs idle).
constexpr int PAIR64_LANES = 32;

__global__ void __launch_bounds__(128) k_pair64(PairParams p, const double* __restrict__ x,
                                                const double* __restrict__ y, const double* __restrict__ z,
                                                const int* __restrict__ type, const unsigned* __restrict__ nbr,
                                                const int* __restrict__ nnb, double* __restrict__ f64,
                                                float* __restrict__ pe, float* __restrict__ vir, unsigned* status) {
    const int lane = threadIdx.x & (PAIR64_LANES - 1);
    const int i = blockIdx.x * (blockDim.x / PAIR64_LANES) + threadIdx.x / PAIR64_LANES;
    if (i >= p.n) return;  // whole warps leave together
    const int ti = type[i];
    const double xi = x[i], yi = y[i], zi = z[i];
    double ax = 0, ay = 0, az = 0, ae = 0, av = 0;
    const bool any = p.all_types || ti == p.ta || ti == p.tb;
    const int m = any ? nnb[i] : 0;
    for (int s = lane; s < m; s += PAIR64_LANES) {
        const unsigned e = __ldg(&nbr[nbr_at(i, s, p.hshift, p.maxnb)]);
        const int j = nbr_index(e);
        if (!p.all_types && !types_match(ti, type[j], p.ta, p.tb)) continue;
        const int sx = nbr_sx(e), sy = nbr_sy(e), sz = nbr_sz(e);
        const double gx = __dadd_rn(x[j], sx == 0 ? 0.0 : (sx > 0 ? p.L64[0] : -p.L64[0]));
        const double gy = __dadd_rn(y[j], sy == 0 ? 0.0 : (sy > 0 ? p.L64[1] : -p.L64[1]));
        const double gz = __dadd_rn(z[j], sz == 0 ? 0.0 : (sz > 0 ? p.L64[2] : -p.L64[2]));
        const double dx = __dsub_rn(xi, gx), dy = __dsub_rn(yi, gy), dz = __dsub_rn(zi, gz);
        const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
        const double r = __dsqrt_rn(r2);
        if (!(r < p.rc64)) continue;
        double ph, dph;
        tab_read64(p.phi, r, ph, dph, status);
        const double fr = __ddiv_rn(-dph, r);
        ax = __dadd_rn(ax, __dmul_rn(dx, fr));
        ay = __dadd_rn(ay, __dmul_rn(dy, fr));
        az = __dadd_rn(az, __dmul_rn(dz, fr));
        ae = __dadd_rn(ae, __dmul_rn(0.5, ph));
        av = __dadd_rn(av, __dmul_rn(fr, r2));
    }
    for (int o = PAIR64_LANES / 2; o > 0; o >>= 1) {
        ax += __shfl_xor_sync(0xffffffffu, ax, o);
        ay += __shfl_xor_sync(0xffffffffu, ay, o);
        az += __shfl_xor_sync(0xffffffffu, az, o);
        ae += __shfl_xor_sync(0xffffffffu, ae, o);
        av += __shfl_xor_sync(0xffffffffu, av, o);
    }
    if (lane != 0) return;
    if (p.first) {
        f64[3 * (size_t)i + 0] = ax;
        f64[3 * (size_t)i + 1] = ay;
        f64[3 * (size_t)i + 2] = az;
        pe[i] = (float)ae;
        vir[i] = (float)av;
        f64[3 * (size_t)p.n + i] = ae;
    } else if (m) {
        f64[3 * (size_t)i + 0] += ax;
        f64[3 * (size_t)i + 1] += ay;
        f64[3 * (size_t)i + 2] += az;
        pe[i] += (float)ae;
        vir[i] += (float)av;
        f64[3 * (size_t)p.n + i] += ae;
    }
}

template <int LANES>
static void launch32(Context* c, const PairParams& p, int block) {
    int per_block = block / LANES;
    k_pair32<LANES><<<grid_for(c->n, per_block), block, 0, c->stream>>>(
        p, c->pack, reinterpret_cast<const unsigned*>(c->nbr), c->nnb, c->fx, c->fy, c->fz, c->pe, c->vir,
        c->d_status, c->nbmask_valid ? c->nbmask : nullptr);
}

int pair_launch(Context* c, Potential& pot, bool first) {
    PairParams p;
    p.n = c->n;
    p.hshift = c->nbr_hshift;
    p.maxnb = c->maxnb;
    p.L = make_shift(c->box);
    for (int d = 0; d < 3; d++) p.L64[d] = c->box.L[d];
    p.phi = pot.dt[0];
    p.rc64 = pot.t0.max_range();
    p.rc = (float)p.rc64;
    p.rc2 = p.rc * p.rc * 1.0001f;
    p.ta = pot.ta;
    p.tb = pot.tb;
    p.all_types = c->ntypes == 1 ? 1 : 0;
    p.first = first ? 1 : 0;
    p.rep_L = c->nrep > 0 ? static_cast<const ShiftF*>(c->d_rep_shift) : nullptr;
    p.rep_of = c->nrep > 0 ? c->d_rep_of : nullptr;
    if (pot.fp64 && c->nrep > 0) return set_error(c, OMDG_EINVAL, "replica mode has no FP64 pair kernel");
    int block = c->pair_block;
    if (pot.fp64) {
        prof_begin(c, "pair64");
        k_pair64<<<grid_for(c->n, 128 / PAIR64_LANES), 128, 0, c->stream>>>(p, c->x, c->y, c->z, c->type,
                                                              reinterpret_cast<const unsigned*>(c->nbr), c->nnb,
                                                              c->f64, c->pe, c->vir, c->d_status);
    } else {
        prof_begin(c, "pair32");
        switch (c->pair_lanes) {
            case 1: launch32<1>(c, p, block); break;
            case 2: launch32<2>(c, p, block); break;
            case 4: launch32<4>(c, p, block); break;
            case 8: launch32<8>(c, p, block); break;
            case 16: launch32<16>(c, p, block); break;
            default: launch32<32>(c, p, block); break;
        }
    }
    prof_end(c);
    c->launches++;
    return check_cuda(c, cudaGetLastError(), "pair");
}

}  // namespace omdg
