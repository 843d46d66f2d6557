// Tabulated EAM (TEmbedding + TForceEAM, team.cpp:68-237) as two kernels
// over the full Verlet list, owner-computes (no atomics, deterministic):
//
//   eam_density  rho_i = sum_j rho(r_ij) for r <= rc_rho   (team.cpp:81-92)
//                then F(rho_i), F'(rho_i) from the EMBED table  (team.cpp:116-145)
//   eam_force    fr = -(F'_i rho'(r) + F'_j rho'(r) + phi'(r)) / r  (team.cpp:224-237)
//                f_i += fr d, potential_i += phi/2 + F(rho_i), virial_i += fr r^2
//                (ReturnForce, forcekernel.h:92-110, on the owner side only)
//
// GB300 mapping: LANES threads share one atom and stride over its
// sliced-ELL row, so a warp keeps 32 independent neighbour gathers in
// flight; partial sums are Kahan accumulators combined across the lanes
// with a TwoSum shuffle tree.  CTAs are persistent (a grid sized to the SM
// count) and stage the PAIR and EDENS spline knots of [r_stage, rc] in
// shared memory once, interleaved so one knot index fetches both tables.
// Arithmetic is FP32 on relative vectors from the FP64 positions.
#include "device_common.cuh"

namespace omdg {

struct EAMParams {
    int n;
    int hshift, maxnb;
    ShiftF L;
    DevTable phi, rho, emb;
    const float4* coef2;    // interleaved (phi knot k, rho knot k) when the grids agree
    int same_grid;
    float rc_phi, rc_rho;   // max_range of PAIR and EDENS
    float rc2_screen;       // slightly above max(rc_phi, rc_rho)^2
    int single_type;        // all atoms are of the EAM type
    int type_a;
    int stage_k0, stage_n;  // knots [k0, k0+n) live in shared memory
    int first;              // 1: write outputs, 0: accumulate
};

template <int LANES>
__device__ __forceinline__ void lane_reduce(float& s, float& c) {
#pragma unroll
    for (int off = LANES / 2; off > 0; off >>= 1) {
        float s2 = __shfl_xor_sync(0xffffffffu, s, off);
        float c2 = __shfl_xor_sync(0xffffffffu, c, off);
        // TwoSum(s, s2) = t + e exactly; the lost part joins the compensation
        float t = __fadd_rn(s, s2);
        float bp = __fsub_rn(t, s);
        float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(s2, bp));
        c = __fsub_rn(__fadd_rn(c, c2), e);
        s = t;
    }
}

// Knot index and offset by the reference rule (treader.cpp:195-221); returns
// false if the read is out of range (status set unless the table allows it).
__device__ __forceinline__ int knot(const DevTable& t, float r, float& dx, int& state) {
    float rval = r - t.off;
    int x = (int)(rval * t.inv_dr);
    dx = fmaf(-(float)x, t.dr, rval);
    state = 0;
    if ((unsigned)x < (unsigned)(t.n - 1)) return x;
    if (x > t.n - 1) {
        state = t.allow_hi ? 2 : 3;
        return 0;
    }
    if (x < -1) {
        state = t.allow_lo ? 1 : 3;
        return 0;
    }
    if (x == t.n - 1) {
        dx += t.dr;
        return x - 1;
    }
    return 0;  // x == -1
}

__device__ __forceinline__ void cubic(const float4& cf, float dx, float& v, float& dv) {
    v = fmaf(dx, fmaf(dx, fmaf(dx, cf.x, cf.y), cf.z), cf.w);
    dv = fmaf(dx, fmaf(3.0f * dx, cf.x, 2.0f * cf.y), cf.z);
}

template <int LANES>
__global__ void __launch_bounds__(512) k_eam_density(EAMParams p, const PosPack* __restrict__ pack,
                                                     const unsigned* __restrict__ nbr, const int* __restrict__ nnb,
                                                     float* __restrict__ fp, float* __restrict__ femb,
                                                     unsigned* status) {
    extern __shared__ float4 s_tab[];  // rho knots [k0, k0+ns) (stride 2 when interleaved)
    const int stride = p.same_grid ? 2 : 1;
    const float4* g_rho = p.same_grid ? p.coef2 + 1 : p.rho.coef;
    for (int k = threadIdx.x; k < p.stage_n; k += blockDim.x) s_tab[k] = g_rho[(size_t)stride * (p.stage_k0 + k)];
    __syncthreads();
    const int lane = threadIdx.x & (LANES - 1);
    const int per_block = blockDim.x / LANES;
    const float rc2 = p.rc_rho * p.rc_rho * 1.0001f;
    for (int base = blockIdx.x * per_block; base < p.n; base += gridDim.x * per_block) {
        int i = base + threadIdx.x / LANES;
        bool valid = i < p.n;
        int ii = valid ? i : p.n - 1;
        PosPack pi = pack[ii];
        bool mine = valid && (p.single_type || pack_type(pi.hi) == p.type_a);
        int m = mine ? nnb[ii] : 0;
        Kahan acc;
        int bad = 0;
        for (int s = lane; s < m; s += LANES) {
            unsigned e = __ldg(&nbr[nbr_at(ii, s, p.hshift, p.maxnb)]);
            int j = nbr_index(e);
            const float4* pj = reinterpret_cast<const float4*>(pack + j);
            float4 hj = __ldg(pj), lj = __ldg(pj + 1);
            if (!p.single_type && pack_type(hj) != p.type_a) continue;
            float3 d = pair_delta(pi.hi, pi.lo, hj, lj, e, p.L);
            float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
            if (r2 > rc2) continue;
            float r = r2 * rsqrtf(r2);
            if (!(r <= p.rc_rho)) continue;
            float dx;
            int st;
            int x = knot(p.rho, r, dx, st);
            if (st) {
                if (st == 3) {
                    if (!bad) report_range(status, r, p.rho.src);
                    bad = 1;
                } else {
                    acc.add(st == 1 ? p.rho.out_lo : p.rho.out_hi);
                }
                continue;
            }
            int xs = x - p.stage_k0;
            float4 cf = ((unsigned)xs < (unsigned)p.stage_n) ? s_tab[xs] : __ldg(&g_rho[(size_t)stride * x]);
            float v, dv;
            cubic(cf, dx, v, dv);
            if (p.rho.rmult) v = v / r;
            acc.add(v);
        }
        float s = acc.s, c = acc.c;
        lane_reduce<LANES>(s, c);
        if (lane == 0 && valid) {
            if (mine) {
                float rho = __fsub_rn(s, c);
                float F, dF;
                tab_value(p.emb, p.emb.coef, rho, F, dF, status);
                fp[i] = dF;
                femb[i] = F;
            } else {
                fp[i] = 0.f;
                femb[i] = 0.f;
            }
        }
    }
}

template <int LANES>
__global__ void __launch_bounds__(512) k_eam_force(EAMParams p, const PosPack* __restrict__ pack,
                                                   const unsigned* __restrict__ nbr, const int* __restrict__ nnb,
                                                   const float* __restrict__ fp, const float* __restrict__ femb,
                                                   float* __restrict__ fx, float* __restrict__ fy,
                                                   float* __restrict__ fz, float* __restrict__ pe,
                                                   float* __restrict__ vir, unsigned* status) {
    extern __shared__ float4 s_tab[];  // interleaved (phi, rho) knots [k0, k0+ns)
    if (p.same_grid)
        for (int k = threadIdx.x; k < 2 * p.stage_n; k += blockDim.x) s_tab[k] = p.coef2[2 * (size_t)p.stage_k0 + k];
    __syncthreads();
    const int lane = threadIdx.x & (LANES - 1);
    const int per_block = blockDim.x / LANES;
    for (int base = blockIdx.x * per_block; base < p.n; base += gridDim.x * per_block) {
        int i = base + threadIdx.x / LANES;
        bool valid = i < p.n;
        int ii = valid ? i : p.n - 1;
        PosPack pi = pack[ii];
        bool mine = valid && (p.single_type || pack_type(pi.hi) == p.type_a);
        int m = mine ? nnb[ii] : 0;
        float fpi = mine ? fp[ii] : 0.f;
        Kahan ax, ay, az, ae;
        float av = 0.f;
        int bad = 0;
        for (int s = lane; s < m; s += LANES) {
            unsigned e = __ldg(&nbr[nbr_at(ii, s, p.hshift, p.maxnb)]);
            int j = nbr_index(e);
            const float4* pj = reinterpret_cast<const float4*>(pack + j);
            float4 hj = __ldg(pj), lj = __ldg(pj + 1);
            if (!p.single_type && pack_type(hj) != p.type_a) continue;
            float fpj = __ldg(&fp[j]);
            float3 d = pair_delta(pi.hi, pi.lo, hj, lj, e, p.L);
            float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
            if (r2 > p.rc2_screen) continue;
            float rinv = rsqrtf(r2);
            float r = r2 * rinv;
            if (!(r <= p.rc_phi)) continue;
            float ph, dph, drho = 0.f;
            if (p.same_grid) {
                float dx;
                int st;
                int x = knot(p.phi, r, dx, st);
                if (st) {
                    // out-of-range reads keep the reference's OutOfRange values
                    if (st == 3) {
                        if (!bad) report_range(status, r, p.phi.src);
                        bad = 1;
                    }
                    ph = dph = st == 1 ? p.phi.out_lo : p.phi.out_hi;
                    if (!(r > p.rc_rho)) drho = st == 1 ? p.rho.out_lo : p.rho.out_hi;
                } else {
                    int xs = x - p.stage_k0;
                    float4 c_phi, c_rho;
                    if ((unsigned)xs < (unsigned)p.stage_n) {
                        c_phi = s_tab[2 * xs];
                        c_rho = s_tab[2 * xs + 1];
                    } else {
                        c_phi = __ldg(&p.coef2[2 * (size_t)x]);
                        c_rho = __ldg(&p.coef2[2 * (size_t)x + 1]);
                    }
                    cubic(c_phi, dx, ph, dph);
                    if (p.phi.rmult) {
                        ph = ph * rinv;
                        dph = (dph - ph) * rinv;
                    }
                    if (!(r > p.rc_rho)) {
                        float rv;
                        cubic(c_rho, dx, rv, drho);
                        if (p.rho.rmult) drho = (drho - rv * rinv) * rinv;
                    }
                }
            } else {
                if (!tab_read(p.phi, p.phi.coef, r, rinv, ph, dph, status)) bad = 1;
                if (!(r > p.rc_rho)) {
                    float rv;
                    if (!tab_read(p.rho, p.rho.coef, r, rinv, rv, drho, status)) bad = 1;
                }
            }
            float fr = -((fpi * drho + fpj * drho) + dph) * rinv;
            ax.add(d.x * fr);
            ay.add(d.y * fr);
            az.add(d.z * fr);
            ae.add(0.5f * ph);
            av = fmaf(fr, r2, av);
        }

        lane_reduce<LANES>(ax.s, ax.c);
        lane_reduce<LANES>(ay.s, ay.c);
        lane_reduce<LANES>(az.s, az.c);
        if (lane == 0 && mine) ae.add(femb[i]);
        lane_reduce<LANES>(ae.s, ae.c);
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
            } else {
                fx[i] += vfx;
                fy[i] += vfy;
                fz[i] += vfz;
                pe[i] += ve;
                vir[i] += av;
            }
        }
    }
}

template <int LANES>
static void launch_pair_of_kernels(Context* c, const EAMParams& p, int grid, int block, size_t smem1, size_t smem2) {
    prof_begin(c, "eam_density");
    k_eam_density<LANES><<<grid, block, smem1, c->stream>>>(p, c->pack, reinterpret_cast<const unsigned*>(c->nbr),
                                                             c->nnb, c->fp, c->femb, c->d_status);
    prof_end(c);
    prof_begin(c, "eam_force");
    k_eam_force<LANES><<<grid, block, smem2, c->stream>>>(p, c->pack, reinterpret_cast<const unsigned*>(c->nbr),
                                                           c->nnb, c->fp, c->femb, c->fx, c->fy, c->fz, c->pe,
                                                           c->vir, c->d_status);
    prof_end(c);
}

template <int LANES>
static void set_smem_attr() {
    static bool done = false;
    if (done) return;
    cudaFuncSetAttribute(k_eam_force<LANES>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    cudaFuncSetAttribute(k_eam_density<LANES>, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    done = true;
}

int eam_prepare(Context* c, Potential& pot) {
    // interleaved (phi, rho) knots when PAIR and EDENS share a grid
    bool same = pot.t0.n == pot.t1.n && pot.t0.dr == pot.t1.dr && pot.t0.off == pot.t1.off &&
                pot.t0.allow_lo == pot.t1.allow_lo && pot.t0.allow_hi == pot.t1.allow_hi;
    if (!same || pot.d_coef2) return OMDG_OK;
    std::vector<float4> h(2 * (size_t)pot.t0.n);
    for (int i = 0; i < pot.t0.n; i++) {
        h[2 * i] = make_float4((float)pot.t0.a[i], (float)pot.t0.b[i], (float)pot.t0.c[i], (float)pot.t0.d[i]);
        h[2 * i + 1] = make_float4((float)pot.t1.a[i], (float)pot.t1.b[i], (float)pot.t1.c[i], (float)pot.t1.d[i]);
    }
    if (cudaMalloc(&pot.d_coef2, sizeof(float4) * h.size()) != cudaSuccess)
        return set_error(c, OMDG_ENOMEM, "EAM table");
    cudaMemcpy(pot.d_coef2, h.data(), sizeof(float4) * h.size(), cudaMemcpyHostToDevice);
    return OMDG_OK;
}

bool eam_fast_ok(const Context* c, const Potential& pot);
int eam_fast_launch(Context* c, Potential& pot, bool first);

int eam_launch(Context* c, Potential& pot, bool first) {
    int rc = eam_prepare(c, pot);
    if (rc) return rc;
    if (eam_fast_ok(c, pot)) return eam_fast_launch(c, pot, first);
    EAMParams p;
    p.n = c->n;
    p.hshift = c->nbr_hshift;
    p.maxnb = c->maxnb;
    p.L = make_shift(c->box);
    p.phi = pot.dt[0];
    p.rho = pot.dt[1];
    p.emb = pot.dt[2];
    p.coef2 = pot.d_coef2;
    p.same_grid = pot.d_coef2 ? 1 : 0;
    p.rc_phi = (float)pot.t0.max_range();
    p.rc_rho = (float)pot.t1.max_range();
    float rcm = p.rc_phi > p.rc_rho ? p.rc_phi : p.rc_rho;
    p.rc2_screen = rcm * rcm * 1.0001f;
    p.single_type = (c->ntypes == 1) ? 1 : 0;
    p.type_a = pot.ta;
    p.first = first ? 1 : 0;
    // staged window: knots from r = stage_frac * rc to the end of the table
    int k0 = 0, ns = 0;
    if (p.same_grid && c->eam_stage) {
        k0 = (int)((c->eam_stage_frac * pot.t1.max_range() - pot.t1.off) / pot.t1.dr);
        if (k0 < 0) k0 = 0;
        ns = pot.t1.n - k0;
        int max_stage = (200 * 1024) / (2 * (int)sizeof(float4));
        if (ns > max_stage) {
            k0 = pot.t1.n - max_stage;
            ns = max_stage;
        }
    }
    p.stage_k0 = k0;
    p.stage_n = ns;
    int block = c->eam_block;
    int lanes = c->eam_lanes;
    int per_block = block / lanes;
    int want = grid_for(c->n, per_block);
    int grid = want;
    if (ns > 0) {
        int per_sm = c->eam_ctas_per_sm > 0 ? c->eam_ctas_per_sm : 1;
        int cap = c->num_sms * per_sm;
        grid = want < cap ? want : cap;
    }
    size_t smem1 = (size_t)ns * sizeof(float4);
    size_t smem2 = 2 * smem1;
    switch (lanes) {
        case 1: set_smem_attr<1>(); launch_pair_of_kernels<1>(c, p, grid, block, smem1, smem2); break;
        case 2: set_smem_attr<2>(); launch_pair_of_kernels<2>(c, p, grid, block, smem1, smem2); break;
        case 4: set_smem_attr<4>(); launch_pair_of_kernels<4>(c, p, grid, block, smem1, smem2); break;
        case 8: set_smem_attr<8>(); launch_pair_of_kernels<8>(c, p, grid, block, smem1, smem2); break;
        case 16: set_smem_attr<16>(); launch_pair_of_kernels<16>(c, p, grid, block, smem1, smem2); break;
        default: set_smem_attr<32>(); launch_pair_of_kernels<32>(c, p, grid, block, smem1, smem2); break;
    }
    c->launches += 2;
    return check_cuda(c, cudaGetLastError(), "eam");
}

}  // namespace omdg
