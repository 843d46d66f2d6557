// Tabulated EAM (TEmbedding + TForceEAM, team.cpp:68-237) as two kernels
// over the full Verlet list, owner-computes (no atomics, deterministic):
//
//   eam_density  rho_i = sum_j rho(r_ij) for r <= rc_rho   (team.cpp:81-92)
//                then F(rho_i), F'(rho_i) from the EMBED table  (team.cpp:116-145)
//   eam_force    fr = -(F'_i rho'(r) + F'_j rho'(r) + phi'(r)) / r  (team.cpp:224-237)
//                f_i += fr d, potential_i += phi/2 + F(rho_i), virial_i += fr r^2
//                (ReturnForce, forcekernel.h:92-110, on the owner side only)
//
// FP32 arithmetic on relative vectors from the FP64 positions (pair_delta),
// spline coefficients staged in shared memory per block (the knots that
// cover [r_stage, rc]; closer pairs read the L1-cached global copy), Kahan
// sums for rho, force, energy and virial.
#include "device_common.cuh"

namespace omdg {

struct EAMParams {
    int n;
    ShiftF L;
    DevTable phi, rho, emb;
    float rc_phi, rc_rho;   // max_range of PAIR and EDENS
    float rc2_screen;       // slightly above max(rc_phi, rc_rho)^2
    int single_type;        // all atoms are of this EAM type
    int type_a;
    int stage_k0, stage_n;  // knots [k0, k0+n) of the PAIR/EDENS tables are in shared memory
    int first;              // 1: write outputs, 0: accumulate
};

constexpr int EAM_BLOCK = 512;  // upper bound; the launch block size is tunable

// Reads knot k of a table from shared memory when it is staged, else global.
__device__ __forceinline__ const float4* knot_base(const float4* smem, const float4* gmem, int k0, int ns, int x) {
    return (x >= k0 && x < k0 + ns) ? smem - k0 : gmem;
}

__device__ __forceinline__ bool tab_read_staged(const DevTable& t, const float4* smem, int k0, int ns, float r,
                                                float rinv, float& v, float& dv, unsigned* status) {
    float rval = r - t.off;
    int x = (int)(rval * t.inv_dr);
    // pick the coefficient source for the knot the read will use
    int xx = x == t.n - 1 ? x - 1 : (x == -1 ? 0 : x);
    const float4* base = knot_base(smem, t.coef, k0, ns, xx);
    DevTable tt = t;
    tt.coef = base;
    return tab_read(tt, base, r, rinv, v, dv, status);
}

__global__ void __launch_bounds__(EAM_BLOCK) k_eam_density(EAMParams p, const PosPack* __restrict__ pack,
                                                           const unsigned* __restrict__ nbr,
                                                           const int* __restrict__ nnb, float* __restrict__ fp,
                                                           float* __restrict__ femb, unsigned* status) {
    extern __shared__ float4 s_rho[];
    for (int k = threadIdx.x; k < p.stage_n; k += blockDim.x) s_rho[k] = p.rho.coef[p.stage_k0 + k];
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    PosPack pi = pack[i];
    int ti = pack_type(pi.hi);
    if (!p.single_type && ti != p.type_a) {
        fp[i] = 0.f;
        femb[i] = 0.f;
        return;
    }
    int m = nnb[i];
    float rc2 = p.rc_rho * p.rc_rho * 1.0001f;
    Kahan acc;
    for (int s = 0; s < m; s++) {
        unsigned e = __ldg(&nbr[(size_t)s * p.n + i]);
        int j = nbr_index(e);
        const float4* pj = reinterpret_cast<const float4*>(pack + j);
        float4 hj = __ldg(pj), lj = __ldg(pj + 1);
        if (!p.single_type && pack_type(hj) != p.type_a) continue;
        float3 d = pair_delta(pi.hi, pi.lo, hj, lj, e, p.L);
        float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
        if (r2 > rc2) continue;
        float rinv = rsqrtf(r2);
        float r = r2 * rinv;
        if (!(r <= p.rc_rho)) continue;
        float v, dv;
        tab_read_staged(p.rho, s_rho, p.stage_k0, p.stage_n, r, rinv, v, dv, status);
        acc.add(v);
    }
    float rho = acc.value();
    float F, dF;
    tab_value(p.emb, p.emb.coef, rho, F, dF, status);
    fp[i] = dF;
    femb[i] = F;
}

__global__ void __launch_bounds__(EAM_BLOCK) k_eam_force(EAMParams p, const PosPack* __restrict__ pack,
                                                         const unsigned* __restrict__ nbr, const int* __restrict__ nnb,
                                                         const float* __restrict__ fp,
                                                         const float* __restrict__ femb, float* __restrict__ fx,
                                                         float* __restrict__ fy, float* __restrict__ fz,
                                                         float* __restrict__ pe, float* __restrict__ vir,
                                                         unsigned* status) {
    extern __shared__ float4 s_tab[];
    float4* s_phi = s_tab;
    float4* s_rho = s_tab + p.stage_n;
    for (int k = threadIdx.x; k < p.stage_n; k += blockDim.x) {
        s_phi[k] = p.phi.coef[p.stage_k0 + k];
        s_rho[k] = p.rho.coef[p.stage_k0 + k];
    }
    __syncthreads();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    PosPack pi = pack[i];
    int ti = pack_type(pi.hi);
    bool mine = p.single_type || ti == p.type_a;
    Kahan ax, ay, az, ae, av;
    if (mine) {
        float fpi = fp[i];
        int m = nnb[i];
        for (int s = 0; s < m; s++) {
            unsigned e = __ldg(&nbr[(size_t)s * p.n + i]);
            int j = nbr_index(e);
            const float4* pj = reinterpret_cast<const float4*>(pack + j);
            float4 hj = __ldg(pj), lj = __ldg(pj + 1);
            if (!p.single_type && pack_type(hj) != p.type_a) continue;
            float3 d = pair_delta(pi.hi, pi.lo, hj, lj, e, p.L);
            float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
            if (r2 > p.rc2_screen) continue;
            float rinv = rsqrtf(r2);
            float r = r2 * rinv;
            if (!(r <= p.rc_phi)) continue;
            float ph, dph;
            tab_read_staged(p.phi, s_phi, p.stage_k0, p.stage_n, r, rinv, ph, dph, status);
            float drho = 0.f;
            if (!(r > p.rc_rho)) {
                float rv;
                tab_read_staged(p.rho, s_rho, p.stage_k0, p.stage_n, r, rinv, rv, drho, status);
            }
            float fpj = __ldg(&fp[j]);
            float fr = -((fpi * drho + fpj * drho) + dph) * rinv;
            ax.add(d.x * fr);
            ay.add(d.y * fr);
            az.add(d.z * fr);
            ae.add(0.5f * ph);
            av.add(fr * r2);
        }
        ae.add(femb[i]);
    }
    if (p.first) {
        fx[i] = ax.value();
        fy[i] = ay.value();
        fz[i] = az.value();
        pe[i] = ae.value();
        vir[i] = av.value();
    } else {
        fx[i] += ax.value();
        fy[i] += ay.value();
        fz[i] += az.value();
        pe[i] += ae.value();
        vir[i] += av.value();
    }
}

int eam_launch(Context* c, Potential& pot, bool first) {
    EAMParams p;
    p.n = c->n;
    p.L = make_shift(c->box);
    p.phi = pot.dt[0];
    p.rho = pot.dt[1];
    p.emb = pot.dt[2];
    p.rc_phi = (float)pot.t0.max_range();
    p.rc_rho = (float)pot.t1.max_range();
    float rcm = p.rc_phi > p.rc_rho ? p.rc_phi : p.rc_rho;
    p.rc2_screen = rcm * rcm * 1.0001f;
    p.single_type = (c->ntypes == 1) ? 1 : 0;
    p.type_a = pot.ta;
    p.first = first ? 1 : 0;
    // stage the knots from r = 0.35 rc upward (PAIR and EDENS share a grid in
    // the reference tables; when they do not, only the density table's own
    // staging is used and reads fall back to global memory)
    bool same_grid = pot.t0.n == pot.t1.n && pot.t0.dr == pot.t1.dr && pot.t0.off == pot.t1.off;
    int n_knots = pot.t1.n;
    int k0 = (int)((0.35 * pot.t1.max_range() - pot.t1.off) / pot.t1.dr);
    if (k0 < 0) k0 = 0;
    int ns = n_knots - k0;
    int max_stage = (96 * 1024) / (2 * (int)sizeof(float4));
    if (ns > max_stage) {
        k0 = n_knots - max_stage;
        ns = max_stage;
    }
    if (!same_grid || !c->eam_stage) ns = 0;
    p.stage_k0 = k0;
    p.stage_n = ns;
    int block = c->eam_block;
    int grid = grid_for(c->n, block);
    size_t smem1 = (size_t)ns * sizeof(float4);
    size_t smem2 = 2 * smem1;
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_eam_force, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(k_eam_density, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr_set = true;
    }
    prof_begin(c, "eam_density");
    k_eam_density<<<grid, block, smem1, c->stream>>>(p, c->pack, reinterpret_cast<const unsigned*>(c->nbr),
                                                          c->nnb, c->fp, c->femb, c->d_status);
    prof_end(c);
    prof_begin(c, "eam_force");
    k_eam_force<<<grid, block, smem2, c->stream>>>(p, c->pack, reinterpret_cast<const unsigned*>(c->nbr),
                                                        c->nnb, c->fp, c->femb, c->fx, c->fy, c->fz, c->pe, c->vir,
                                                        c->d_status);
    prof_end(c);
    c->launches += 2;
    return check_cuda(c, cudaGetLastError(), "eam");
}

}  // namespace omdg
