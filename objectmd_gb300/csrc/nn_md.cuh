// The surrogate's per-atom descriptors from the Verlet list, shared by the
// descriptor kernel and the fused descriptor + network kernel (no reference
// counterpart).
#pragma once

#include "device_common.cuh"
#include "nn_desc.cuh"

namespace omdg {

struct NNMD {
    int n, hshift, maxnb, first;
    ShiftF L;
    float rc2;
};

// Neighbours of i inside the descriptor cutoff: vectors x_j - x_i, distances
// and list slots.  Returns the count (capped at NN_MAXN, overflow flagged).
__device__ __forceinline__ int nn_gather(const NNMD& q, const NNDescParams& p, int i, const PosPack& pi,
                                         const PosPack* __restrict__ pack, const unsigned* __restrict__ nbr, int m,
                                         float* vx, float* vy, float* vz, float* rr, int* sl, unsigned* status) {
    int nc = 0;
    for (int s = 0; s < m; s++) {
        const unsigned e = nbr[nbr_at(i, s, q.hshift, q.maxnb)];
        const PosPack pj = pack[nbr_index(e)];
        const float3 d = pair_delta(pi.hi, pi.lo, pj.hi, pj.lo, e, q.L);  // x_i - x_j
        const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
        if (!(r2 < q.rc2)) continue;
        const float r = sqrtf(r2);
        if (!(r < p.rc)) continue;
        if (nc < NN_MAXN) {
            vx[nc] = -d.x;
            vy[nc] = -d.y;
            vz[nc] = -d.z;
            rr[nc] = r;
            sl[nc] = s;
            nc++;
        } else {
            atomicOr(status, ERR_NBR_OVERFLOW);
        }
    }
    return nc;
}

// Raw descriptors g[32] of atom i (radial, then angular over its neighbour
// pairs inside the cutoff); STD: the default angular layout.
template <bool STD>
__device__ __forceinline__ void nn_md_descriptors(const NNMD& q, const NNDescParams& p, int i,
                                                  const PosPack* __restrict__ pack, const unsigned* __restrict__ nbr,
                                                  int m, float* g, unsigned* status) {
    float vx[NN_MAXN], vy[NN_MAXN], vz[NN_MAXN], rr[NN_MAXN];
    int sl[NN_MAXN];
    const int nc = nn_gather(q, p, i, pack[i], pack, nbr, m, vx, vy, vz, rr, sl, status);
#pragma unroll
    for (int k = 0; k < NN_DESC; k++) g[k] = 0.f;
    for (int a = 0; a < nc; a++) {
        float dfc;
        const float fc = nn_fc(p, rr[a], dfc);
#pragma unroll
        for (int k = 0; k < NN_RAD; k++) {
            float v, ddr;
            nn_radial(p, rr[a], fc, dfc, k, v, ddr);
            g[k] += v;
        }
    }
    for (int a = 0; a < nc; a++) {
        float dfa;
        const float fa = nn_fc(p, rr[a], dfa);
        const float ia = 1.f / rr[a];
        for (int b = a + 1; b < nc; b++) {
            float dfb;
            const float fb = nn_fc(p, rr[b], dfb);
            const float cs = (vx[a] * vx[b] + vy[a] * vy[b] + vz[a] * vz[b]) * ia / rr[b];
            const float s2 = rr[a] * rr[a] + rr[b] * rr[b];
            NNAngExp ex;
#pragma unroll
            for (int m2 = 0; m2 < NN_ANG; m2++) {
                float v, d1, d2, d3;
                nn_angular<STD>(p, m2, rr[a], rr[b], cs, fa, dfa, fb, dfb, ex.get(p.eta_a[m2], s2), v, d1, d2, d3);
                g[NN_RAD + m2] += v;
            }
        }
    }
}

// Outside the training range in any descriptor: the atom falls back to Tersoff.
__device__ __forceinline__ bool nn_out_of_range(const NNDescParams& p, const float* g) {
    bool out = false;
#pragma unroll
    for (int k = 0; k < NN_DESC; k++) out |= !(g[k] >= p.gmin[k] && g[k] <= p.gmax[k]);
    return out;
}

}  // namespace omdg
