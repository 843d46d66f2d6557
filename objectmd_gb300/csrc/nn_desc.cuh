// Descriptor terms of the neural surrogate (FP32), shared by the training
// kernels (which store the Jacobian) and the MD kernels (which contract it
// with dE/dG on the fly).  Behler-Parrinello radial G2 and angular G5 terms
// (J. Behler, J. Chem. Phys. 134, 074106 (2011)).  The exponentials and the
// cutoff's sine and cosine use the hardware approximations (__expf,
// __sincosf: a few 1e-7 relative for the arguments met here), far below the
// BF16 rounding of the network's input.
#pragma once

#include "nn_internal.h"

namespace omdg {

__device__ __forceinline__ float nn_fc(const NNDescParams& p, float r, float& dfc) {
    if (r <= p.rin) {
        dfc = 0.f;
        return 1.f;
    }
    float s, c;
    __sincosf((r - p.rin) * p.pi_rc, &s, &c);
    dfc = -0.5f * p.pi_rc * s;
    return 0.5f * (c + 1.f);
}

// b^z for a small non-negative integer z (square and multiply)
__device__ __forceinline__ float nn_ipow(float b, int z) {
    float r = 1.f;
    while (z > 0) {
        if (z & 1) r *= b;
        b *= b;
        z >>= 1;
    }
    return r;
}

// Radial terms of one neighbour at distance r: value g[k] fc and dG_k/dr.
__device__ __forceinline__ void nn_radial(const NNDescParams& p, float r, float fc, float dfc, int k, float& val,
                                          float& ddr) {
    const float x = r - p.rs[k];
    const float g = __expf(-p.eta_r[k] * x * x);
    val = g * fc;
    ddr = g * (dfc - 2.f * p.eta_r[k] * x * fc);
}

// exp(-eta (r_a^2 + r_b^2)) of the angular terms, recomputed only when eta
// changes from one term to the next (the descriptor set groups its terms by
// eta, so a pair takes one exponential per distinct eta, not one per term).
struct NNAngExp {
    float eta = -1.f, ex = 1.f;
    __device__ __forceinline__ float get(float e, float s2) {
        if (e != eta) {
            eta = e;
            ex = e == 0.f ? 1.f : __expf(-e * s2);
        }
        return ex;
    }
};

// The default angular set's layout: term m has zeta 2^((m >> 1) & 3) and
// lambda +1 for even m, -1 for odd m (two eta groups of eight).  Kernels
// built for it (STD) take zeta and lambda as constants of the unrolled term
// loop, so the powers of the two bases 1 +- cos are formed once per pair and
// shared by the terms (the same products in the same order as nn_ipow).
__host__ __device__ constexpr int nn_std_zeta(int m) { return 1 << ((m >> 1) & 3); }
__host__ __device__ constexpr float nn_std_lam(int m) { return (m & 1) ? -1.f : 1.f; }

inline bool nn_std_angular(const NNDescParams& p) {
    for (int m = 0; m < NN_ANG; m++)
        if (p.zeta[m] != nn_std_zeta(m) || p.lam[m] != nn_std_lam(m)) return false;
    return true;
}

// Angular term m of the neighbour pair (a, b): the value and its derivatives
// with respect to r_a, r_b and cos(theta); ex = exp(-eta_a[m] (r_a^2 + r_b^2)).
template <bool STD = false>
__device__ __forceinline__ void nn_angular(const NNDescParams& p, int m, float ra, float rb, float cs, float fa,
                                           float dfa, float fb, float dfb, float ex, float& val, float& d_ra,
                                           float& d_rb, float& d_cs) {
    const float lam = STD ? nn_std_lam(m) : p.lam[m];
    float base = 1.f + lam * cs;
    base = base > 0.f ? base : 0.f;
    const int z = STD ? nn_std_zeta(m) : p.zeta[m];
    const float pm1 = nn_ipow(base, z - 1);
    const float pw = pm1 * base;
    const float k = p.pref[m] * ex;
    val = k * pw * fa * fb;
    d_ra = k * pw * fb * (dfa - 2.f * p.eta_a[m] * ra * fa);
    d_rb = k * pw * fa * (dfb - 2.f * p.eta_a[m] * rb * fb);
    d_cs = base > 0.f ? k * (float)z * pm1 * lam * fa * fb : 0.f;
}

}  // namespace omdg
