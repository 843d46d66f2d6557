// Three-body potentials, owner-computes in two passes over the full Verlet
// list (no atomics, deterministic):
//
//   pass A  for atom i: every term centred on i -- the two-body halves of
//           i's pairs and the triplets (SW, sw.cpp:166-236) or bonds
//           (Tersoff) whose centre is i.  The force and energy a term gives
//           to i accumulate in registers; what it gives to a neighbour j is
//           written to j's slot in i's row of a per-slot buffer.
//   pass B  for atom i: own part + sum over i's slots s of the buffer entry
//           its neighbour j wrote for i (slot rev(i,s) of j's row).
//
// FP32 arithmetic on relative vectors from the FP64 positions, Kahan sums in
// pass B.  Per-atom energies follow the reference: each pair half to each
// atom, V3/3 to each triplet member (sw.cpp:182-233); Tersoff: 1/2 V_ij to i.
#include <cmath>

#include "device_common.cuh"

namespace omdg {

constexpr int TB_MAXN = 24;  // neighbours within the cutoff one atom can hold

// f(b) for the in-cutoff neighbours b < nc: fully unrolled over K (the
// arrays f touches stay in registers), or a rolled loop over local arrays
// (then the kernel's register count stays that of the unrolled path).
template <int K, bool UNR, class F>
__device__ __forceinline__ void for_nbrs(int nc, F&& f) {
    if constexpr (UNR) {
#pragma unroll
        for (int b = 0; b < K; b++)
            if (b < nc) f(b);
    } else {
#pragma unroll 1
        for (int b = 0; b < nc; b++) f(b);
    }
}


struct SWDev {
    int n, hshift, maxnb, single_type, ta;
    ShiftF L;
    float rc, rc2;
    float A, B, p, q, sigma, eps;
    float c1, c2, c3, c4, c5, c6, c7, c8, c9, c10;
    int usezbl;
    float sx0, sx1, sa0, sa1, sa2, sa3;
    float zc, ze0, ze1, ze2, ze3;
    int first;
    int ip, iq;  // p and q as integers when they are (then r^-p by multiplication), else -1
};

// r^-k for a small non-negative integer k
__device__ __forceinline__ float inv_ipow(float r, int k) {
    const float ir = 1.0f / r;
    float res = 1.0f, b = ir;
    while (k > 0) {
        if (k & 1) res *= b;
        b *= b;
        k >>= 1;
    }
    return res;
}

__device__ __forceinline__ void sw_two_body(const SWDev& p, float r, float& fr, float& half_e) {
    if (p.usezbl && r < p.sx0) {
        // sw.cpp:118-146
        const float rinv = 1.0f / r;
        const float f0 = 0.1818f * expf(-p.ze0 * r), f1 = 0.5099f * expf(-p.ze1 * r);
        const float f2 = 0.2802f * expf(-p.ze2 * r), f3 = 0.02817f * expf(-p.ze3 * r);
        const float fpot = (f0 + f1 + f2 + f3) * p.zc * rinv;
        fr = ((rinv + p.ze0) * f0 + (rinv + p.ze1) * f1 + (rinv + p.ze2) * f2 + (rinv + p.ze3) * f3) * p.zc *
             (rinv * rinv);
        half_e = 0.5f * fpot;
    } else if (p.usezbl && r < p.sx1) {
        // sw.cpp:148-164 (force factor applied with the opposite sign)
        const float f = p.sa1 + p.sa2 * r + p.sa3 * r * r;
        fr = -f;
        half_e = 0.5f * (p.sa0 + f * r);
    } else {
        // sw.cpp:166-189
        const float ira = 1.0f / (r - p.rc);
        const float rp = p.ip >= 0 ? inv_ipow(r, p.ip) : powf(r, -p.p);
        const float rq = p.iq >= 0 ? inv_ipow(r, p.iq) : powf(r, -p.q);
        const float fex = expf(p.sigma * ira);
        fr = (p.c1 * rp - p.c2 * rq + (p.c3 * rp - p.c4 * rq) * ira * ira * r) * fex / (r * r);
        half_e = 0.5f * (p.c5 * rp - p.c6 * rq) * fex;
    }
}

// A centre with more in-cutoff neighbours than the register path holds:
// up to TB_MAXN of them over local arrays (the two-body terms as well).
__device__ __noinline__ void sw_centre_wide(const SWDev& p, int i, const PosPack* __restrict__ pack,
                                            const unsigned* __restrict__ nbr, const int* __restrict__ nnb,
                                            float4* __restrict__ slot, float* __restrict__ fx, float* __restrict__ fy,
                                            float* __restrict__ fz, float* __restrict__ pe, unsigned* status) {
    const PosPack pi = pack[i];
    const int ti = pack_type(pi.hi);
    const bool mine = p.single_type || ti == p.ta;
    const int m = nnb[i];
    // neighbours inside the cutoff, vectors from i to the neighbour
    float vx[TB_MAXN], vy[TB_MAXN], vz[TB_MAXN], rr[TB_MAXN];
    int sl[TB_MAXN];
    int nc = 0;
    float ax = 0.f, ay = 0.f, az = 0.f, ae = 0.f;
    for (int s = 0; s < m; s++) {
        const size_t at = nbr_at(i, s, p.hshift, p.maxnb);
        slot[at] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (!mine) continue;
        const unsigned e = nbr[at];
        const int j = nbr_index(e);
        const PosPack pj = pack[j];
        if (!p.single_type && pack_type(pj.hi) != p.ta) continue;
        const float3 d = pair_delta(pi.hi, pi.lo, pj.hi, pj.lo, e, p.L);  // x_i - x_j
        const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
        if (!(r2 < p.rc2)) continue;
        const float r = sqrtf(r2);
        // r2 just below rc^2 can round to r == rc, where 1/(r - rc) is infinite
        // and 0 * inf gives NaN; every SW term is zero there, so drop the pair
        if (!(r < p.rc)) continue;
        float fr, he;
        sw_two_body(p, r, fr, he);
        ax += d.x * fr;
        ay += d.y * fr;
        az += d.z * fr;
        ae += he;
        if (nc < TB_MAXN) {
            vx[nc] = -d.x;
            vy[nc] = -d.y;
            vz[nc] = -d.z;
            rr[nc] = r;
            sl[nc] = s;
        } else {
            atomicOr(status, ERR_NBR_OVERFLOW);
        }
        nc++;
    }
    if (nc > TB_MAXN) nc = TB_MAXN;
    // triplets centred on i (sw.cpp:191-236), each unordered pair (j, k) once;
    // every neighbour's share is summed here and stored in its slot once.  The
    // per-neighbour factors exp(c7 / (r - rc)), 1 / r and c7 / ((r - rc)^2 r)
    // are computed once per neighbour instead of once per triplet.
    float sjx[TB_MAXN], sjy[TB_MAXN], sjz[TB_MAXN], sje[TB_MAXN];
    float ex[TB_MAXN], ir[TB_MAXN], gr[TB_MAXN];
    for (int a = 0; a < nc; a++) {
        sjx[a] = sjy[a] = sjz[a] = sje[a] = 0.f;
        const float ira = 1.0f / (rr[a] - p.rc), fira = p.c7 * ira;
        ex[a] = expf(fira);
        ir[a] = 1.0f / rr[a];
        gr[a] = fira * ira * ir[a];
    }
    for (int a = 0; a < nc; a++) {
        const float dx1 = vx[a], dy1 = vy[a], dz1 = vz[a];
        const float ex0 = ex[a], ir1 = ir[a], g0 = gr[a];
        float gjx = 0.f, gjy = 0.f, gjz = 0.f, gje = 0.f;
        for (int b = a + 1; b < nc; b++) {
            const float dx2 = vx[b], dy2 = vy[b], dz2 = vz[b];
            const float ir2 = ir[b];
            const float ir1r2 = ir1 * ir2;
            const float fex = ex0 * ex[b];
            const float cs = (dx1 * dx2 + dy1 * dy2 + dz1 * dz2) * ir1r2;
            const float dcos = cs - p.c10;
            const float ftheta = p.c9 * fex * dcos;
            const float ft12 = ir1r2 * ftheta;
            const float fpot = p.c8 * fex * dcos * dcos;
            const float fcos = cs * ftheta;
            const float fr0 = fpot * g0, fr1 = fpot * gr[b];
            const float ft0 = fcos * ir1 * ir1, ft1 = fcos * ir2 * ir2;
            const float fx0 = dx1 * (fr0 + ft0) - dx2 * ft12, fx1 = dx2 * (fr1 + ft1) - dx1 * ft12;
            const float fy0 = dy1 * (fr0 + ft0) - dy2 * ft12, fy1 = dy2 * (fr1 + ft1) - dy1 * ft12;
            const float fz0 = dz1 * (fr0 + ft0) - dz2 * ft12, fz1 = dz2 * (fr1 + ft1) - dz1 * ft12;
            ax -= fx0 + fx1;
            ay -= fy0 + fy1;
            az -= fz0 + fz1;
            const float third = fpot * (1.0f / 3.0f);
            ae += third;
            gjx += fx0;
            gjy += fy0;
            gjz += fz0;
            gje += third;
            sjx[b] += fx1;
            sjy[b] += fy1;
            sjz[b] += fz1;
            sje[b] += third;
        }
        sjx[a] += gjx;
        sjy[a] += gjy;
        sjz[a] += gjz;
        sje[a] += gje;
    }
    for (int a = 0; a < nc; a++)
        slot[nbr_at(i, sl[a], p.hshift, p.maxnb)] = make_float4(sjx[a], sjy[a], sjz[a], sje[a]);
    if (p.first) {
        fx[i] = ax;
        fy[i] = ay;
        fz[i] = az;
        pe[i] = ae;
    } else {
        fx[i] += ax;
        fy[i] += ay;
        fz[i] += az;
        pe[i] += ae;
    }
}

constexpr int SW_REG = 8;  // in-cutoff neighbours the register path holds (diamond: 4 + thermal second shell)
// k_sw_a at six 128-thread blocks a SM (80 registers, 252 bytes spilled) ran
// the Si 512k step faster than at its natural 121 registers (427 vs 458 us)

__device__ __forceinline__ void sw_store(const SWDev& p, int i, float ax, float ay, float az, float ae,
                                         float* __restrict__ fx, float* __restrict__ fy, float* __restrict__ fz,
                                         float* __restrict__ pe) {
    if (p.first) {
        fx[i] = ax;
        fy[i] = ay;
        fz[i] = az;
        pe[i] = ae;
    } else {
        fx[i] += ax;
        fy[i] += ay;
        fz[i] += az;
        pe[i] += ae;
    }
}

// Pass A of SW for centre i with up to SW_REG in-cutoff neighbours in
// registers (fully unrolled loops, insertion by select); centres with more
// are queued for k_sw_wide.  Same terms and summation order as the wide
// path.
__global__ void __launch_bounds__(128, 6) k_sw_a(SWDev p, const PosPack* __restrict__ pack,
                                              const unsigned* __restrict__ nbr, const int* __restrict__ nnb,
                                              float4* __restrict__ slot, float* __restrict__ fx,
                                              float* __restrict__ fy, float* __restrict__ fz, float* __restrict__ pe,
                                              unsigned* status, int* __restrict__ wide) {
    constexpr int K = SW_REG;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const PosPack pi = pack[i];
    const int ti = pack_type(pi.hi);
    const bool mine = p.single_type || ti == p.ta;
    const int m = nnb[i];
    float vx[K], vy[K], vz[K], rr[K];
    int sl[K];
#pragma unroll
    for (int k = 0; k < K; k++) vx[k] = vy[k] = vz[k] = 0.f, rr[k] = 1.f, sl[k] = 0;
    int nc = 0;
    float ax = 0.f, ay = 0.f, az = 0.f, ae = 0.f;
    for (int s = 0; s < m; s++) {
        const size_t at = nbr_at(i, s, p.hshift, p.maxnb);
        slot[at] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (!mine) continue;
        const unsigned e = nbr[at];
        const PosPack pj = pack[nbr_index(e)];
        if (!p.single_type && pack_type(pj.hi) != p.ta) continue;
        const float3 d = pair_delta(pi.hi, pi.lo, pj.hi, pj.lo, e, p.L);  // x_i - x_j
        const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
        if (!(r2 < p.rc2)) continue;
        const float r = sqrtf(r2);
        if (!(r < p.rc)) continue;  // r == rc: every SW term is zero (and 1/(r - rc) infinite)
        float fr, he;
        sw_two_body(p, r, fr, he);
        ax += d.x * fr;
        ay += d.y * fr;
        az += d.z * fr;
        ae += he;
#pragma unroll
        for (int k = 0; k < K; k++)
            if (k == nc) vx[k] = -d.x, vy[k] = -d.y, vz[k] = -d.z, rr[k] = r, sl[k] = s;
        nc++;
    }
    if (nc > K) {  // queued: k_sw_wide evaluates the whole centre
        wide[1 + atomicAdd(wide, 1)] = i;
        return;
    }
    // triplets centred on i (sw.cpp:191-236), each unordered pair (j, k) once
    float sjx[K], sjy[K], sjz[K], sje[K], ex[K], ir[K], gr[K];
    for_nbrs<K, true>(nc, [&](int a) {
        sjx[a] = sjy[a] = sjz[a] = sje[a] = 0.f;
        const float ira = 1.0f / (rr[a] - p.rc), fira = p.c7 * ira;
        ex[a] = expf(fira);
        ir[a] = 1.0f / rr[a];
        gr[a] = fira * ira * ir[a];
    });
    for_nbrs<K, true>(nc, [&](int a) {
        const float dx1 = vx[a], dy1 = vy[a], dz1 = vz[a];
        const float ex0 = ex[a], ir1 = ir[a], g0 = gr[a];
        float gjx = 0.f, gjy = 0.f, gjz = 0.f, gje = 0.f;
        for_nbrs<K, true>(nc, [&](int b) {
            if (b <= a) return;
            const float dx2 = vx[b], dy2 = vy[b], dz2 = vz[b];
            const float ir2 = ir[b];
            const float ir1r2 = ir1 * ir2;
            const float fex = ex0 * ex[b];
            const float cs = (dx1 * dx2 + dy1 * dy2 + dz1 * dz2) * ir1r2;
            const float dcos = cs - p.c10;
            const float ftheta = p.c9 * fex * dcos;
            const float ft12 = ir1r2 * ftheta;
            const float fpot = p.c8 * fex * dcos * dcos;
            const float fcos = cs * ftheta;
            const float fr0 = fpot * g0, fr1 = fpot * gr[b];
            const float ft0 = fcos * ir1 * ir1, ft1 = fcos * ir2 * ir2;
            const float fx0 = dx1 * (fr0 + ft0) - dx2 * ft12, fx1 = dx2 * (fr1 + ft1) - dx1 * ft12;
            const float fy0 = dy1 * (fr0 + ft0) - dy2 * ft12, fy1 = dy2 * (fr1 + ft1) - dy1 * ft12;
            const float fz0 = dz1 * (fr0 + ft0) - dz2 * ft12, fz1 = dz2 * (fr1 + ft1) - dz1 * ft12;
            ax -= fx0 + fx1;
            ay -= fy0 + fy1;
            az -= fz0 + fz1;
            const float third = fpot * (1.0f / 3.0f);
            ae += third;
            gjx += fx0;
            gjy += fy0;
            gjz += fz0;
            gje += third;
            sjx[b] += fx1;
            sjy[b] += fy1;
            sjz[b] += fz1;
            sje[b] += third;
        });
        sjx[a] += gjx;
        sjy[a] += gjy;
        sjz[a] += gjz;
        sje[a] += gje;
    });
    for_nbrs<K, true>(nc, [&](int a) {
        slot[nbr_at(i, sl[a], p.hshift, p.maxnb)] = make_float4(sjx[a], sjy[a], sjz[a], sje[a]);
    });
    sw_store(p, i, ax, ay, az, ae, fx, fy, fz, pe);
}

// The queued centres (wide[0] of them, indices from wide[1]).
__global__ void __launch_bounds__(128) k_sw_wide(SWDev p, const PosPack* __restrict__ pack,
                                                 const unsigned* __restrict__ nbr, const int* __restrict__ nnb,
                                                 const int* __restrict__ wide, float4* __restrict__ slot,
                                                 float* __restrict__ fx, float* __restrict__ fy,
                                                 float* __restrict__ fz, float* __restrict__ pe, unsigned* status) {
    const int cnt = wide[0];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x)
        sw_centre_wide(p, wide[1 + k], pack, nbr, nnb, slot, fx, fy, fz, pe, status);
}

// Gathers what every neighbour's pass A left for i; clears no state.
__global__ void __launch_bounds__(128) k_slot_gather(int n, int hshift, int maxnb, const unsigned* __restrict__ nbr,
                                                     const int* __restrict__ nnb, const int* __restrict__ rev,
                                                     const float4* __restrict__ slot, float* __restrict__ fx,
                                                     float* __restrict__ fy, float* __restrict__ fz,
                                                     float* __restrict__ pe, float* __restrict__ vir,
                                                     int zero_virial) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Kahan gx, gy, gz, ge;
    gx.add(fx[i]);
    gy.add(fy[i]);
    gz.add(fz[i]);
    ge.add(pe[i]);
    const int m = nnb[i];
    for (int s = 0; s < m; s++) {
        const size_t at = nbr_at(i, s, hshift, maxnb);
        const int j = nbr_index(nbr[at]);
        const float4 c = slot[nbr_at(j, rev[at], hshift, maxnb)];
        gx.add(c.x);
        gy.add(c.y);
        gz.add(c.z);
        ge.add(c.w);
    }
    fx[i] = gx.value();
    fy[i] = gy.value();
    fz[i] = gz.value();
    pe[i] = ge.value();
    if (zero_virial) vir[i] = 0.f;  // the reference SW does not accumulate a virial (sw.cpp:238)
}

// ------------------------------------------------------------------ Tersoff
struct TersDev {
    int n, hshift, maxnb, single_type, ta;
    ShiftF L;
    const ShiftF* rep_L;  // replica mode: periodic lengths of each replica (else null)
    const int* rep_of;
    float A, B, l1, l2, l3c, beta, nn, c2, d2, h, R, D, rc, rc2;
    int first;
};

// b = (1 + (beta zeta)^n)^(-1/2n) and db/dzeta.  In a close collision the
// exp(lambda3^3 (r_ij - r_ik)^3) factor makes zeta large enough for
// (beta zeta)^n to overflow FP32; there b is its limit (beta zeta)^(-1/2)
// (relative difference (beta zeta)^(-n) / 2n < 1e-26 for n ln(beta zeta) > 60).
__device__ __forceinline__ void ters_bond_order(const TersDev& p, float zeta, float& b, float& db) {
    if (!(zeta > 0.f)) {
        b = 1.f;
        db = 0.f;
        return;
    }
    // hardware logarithm and exponential: n ln(beta zeta) is off by ~1e-5
    // absolute, which moves b by ~2e-7 relative (the 1/2n power damps it)
    const float x = p.beta * zeta;
    const float nlx = p.nn * __logf(x);
    if (nlx > 60.f) {
        b = rsqrtf(x);
        db = -0.5f * b / zeta;
        return;
    }
    const float bn = __expf(nlx);
    b = exp2f((-0.5f / p.nn) * __log2f(1.f + bn));  // (1 + bn)^(-1/2n), |exponent| < 2: ~3e-7 relative
    db = __fdividef(-0.5f * b * bn, (1.f + bn) * zeta);
}

__device__ __forceinline__ float ters_fc(const TersDev& p, float r, float& dfc) {
    if (r < p.R - p.D) {
        dfc = 0.f;
        return 1.f;
    }
    if (r < p.R + p.D) {
        float sn, cs;
        sincospif(0.5f * (r - p.R) / p.D, &sn, &cs);  // sin, cos of pi (r-R) / (2D)
        dfc = -0.78539816339744831f / p.D * cs;  // -pi/(4D) cos
        return 0.5f - 0.5f * sn;
    }
    dfc = 0.f;
    return 0.f;
}

// The bonds centred on one atom, for its nc <= K in-cutoff neighbours
// (unit vectors u from the centre, distances r).  Per neighbour the cutoff
// f_c(r), f_c'(r) and 1/r are evaluated once; per triplet (a, b) the angular
// and radial factors once, in the zeta sweep, with what the x_k gradient
// needs kept for its sweep.
template <int K, bool UNR>
__device__ __forceinline__ void ters_bonds(const TersDev& p, const int nc, const float (&ux)[K],
                                           const float (&uy)[K], const float (&uz)[K], const float (&rr)[K],
                                           float (&skx)[K], float (&sky)[K], float (&skz)[K], float& fix,
                                           float& fiy, float& fiz, float& ei, float& wi) {
    float fc[K], dfc[K], ir[K];
    for_nbrs<K, UNR>(nc, [&](int b) {
        fc[b] = ters_fc(p, rr[b], dfc[b]);
        ir[b] = 1.0f / rr[b];
        skx[b] = sky[b] = skz[b] = 0.f;
    });
    const float g0 = 1.f + p.c2 / p.d2;
    for_nbrs<K, UNR>(nc, [&](int a) {
        const float rij = rr[a];
        const float ex_ = ux[a], ey_ = uy[a], ez_ = uz[a];
        // zeta_ij and its gradient w.r.t. x_j; per k the x_k coefficients
        float zeta = 0.f, gjx = 0.f, gjy = 0.f, gjz = 0.f;
        float ck[K], cc[K], cs[K];
        for_nbrs<K, UNR>(nc, [&](int b) {
            if (b == a) return;
            const float c = ex_ * ux[b] + ey_ * uy[b] + ez_ * uz[b];
            const float hc = p.h - c;
            const float rden = __fdividef(1.f, p.d2 + hc * hc);
            const float g = g0 - p.c2 * rden;
            const float dg = -2.f * p.c2 * hc * rden * rden;
            const float dr = rij - rr[b];
            const float ex = __expf(p.l3c * dr * dr * dr);
            const float dex = 3.f * p.l3c * dr * dr * ex;
            zeta += fc[b] * g * ex;
            const float cj = fc[b] * dg * ex * ir[a], cu = fc[b] * g * dex;
            gjx += cj * (ux[b] - c * ex_) + cu * ex_;
            gjy += cj * (uy[b] - c * ey_) + cu * ey_;
            gjz += cj * (uz[b] - c * ez_) + cu * ez_;
            ck[b] = dfc[b] * g * ex - fc[b] * g * dex;
            cc[b] = fc[b] * dg * ex * ir[b];
            cs[b] = c;
        });
        const float fR = p.A * __expf(-p.l1 * rij), fA = p.B * __expf(-p.l2 * rij);
        float bij, dbdz;
        ters_bond_order(p, zeta, bij, dbdz);
        const float vij = fc[a] * (fR - bij * fA);
        const float dv_dr = dfc[a] * (fR - bij * fA) + fc[a] * (-p.l1 * fR + bij * p.l2 * fA);
        const float dv_dz = -fc[a] * fA * dbdz;
        // gradient of 1/2 V_ij: x_j part
        const float sjx = 0.5f * (dv_dr * ex_ + dv_dz * gjx);
        const float sjy = 0.5f * (dv_dr * ey_ + dv_dz * gjy);
        const float sjz = 0.5f * (dv_dr * ez_ + dv_dz * gjz);
        fix += sjx;  // the x_i gradient is minus the sum of the others
        fiy += sjy;
        fiz += sjz;
        const float s = 0.5f * dv_dz;
        // x_k parts
        for_nbrs<K, UNR>(nc, [&](int b) {
            if (b == a) return;
            const float kx = s * (ck[b] * ux[b] + cc[b] * (ex_ - cs[b] * ux[b]));
            const float ky = s * (ck[b] * uy[b] + cc[b] * (ey_ - cs[b] * uy[b]));
            const float kz = s * (ck[b] * uz[b] + cc[b] * (ez_ - cs[b] * uz[b]));
            fix += kx;
            fiy += ky;
            fiz += kz;
            // force on k = -gradient
            skx[b] -= kx;
            sky[b] -= ky;
            skz[b] -= kz;
        });
        skx[a] -= sjx;
        sky[a] -= sjy;
        skz[a] -= sjz;
        ei += 0.5f * vij;
        wi += 0.5f * dv_dr * rij;
    });
}

// Relative vector from centre i to its list entry at `at`, when the pair is
// one this potential evaluates and lies within the cutoff.
__device__ __forceinline__ bool ters_neighbor(const TersDev& p, const PosPack& pi, const ShiftF& L,
                                              const PosPack* __restrict__ pack, unsigned e, float3& u, float& r) {
    const PosPack pj = pack[nbr_index(e)];
    if (!p.single_type && pack_type(pj.hi) != p.ta) return false;
    const float3 d = pair_delta(pi.hi, pi.lo, pj.hi, pj.lo, e, L);
    const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
    if (!(r2 < p.rc2)) return false;
    r = sqrtf(r2);
    if (!(r < p.rc)) return false;
    const float ri = 1.0f / r;
    u = make_float3(-d.x * ri, -d.y * ri, -d.z * ri);  // unit vector from i to the neighbour
    return true;
}

__device__ __forceinline__ void ters_store(const TersDev& p, int i, float fix, float fiy, float fiz, float ei,
                                           float wi, float* __restrict__ fx, float* __restrict__ fy,
                                           float* __restrict__ fz, float* __restrict__ pe, float* __restrict__ vir) {
    if (p.first) {
        fx[i] = fix;
        fy[i] = fiy;
        fz[i] = fiz;
        pe[i] = ei;
        vir[i] = wi;
    } else {
        fx[i] += fix;
        fy[i] += fiy;
        fz[i] += fiz;
        pe[i] += ei;
        vir[i] += wi;
    }
}

// A centre with more in-cutoff neighbours than the register path holds (a
// collision cascade): up to TB_MAXN of them over local arrays.
__device__ __noinline__ void ters_centre_wide(const TersDev& p, int i, const PosPack pi, const ShiftF L,
                                              const PosPack* __restrict__ pack, const unsigned* __restrict__ nbr,
                                              int m, float4* __restrict__ slot, float* __restrict__ fx,
                                              float* __restrict__ fy, float* __restrict__ fz, float* __restrict__ pe,
                                              float* __restrict__ vir, unsigned* status) {
    float ux[TB_MAXN], uy[TB_MAXN], uz[TB_MAXN], rr[TB_MAXN];
    int sl[TB_MAXN];
    int nc = 0;
    for (int s = 0; s < m; s++) {
        const size_t at = nbr_at(i, s, p.hshift, p.maxnb);
        float3 u;
        float r;
        if (!ters_neighbor(p, pi, L, pack, nbr[at], u, r)) continue;
        if (nc < TB_MAXN) {
            ux[nc] = u.x;
            uy[nc] = u.y;
            uz[nc] = u.z;
            rr[nc] = r;
            sl[nc] = s;
        } else {
            atomicOr(status, ERR_NBR_OVERFLOW);
        }
        nc++;
    }
    if (nc > TB_MAXN) nc = TB_MAXN;
    float fix = 0.f, fiy = 0.f, fiz = 0.f, ei = 0.f, wi = 0.f;
    float skx[TB_MAXN], sky[TB_MAXN], skz[TB_MAXN];
    ters_bonds<TB_MAXN, false>(p, nc, ux, uy, uz, rr, skx, sky, skz, fix, fiy, fiz, ei, wi);
    for (int a = 0; a < nc; a++)
        slot[nbr_at(i, sl[a], p.hshift, p.maxnb)] = make_float4(skx[a], sky[a], skz[a], 0.f);
    ters_store(p, i, fix, fiy, fiz, ei, wi, fx, fy, fz, pe, vir);
}

constexpr int TERS_REG = 4;  // in-cutoff neighbours the register path holds (diamond: 4)

__device__ __forceinline__ void ters_reg_centre(const TersDev& p, int i, const PosPack* __restrict__ pack,
                                                const unsigned* __restrict__ nbr, const int* __restrict__ nnb,
                                                float4* __restrict__ slot, float* __restrict__ fx,
                                                float* __restrict__ fy, float* __restrict__ fz,
                                                float* __restrict__ pe, float* __restrict__ vir,
                                                const int* __restrict__ mask, int* __restrict__ wide);

// One thread per centre.  Launched with fewer threads than centres (the
// persistent form: one resident grid over the flattened atoms of every
// replica), each thread strides over the centres.
constexpr int TERS_CTAS_PER_SM = 8;  // 64 registers: the Si 512k register pass 54.8 -> 51.6 us against 6 (80)

template <bool PERSISTENT>
__global__ void __launch_bounds__(128, TERS_CTAS_PER_SM) k_tersoff_a(TersDev p, const PosPack* __restrict__ pack,
                                                   const unsigned* __restrict__ nbr, const int* __restrict__ nnb,
                                                   float4* __restrict__ slot, float* __restrict__ fx,
                                                   float* __restrict__ fy, float* __restrict__ fz,
                                                   float* __restrict__ pe, float* __restrict__ vir, unsigned* status,
                                                   const int* __restrict__ mask, int* __restrict__ wide,
                                                   const int* __restrict__ nmask) {
    if (nmask && *nmask == 0) return;  // a mask with no centre in it
    if (PERSISTENT) {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += gridDim.x * blockDim.x)
            ters_reg_centre(p, i, pack, nbr, nnb, slot, fx, fy, fz, pe, vir, mask, wide);
    } else {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        if (i < p.n) ters_reg_centre(p, i, pack, nbr, nnb, slot, fx, fy, fz, pe, vir, mask, wide);
    }
}

__device__ __forceinline__ void ters_reg_centre(const TersDev& p, int i, const PosPack* __restrict__ pack,
                                                const unsigned* __restrict__ nbr, const int* __restrict__ nnb,
                                                float4* __restrict__ slot, float* __restrict__ fx,
                                                float* __restrict__ fy, float* __restrict__ fz,
                                                float* __restrict__ pe, float* __restrict__ vir,
                                                const int* __restrict__ mask, int* __restrict__ wide) {
    if (mask && !mask[i]) return;  // centres another potential evaluates
    const PosPack pi = pack[i];
    const bool mine = p.single_type || pack_type(pi.hi) == p.ta;
    const ShiftF L = p.rep_L ? p.rep_L[p.rep_of[i]] : p.L;
    const int m = nnb[i];
    // the in-cutoff neighbours go to registers by select; every other slot
    // of the row gets its zero here
    float ux[TERS_REG], uy[TERS_REG], uz[TERS_REG], rr[TERS_REG];
    int sl[TERS_REG];
#pragma unroll
    for (int k = 0; k < TERS_REG; k++) ux[k] = uy[k] = uz[k] = rr[k] = 0.f, sl[k] = 0;
    int nc = 0;
    for (int s = 0; s < m; s++) {
        const size_t at = nbr_at(i, s, p.hshift, p.maxnb);
        float3 u;
        float r;
        if (mine && ters_neighbor(p, pi, L, pack, nbr[at], u, r)) {
#pragma unroll
            for (int k = 0; k < TERS_REG; k++)
                if (k == nc) ux[k] = u.x, uy[k] = u.y, uz[k] = u.z, rr[k] = r, sl[k] = s;
            nc++;
        } else {
            slot[at] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
    if (nc > TERS_REG) {  // queued for k_tersoff_wide, so its warp does not wait on it
        wide[1 + atomicAdd(wide, 1)] = i;
        return;
    }
    float fix = 0.f, fiy = 0.f, fiz = 0.f, ei = 0.f, wi = 0.f;
    float skx[TERS_REG], sky[TERS_REG], skz[TERS_REG];
    ters_bonds<TERS_REG, true>(p, nc, ux, uy, uz, rr, skx, sky, skz, fix, fiy, fiz, ei, wi);
#pragma unroll
    for (int a = 0; a < TERS_REG; a++)
        if (a < nc) slot[nbr_at(i, sl[a], p.hshift, p.maxnb)] = make_float4(skx[a], sky[a], skz[a], 0.f);
    ters_store(p, i, fix, fiy, fiz, ei, wi, fx, fy, fz, pe, vir);
}

// The queued centres (wide[0] of them, indices from wide[1]): a grid-stride
// loop, so the few centres of a collision cascade run in dense warps.
__global__ void __launch_bounds__(128) k_tersoff_wide(TersDev p, const PosPack* __restrict__ pack,
                                                      const unsigned* __restrict__ nbr, const int* __restrict__ nnb,
                                                      const int* __restrict__ wide, float4* __restrict__ slot,
                                                      float* __restrict__ fx, float* __restrict__ fy,
                                                      float* __restrict__ fz, float* __restrict__ pe,
                                                      float* __restrict__ vir, unsigned* status) {
    const int cnt = wide[0];
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x) {
        const int i = wide[1 + k];
        const PosPack pi = pack[i];
        const ShiftF L = p.rep_L ? p.rep_L[p.rep_of[i]] : p.L;
        ters_centre_wide(p, i, pi, L, pack, nbr, nnb[i], slot, fx, fy, fz, pe, vir, status);
    }
}

// ------------------------------------------------------------------ ZBL pair
struct ZBLDev {
    int n, hshift, maxnb, ta, tb;
    ShiftF L;
    const ShiftF* rep_L;  // replica mode (else null)
    const int* rep_of;
    float rc, rsw, zc, ze0, ze1, ze2, ze3;
    int first;
};

// Universal ZBL screened Coulomb (sw.cpp:118-146 form), multiplied by a
// smooth switch S(r) that goes from 1 at rsw to 0 at rc.
__global__ void __launch_bounds__(128) k_zbl(ZBLDev p, const PosPack* __restrict__ pack,
                                             const unsigned* __restrict__ nbr, const int* __restrict__ nnb,
                                             float* __restrict__ fx, float* __restrict__ fy, float* __restrict__ fz,
                                             float* __restrict__ pe, float* __restrict__ vir) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const PosPack pi = pack[i];
    const int ti = pack_type(pi.hi);
    const ShiftF L = p.rep_L ? p.rep_L[p.rep_of[i]] : p.L;
    float ax = 0.f, ay = 0.f, az = 0.f, ae = 0.f, av = 0.f;
    if (ti == p.ta || ti == p.tb) {
        const int m = nnb[i];
        for (int s = 0; s < m; s++) {
            const unsigned e = nbr[nbr_at(i, s, p.hshift, p.maxnb)];
            const PosPack pj = pack[nbr_index(e)];
            const int tj = pack_type(pj.hi);
            if (!((ti == p.ta && tj == p.tb) || (ti == p.tb && tj == p.ta))) continue;
            const float3 d = pair_delta(pi.hi, pi.lo, pj.hi, pj.lo, e, L);
            const float r2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
            const float r = sqrtf(r2);
            if (!(r < p.rc)) continue;
            const float rinv = 1.f / r;
            const float f0 = 0.1818f * expf(-p.ze0 * r), f1 = 0.5099f * expf(-p.ze1 * r);
            const float f2 = 0.2802f * expf(-p.ze2 * r), f3 = 0.02817f * expf(-p.ze3 * r);
            const float phi = (f0 + f1 + f2 + f3) * p.zc * rinv;
            const float dphi = -((rinv + p.ze0) * f0 + (rinv + p.ze1) * f1 + (rinv + p.ze2) * f2 +
                                 (rinv + p.ze3) * f3) * p.zc * rinv;
            float S = 1.f, dS = 0.f;
            if (r > p.rsw) {
                const float t = (r - p.rsw) / (p.rc - p.rsw);
                S = 1.f - t * t * t * (10.f - 15.f * t + 6.f * t * t);
                dS = -30.f * t * t * (1.f - t) * (1.f - t) / (p.rc - p.rsw);
            }
            const float v = phi * S;
            const float dv = dphi * S + phi * dS;
            const float fr = -dv * rinv;
            ax += d.x * fr;
            ay += d.y * fr;
            az += d.z * fr;
            ae += 0.5f * v;
            av += fr * r2;
        }
    }
    if (p.first) {
        fx[i] = ax;
        fy[i] = ay;
        fz[i] = az;
        pe[i] = ae;
        vir[i] = av;
    } else {
        fx[i] += ax;
        fy[i] += ay;
        fz[i] += az;
        pe[i] += ae;
        vir[i] += av;
    }
}

// ------------------------------------------------------------------ host
int threebody_prepare(Context* c) { return OMDG_OK; }

int gather_slots(Context* c, bool zero_virial) {
    prof_begin(c, "slot_gather");
    k_slot_gather<<<grid_for(c->n, 128), 128, 0, c->stream>>>(
        c->n, c->nbr_hshift, c->maxnb, reinterpret_cast<const unsigned*>(c->nbr), c->nnb, c->rev, c->slot_buf, c->fx,
        c->fy, c->fz, c->pe, c->vir, zero_virial ? 1 : 0);
    prof_end(c);
    c->launches++;
    return check_cuda(c, cudaGetLastError(), "slot gather");
}

int sw_launch(Context* c, Potential& pot, bool first) {
    if (!c->rev || !c->slot_buf) return set_error(c, OMDG_ESTATE, "three-body buffers missing");
    const SWParams& s = pot.sw;
    SWDev p;
    p.n = c->n;
    p.hshift = c->nbr_hshift;
    p.maxnb = c->maxnb;
    p.single_type = c->ntypes == 1;
    p.ta = pot.ta;
    p.L = make_shift(c->box);
    p.rc = (float)s.rc;
    p.rc2 = (float)(s.rc * s.rc);
    p.A = (float)s.A;
    p.B = (float)s.B;
    p.p = (float)s.p;
    p.q = (float)s.q;
    p.ip = (s.p >= 0 && s.p <= 16 && s.p == std::floor(s.p)) ? (int)s.p : -1;
    p.iq = (s.q >= 0 && s.q <= 16 && s.q == std::floor(s.q)) ? (int)s.q : -1;
    p.sigma = (float)s.sigma;
    p.eps = (float)s.eps;
    p.c1 = (float)s.c1;
    p.c2 = (float)s.c2;
    p.c3 = (float)s.c3;
    p.c4 = (float)s.c4;
    p.c5 = (float)s.c5;
    p.c6 = (float)s.c6;
    p.c7 = (float)s.c7;
    p.c8 = (float)s.c8;
    p.c9 = (float)s.c9;
    p.c10 = (float)s.c10;
    p.usezbl = s.usezbl;
    p.sx0 = (float)s.sx0;
    p.sx1 = (float)s.sx1;
    p.sa0 = (float)s.sa0;
    p.sa1 = (float)s.sa1;
    p.sa2 = (float)s.sa2;
    p.sa3 = (float)s.sa3;
    p.zc = (float)s.zc;
    p.ze0 = (float)s.ze0;
    p.ze1 = (float)s.ze1;
    p.ze2 = (float)s.ze2;
    p.ze3 = (float)s.ze3;
    p.first = first ? 1 : 0;
    prof_begin(c, "sw_centre");
    cudaMemsetAsync(c->ters_wide, 0, sizeof(int), c->stream);
    k_sw_a<<<grid_for(c->n, 128), 128, 0, c->stream>>>(p, c->pack, reinterpret_cast<const unsigned*>(c->nbr), c->nnb,
                                                        c->slot_buf, c->fx, c->fy, c->fz, c->pe, c->d_status,
                                                        c->ters_wide);
    k_sw_wide<<<2 * c->num_sms, 128, 0, c->stream>>>(p, c->pack, reinterpret_cast<const unsigned*>(c->nbr), c->nnb,
                                                     c->ters_wide, c->slot_buf, c->fx, c->fy, c->fz, c->pe,
                                                     c->d_status);
    prof_end(c);
    c->launches += 2;
    int rc = check_cuda(c, cudaGetLastError(), "sw");
    if (rc) return rc;
    return gather_slots(c, first);
}

int tersoff_launch(Context* c, Potential& pot, bool first) {
    int rc = tersoff_centre(c, pot, first, nullptr);
    if (rc) return rc;
    return gather_slots(c, false);
}

// Pass A of Tersoff: bond gradients of every centre (or of the centres with
// mask[i] != 0) into the slot buffer; the caller gathers.
int tersoff_centre(Context* c, Potential& pot, bool first, const int* mask, const int* mask_count) {
    if (!c->rev || !c->slot_buf) return set_error(c, OMDG_ESTATE, "three-body buffers missing");
    const TersoffParams& t = pot.ters;
    TersDev p;
    p.n = c->n;
    p.hshift = c->nbr_hshift;
    p.maxnb = c->maxnb;
    p.single_type = c->ntypes == 1;
    p.ta = pot.ta;
    p.L = make_shift(c->box);
    p.rep_L = c->nrep > 0 ? static_cast<const ShiftF*>(c->d_rep_shift) : nullptr;
    p.rep_of = c->d_rep_of;
    p.A = (float)t.A;
    p.B = (float)t.B;
    p.l1 = (float)t.lambda1;
    p.l2 = (float)t.lambda2;
    p.l3c = (float)(t.lambda3 * t.lambda3 * t.lambda3);
    p.beta = (float)t.beta;
    p.nn = (float)t.n;
    p.c2 = (float)(t.c * t.c);
    p.d2 = (float)(t.d * t.d);
    p.h = (float)t.h;
    p.R = (float)t.R;
    p.D = (float)t.D;
    p.rc = (float)(t.R + t.D);
    p.rc2 = p.rc * p.rc * 1.0001f;
    p.first = first ? 1 : 0;
    prof_begin(c, mask ? "tersoff_fallback" : "tersoff_centre");
    cudaMemsetAsync(c->ters_wide, 0, sizeof(int), c->stream);
    // a masked pass (the surrogate's fallback, usually for no centre at all)
    // takes the strided form: one resident grid, each block gone after
    // reading the count
    if (c->tb_persistent || mask_count)
        k_tersoff_a<true><<<std::min(grid_for(c->n, 128), TERS_CTAS_PER_SM * c->num_sms), 128, 0, c->stream>>>(
            p, c->pack, reinterpret_cast<const unsigned*>(c->nbr), c->nnb, c->slot_buf, c->fx, c->fy, c->fz, c->pe,
            c->vir, c->d_status, mask, c->ters_wide, mask_count);
    else
        k_tersoff_a<false><<<grid_for(c->n, 128), 128, 0, c->stream>>>(
            p, c->pack, reinterpret_cast<const unsigned*>(c->nbr), c->nnb, c->slot_buf, c->fx, c->fy, c->fz, c->pe,
            c->vir, c->d_status, mask, c->ters_wide, mask_count);
    k_tersoff_wide<<<2 * c->num_sms, 128, 0, c->stream>>>(p, c->pack, reinterpret_cast<const unsigned*>(c->nbr),
                                                          c->nnb, c->ters_wide, c->slot_buf, c->fx, c->fy, c->fz,
                                                          c->pe, c->vir, c->d_status);
    prof_end(c);
    c->launches += 2;
    return check_cuda(c, cudaGetLastError(), "tersoff");
}

int zbl_launch(Context* c, Potential& pot, bool first) {
    const ZBLParams& z = pot.zbl;
    ZBLDev p;
    p.n = c->n;
    p.hshift = c->nbr_hshift;
    p.maxnb = c->maxnb;
    p.ta = pot.ta;
    p.tb = pot.tb;
    p.L = make_shift(c->box);
    p.rep_L = c->nrep > 0 ? static_cast<const ShiftF*>(c->d_rep_shift) : nullptr;
    p.rep_of = c->d_rep_of;
    p.rc = (float)z.rc;
    p.rsw = (float)(z.rc - z.width);
    p.zc = (float)z.zc;
    p.ze0 = (float)z.ze0;
    p.ze1 = (float)z.ze1;
    p.ze2 = (float)z.ze2;
    p.ze3 = (float)z.ze3;
    p.first = first ? 1 : 0;
    prof_begin(c, "zbl");
    k_zbl<<<grid_for(c->n, 128), 128, 0, c->stream>>>(p, c->pack, reinterpret_cast<const unsigned*>(c->nbr), c->nnb,
                                                       c->fx, c->fy, c->fz, c->pe, c->vir);
    prof_end(c);
    c->launches++;
    return check_cuda(c, cudaGetLastError(), "zbl");
}

}  // namespace omdg
