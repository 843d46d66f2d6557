// Training of the neural surrogate on the GPU (no reference counterpart).
//
// A dataset is a set of periodic configurations (positions, box lengths,
// reference total energies and forces).  Its descriptors G and their
// Jacobian J (dG_i/dx_j for every neighbour j inside the cutoff; dG_i/dx_i is
// minus their sum) are computed once.  One training step over a batch of
// configurations:
//   1. k_nn_fwd        E_i and u_i = dE_i/dG_i (FP32, per atom)
//   2. k_nn_conf_energy  per configuration: dE = (sum E_i - E_ref) / N
//   3. k_nn_force      F_k = sum_s (J_ks^T u_k - J_(j,rev)^T u_j), force residual
//   4. k_nn_vvec       v_i = dL/du_i = sum_s J_is (rho_i - rho_j)
//   5. k_nn_atom_grad  per-atom vectors of the energy and force gradients
//                      (the force term differentiates u_i . v_i through the
//                      network: forward-mode tangent, then reverse mode)
//   6. k_nn_wgrad_*    outer-product sums over atoms, fixed order (deterministic)
//   7. k_nn_adam       Adam update of the FP32 parameters
// Loss: L = wE mean_c (dE_c)^2 + wF mean_(k,a) (F_ka - F_ka^ref)^2.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "nn_desc.cuh"
#include "tc_common.cuh"

struct omdg_nn {
    int device = 0;
    int num_sms = 152;
    cudaStream_t stream = nullptr;
    std::string err;
    omdg::NNModel model;
    bool have_weights = false;
    // dataset (host bookkeeping)
    int nconf = 0;
    long natoms = 0, nslots = 0;
    std::vector<int> conf_start;  // nconf + 1
    // dataset (device)
    int* d_conf_start = nullptr;
    int* d_atom_conf = nullptr;
    double* d_x = nullptr;
    double* d_L = nullptr;
    float* d_eref = nullptr;
    float* d_fref = nullptr;
    float* d_fw = nullptr;      // per-configuration force-loss weight
    float* d_eatom = nullptr;   // per-atom reference energies (per-atom energy loss) or null
    float* d_ewa = nullptr;     // per atom dL/dE_i in the per-atom mode
    std::vector<float> fms;     // per-configuration mean square reference force
    int* d_slot_start = nullptr;
    int* d_slot_j = nullptr;
    int* d_slot_rev = nullptr;
    float4* d_slot_d = nullptr;
    float* d_G = nullptr;   // raw descriptors
    float* d_Gt = nullptr;  // normalised
    float* d_J = nullptr;   // nslots x 3 x 32
    // training state
    float* d_params = nullptr;
    float* d_adam_m = nullptr;
    float* d_adam_v = nullptr;
    float* d_grad = nullptr;
    float* d_E = nullptr;
    float* d_u = nullptr;
    float* d_F = nullptr;
    float* d_rho = nullptr;
    float* d_vvec = nullptr;
    float* d_ew = nullptr;       // per configuration dL/dE_i
    float* d_lossE = nullptr;    // per batch configuration
    float* d_lossF = nullptr;    // per batch atom
    float* d_vecs = nullptr;     // per batch atom: 7 x 64 vectors + e
    float* d_partial = nullptr;  // per chunk x NN_PARAMS
    double* d_loss = nullptr;
    int* d_list = nullptr;       // atom order of the epoch
    int* d_clist = nullptr;      // configuration order of the epoch
    unsigned* d_status = nullptr;
    long cap_batch_atoms = 0;
    long adam_t = 0;
    omdg::NNDevNet net;
};

namespace omdg {

constexpr int NN_VEC_STRIDE = 7 * NN_H + 1;  // zeta1 d1 zeta2 d2 a1 da1 w3g | e
constexpr int NN_CHUNK = 32;                  // atoms per gradient partial

// ------------------------------------------------------------------ dataset kernels
__device__ __forceinline__ double nn_min_image(double d, double L) { return d - L * rint(d / L); }

__global__ void k_nn_count(long n, const int* __restrict__ atom_conf, const int* __restrict__ conf_start,
                           const double* __restrict__ x, const double* __restrict__ L, double rc2,
                           int* __restrict__ count) {
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = atom_conf[i];
    const double lx = L[3 * c], ly = L[3 * c + 1], lz = L[3 * c + 2];
    int k = 0;
    for (int j = conf_start[c]; j < conf_start[c + 1]; j++) {
        if (j == i) continue;
        const double dx = nn_min_image(x[3 * j] - x[3 * i], lx);
        const double dy = nn_min_image(x[3 * j + 1] - x[3 * i + 1], ly);
        const double dz = nn_min_image(x[3 * j + 2] - x[3 * i + 2], lz);
        if (dx * dx + dy * dy + dz * dz < rc2) k++;
    }
    count[i] = k;
}

__global__ void k_nn_fill(long n, const int* __restrict__ atom_conf, const int* __restrict__ conf_start,
                          const double* __restrict__ x, const double* __restrict__ L, double rc2,
                          const int* __restrict__ slot_start, int* __restrict__ slot_j, float4* __restrict__ slot_d) {
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = atom_conf[i];
    const double lx = L[3 * c], ly = L[3 * c + 1], lz = L[3 * c + 2];
    int s = slot_start[i];
    for (int j = conf_start[c]; j < conf_start[c + 1]; j++) {
        if (j == i) continue;
        const double dx = nn_min_image(x[3 * j] - x[3 * i], lx);
        const double dy = nn_min_image(x[3 * j + 1] - x[3 * i + 1], ly);
        const double dz = nn_min_image(x[3 * j + 2] - x[3 * i + 2], lz);
        const double r2 = dx * dx + dy * dy + dz * dz;
        if (r2 < rc2) {
            slot_j[s] = j;
            slot_d[s] = make_float4((float)dx, (float)dy, (float)dz, (float)sqrt(r2));
            s++;
        }
    }
}

__global__ void k_nn_rev(long n, const int* __restrict__ slot_start, const int* __restrict__ slot_j,
                         int* __restrict__ rev, unsigned* status) {
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int s = slot_start[i]; s < slot_start[i + 1]; s++) {
        const int j = slot_j[s];
        int found = -1;
        for (int q = slot_start[j]; q < slot_start[j + 1]; q++)
            if (slot_j[q] == (int)i) found = q;
        if (found < 0) atomicOr(status, ERR_NBR_OVERFLOW);
        rev[s] = found < 0 ? s : found;
    }
}

// G and J of one atom from its neighbour slots (d = x_j - x_i, w = r).
__global__ void k_nn_train_desc(NNDescParams p, long n, const int* __restrict__ slot_start,
                                const float4* __restrict__ slot_d, float* __restrict__ G, float* __restrict__ J) {
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float g[NN_DESC];
#pragma unroll
    for (int k = 0; k < NN_DESC; k++) g[k] = 0.f;
    const int s0 = slot_start[i], s1 = slot_start[i + 1];
    for (int s = s0; s < s1; s++) {
        const float4 d = slot_d[s];
        const float r = d.w, ir = 1.f / r;
        const float e[3] = {d.x * ir, d.y * ir, d.z * ir};
        float dfc;
        const float fc = nn_fc(p, r, dfc);
        float* Js = J + (size_t)s * 3 * NN_DESC;
        for (int k = 0; k < NN_RAD; k++) {
            float v, ddr;
            nn_radial(p, r, fc, dfc, k, v, ddr);
            g[k] += v;
            for (int c = 0; c < 3; c++) Js[c * NN_DESC + k] = ddr * e[c];
        }
        for (int c = 0; c < 3; c++)
            for (int m = 0; m < NN_ANG; m++) Js[c * NN_DESC + NN_RAD + m] = 0.f;
    }
    for (int a = s0; a < s1; a++) {
        const float4 da = slot_d[a];
        const float ra = da.w, ia = 1.f / ra;
        const float ea[3] = {da.x * ia, da.y * ia, da.z * ia};
        float dfa;
        const float fa = nn_fc(p, ra, dfa);
        float* Ja = J + (size_t)a * 3 * NN_DESC + NN_RAD;
        for (int b = a + 1; b < s1; b++) {
            const float4 db = slot_d[b];
            const float rb = db.w, ib = 1.f / rb;
            const float eb[3] = {db.x * ib, db.y * ib, db.z * ib};
            float dfb;
            const float fb = nn_fc(p, rb, dfb);
            const float cs = ea[0] * eb[0] + ea[1] * eb[1] + ea[2] * eb[2];
            float dca[3], dcb[3];
            for (int c = 0; c < 3; c++) {
                dca[c] = (eb[c] - cs * ea[c]) * ia;
                dcb[c] = (ea[c] - cs * eb[c]) * ib;
            }
            float* Jb = J + (size_t)b * 3 * NN_DESC + NN_RAD;
            const float s2 = ra * ra + rb * rb;
            NNAngExp ex;
            for (int m = 0; m < NN_ANG; m++) {
                float v, d_ra, d_rb, d_cs;
                nn_angular(p, m, ra, rb, cs, fa, dfa, fb, dfb, ex.get(p.eta_a[m], s2), v, d_ra, d_rb, d_cs);
                g[NN_RAD + m] += v;
                for (int c = 0; c < 3; c++) {
                    Ja[c * NN_DESC + m] += d_ra * ea[c] + d_cs * dca[c];
                    Jb[c * NN_DESC + m] += d_rb * eb[c] + d_cs * dcb[c];
                }
            }
        }
    }
    for (int k = 0; k < NN_DESC; k++) G[i * NN_DESC + k] = g[k];
}

__global__ void k_nn_normalize(NNDescParams p, long n, const float* __restrict__ G, float* __restrict__ Gt) {
    const long q = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (q >= n * NN_DESC) return;
    const int d = (int)(q % NN_DESC);
    Gt[q] = (G[q] - p.mu[d]) * p.isig[d];
}

// ------------------------------------------------------------------ training kernels
// Parameters staged in shared memory (FP32).
__device__ __forceinline__ void load_params(const float* __restrict__ w, float* s) {
    for (int k = threadIdx.x; k < NN_PARAMS; k += blockDim.x) s[k] = w[k];
    __syncthreads();
}

// E_i and u_i (raw descriptor units) for the atoms list[a0 .. a0 + na).
__global__ void __launch_bounds__(128) k_nn_fwd(const float* __restrict__ w, const float* __restrict__ Gt,
                                                NNDescParams p, const int* __restrict__ list, int a0, int na,
                                                float* __restrict__ E, float* __restrict__ U) {
    extern __shared__ float sw[];
    load_params(w, sw);
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= na) return;
    const int atom = list[a0 + t];
    const float* W1 = sw + NN_OFF_W1;
    const float* W2 = sw + NN_OFF_W2;
    float g[NN_DESC];
    for (int d = 0; d < NN_DESC; d++) g[d] = Gt[(size_t)atom * NN_DESC + d];
    float a1[NN_H];
    for (int j = 0; j < NN_H; j++) {
        float z = sw[NN_OFF_B1 + j];
        for (int d = 0; d < NN_DESC; d++) z = fmaf(W1[j * NN_DESC + d], g[d], z);
        a1[j] = tanhf(z);
    }
    float d2[NN_H];
    float e = sw[NN_OFF_B3];
    for (int o = 0; o < NN_H; o++) {
        float z = sw[NN_OFF_B2 + o];
        for (int j = 0; j < NN_H; j++) z = fmaf(W2[o * NN_H + j], a1[j], z);
        const float a2 = tanhf(z);
        e = fmaf(sw[NN_OFF_W3 + o], a2, e);
        d2[o] = sw[NN_OFF_W3 + o] * (1.f - a2 * a2);
    }
    float u[NN_DESC];
    for (int d = 0; d < NN_DESC; d++) u[d] = 0.f;
    for (int j = 0; j < NN_H; j++) {
        float s = 0.f;
        for (int o = 0; o < NN_H; o++) s = fmaf(d2[o], W2[o * NN_H + j], s);
        const float d1 = s * (1.f - a1[j] * a1[j]);
        for (int d = 0; d < NN_DESC; d++) u[d] = fmaf(d1, W1[j * NN_DESC + d], u[d]);
    }
    E[atom] = e;
    for (int d = 0; d < NN_DESC; d++) U[(size_t)atom * NN_DESC + d] = u[d] * p.isig[d];
}

// One block per batch configuration: energy residual and its loss term.
__global__ void k_nn_conf_energy(const int* __restrict__ clist, int c0, int nb, const int* __restrict__ conf_start,
                                 const float* __restrict__ E, const float* __restrict__ eref, float wE,
                                 float* __restrict__ ew, float* __restrict__ lossE) {
    __shared__ double red[256];
    const int conf = clist[c0 + blockIdx.x];
    const int a = conf_start[conf], b = conf_start[conf + 1];
    double s = 0.0;
    for (int i = a + threadIdx.x; i < b; i += blockDim.x) s += (double)E[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const int n = b - a;
        const double de = (red[0] - (double)eref[conf]) / n;
        ew[conf] = (float)(2.0 * wE * de / ((double)n * nb));
        lossE[blockIdx.x] = (float)(wE * de * de / nb);
    }
}

// Per-atom energy residuals (per-atom energy loss): dL/dE_i and the loss terms.
__global__ void k_nn_atom_energy(const int* __restrict__ list, int a0, int na, const float* __restrict__ E,
                                 const float* __restrict__ eatom, float wE, float* __restrict__ ewa,
                                 float* __restrict__ lossE) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= na) return;
    const int i = list[a0 + t];
    const float r = E[i] - eatom[i];
    ewa[i] = 2.f * wE * r / na;
    lossE[t] = wE * r * r / na;
}

// Forces from J and u; the force residual, rho = dL/dF and its loss term.
__global__ void k_nn_force(const int* __restrict__ list, int a0, int na, const int* __restrict__ slot_start,
                           const int* __restrict__ slot_j, const int* __restrict__ rev, const float* __restrict__ J,
                           const float* __restrict__ U, const float* __restrict__ fref, float wF_over_ncomp,
                           const float* __restrict__ fw, const int* __restrict__ atom_conf, float* __restrict__ F,
                           float* __restrict__ rho, float* __restrict__ lossF) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= na) return;
    const int k = list[a0 + t];
    if (fref) wF_over_ncomp *= fw[atom_conf[k]];
    float uk[NN_DESC];
    for (int d = 0; d < NN_DESC; d++) uk[d] = U[(size_t)k * NN_DESC + d];
    float f[3] = {0.f, 0.f, 0.f};
    for (int s = slot_start[k]; s < slot_start[k + 1]; s++) {
        const int j = slot_j[s];
        const float* Js = J + (size_t)s * 3 * NN_DESC;
        const float* Jr = J + (size_t)rev[s] * 3 * NN_DESC;
        const float* uj = U + (size_t)j * NN_DESC;
        for (int c = 0; c < 3; c++) {
            float acc = 0.f;
            for (int d = 0; d < NN_DESC; d++) acc = fmaf(Js[c * NN_DESC + d], uk[d], acc);
            for (int d = 0; d < NN_DESC; d++) acc = fmaf(-Jr[c * NN_DESC + d], uj[d], acc);
            f[c] += acc;
        }
    }
    float l = 0.f;
    for (int c = 0; c < 3; c++) {
        F[3 * (size_t)k + c] = f[c];
        if (fref) {
            const float r = f[c] - fref[3 * (size_t)k + c];
            rho[3 * (size_t)k + c] = 2.f * wF_over_ncomp * r;
            l = fmaf(r, r, l);
        }
    }
    if (fref) lossF[t] = wF_over_ncomp * l;
}

// v_i = dL/du_i = sum_s J_is (rho_i - rho_j)
__global__ void k_nn_vvec(const int* __restrict__ list, int a0, int na, const int* __restrict__ slot_start,
                          const int* __restrict__ slot_j, const float* __restrict__ J, const float* __restrict__ rho,
                          float* __restrict__ V) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= na) return;
    const int i = list[a0 + t];
    float v[NN_DESC];
    for (int d = 0; d < NN_DESC; d++) v[d] = 0.f;
    const float ri[3] = {rho[3 * (size_t)i], rho[3 * (size_t)i + 1], rho[3 * (size_t)i + 2]};
    for (int s = slot_start[i]; s < slot_start[i + 1]; s++) {
        const int j = slot_j[s];
        const float* Js = J + (size_t)s * 3 * NN_DESC;
        for (int c = 0; c < 3; c++) {
            const float dr = ri[c] - rho[3 * (size_t)j + c];
            for (int d = 0; d < NN_DESC; d++) v[d] = fmaf(Js[c * NN_DESC + d], dr, v[d]);
        }
    }
    for (int d = 0; d < NN_DESC; d++) V[(size_t)i * NN_DESC + d] = v[d];
}

// Per-atom vectors of dL/dw: the energy term (weight e = dL/dE_i) and the
// force term d(u . v)/dw (u = dE/dG, v = dL/du) by a forward tangent dz1 = W1 v~
// followed by reverse mode through the tangent computation.
__global__ void __launch_bounds__(128) k_nn_atom_grad(const float* __restrict__ w, const float* __restrict__ Gt,
                                                      const float* __restrict__ V, NNDescParams p,
                                                      const int* __restrict__ list, const int* __restrict__ atom_conf,
                                                      const float* __restrict__ ew, const int* __restrict__ ew_index,
                                                      int a0, int na,
                                                      float* __restrict__ vecs) {
    extern __shared__ float sw[];
    load_params(w, sw);
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= na) return;
    const int atom = list[a0 + t];
    const float e = ew[ew_index ? ew_index[atom] : atom];
    const float* W1 = sw + NN_OFF_W1;
    const float* W2 = sw + NN_OFF_W2;
    const float* w3 = sw + NN_OFF_W3;
    float g[NN_DESC], vt[NN_DESC];
    for (int d = 0; d < NN_DESC; d++) {
        g[d] = Gt[(size_t)atom * NN_DESC + d];
        vt[d] = V[(size_t)atom * NN_DESC + d] * p.isig[d];
    }
    float a1[NN_H], dz1[NN_H], da1[NN_H];
    for (int j = 0; j < NN_H; j++) {
        float z = sw[NN_OFF_B1 + j], dz = 0.f;
        for (int d = 0; d < NN_DESC; d++) {
            z = fmaf(W1[j * NN_DESC + d], g[d], z);
            dz = fmaf(W1[j * NN_DESC + d], vt[d], dz);
        }
        a1[j] = tanhf(z);
        dz1[j] = dz;
        da1[j] = (1.f - a1[j] * a1[j]) * dz;
    }
    float* out = vecs + (size_t)t * NN_VEC_STRIDE;
    float d2[NN_H], r2[NN_H];
    for (int o = 0; o < NN_H; o++) {
        float z = sw[NN_OFF_B2 + o], dz = 0.f;
        for (int j = 0; j < NN_H; j++) {
            z = fmaf(W2[o * NN_H + j], a1[j], z);
            dz = fmaf(W2[o * NN_H + j], da1[j], dz);
        }
        const float a2 = tanhf(z), s2 = 1.f - a2 * a2;
        d2[o] = w3[o] * s2;
        r2[o] = w3[o] * dz * (-2.f * a2 * s2);
        out[2 * NN_H + o] = e * d2[o] + r2[o];      // zeta2
        out[3 * NN_H + o] = d2[o];                  // delta2
        out[6 * NN_H + o] = e * a2 + s2 * dz;       // w3 gradient
    }
    for (int j = 0; j < NN_H; j++) {
        float sd = 0.f, sr = 0.f;
        for (int o = 0; o < NN_H; o++) {
            sd = fmaf(d2[o], W2[o * NN_H + j], sd);
            sr = fmaf(r2[o], W2[o * NN_H + j], sr);
        }
        const float s1 = 1.f - a1[j] * a1[j];
        const float d1 = sd * s1;
        const float r1 = sr * s1 + sd * dz1[j] * (-2.f * a1[j] * s1);
        out[0 * NN_H + j] = e * d1 + r1;  // zeta1
        out[1 * NN_H + j] = d1;           // delta1
        out[4 * NN_H + j] = a1[j];
        out[5 * NN_H + j] = da1[j];
    }
    out[7 * NN_H] = e;
}

// Partial dL/dw over a chunk of NN_CHUNK batch atoms (fixed order).
__global__ void __launch_bounds__(256) k_nn_wgrad_partial(const float* __restrict__ vecs, const float* __restrict__ Gt,
                                                          const float* __restrict__ V, NNDescParams p,
                                                          const int* __restrict__ list, int a0, int na,
                                                          float* __restrict__ partial) {
    extern __shared__ float sm[];
    float* sv = sm;                              // NN_CHUNK x NN_VEC_STRIDE
    float* sg = sv + NN_CHUNK * NN_VEC_STRIDE;   // NN_CHUNK x 32
    float* sr = sg + NN_CHUNK * NN_DESC;         // NN_CHUNK x 32 (v~)
    const int t0 = blockIdx.x * NN_CHUNK;
    const int cnt = min(NN_CHUNK, na - t0);
    for (int q = threadIdx.x; q < NN_CHUNK * NN_VEC_STRIDE; q += blockDim.x) {
        const int a = q / NN_VEC_STRIDE;
        sv[q] = a < cnt ? vecs[(size_t)(t0 + a) * NN_VEC_STRIDE + q % NN_VEC_STRIDE] : 0.f;
    }
    for (int q = threadIdx.x; q < NN_CHUNK * NN_DESC; q += blockDim.x) {
        const int a = q / NN_DESC, d = q % NN_DESC;
        const int atom = a < cnt ? list[a0 + t0 + a] : 0;
        sg[q] = a < cnt ? Gt[(size_t)atom * NN_DESC + d] : 0.f;
        sr[q] = a < cnt ? V[(size_t)atom * NN_DESC + d] * p.isig[d] : 0.f;
    }
    __syncthreads();
    float* out = partial + (size_t)blockIdx.x * NN_PARAMS;
    for (int k = threadIdx.x; k < NN_PARAMS; k += blockDim.x) {
        float s = 0.f;
        if (k < NN_OFF_B1) {
            const int j = k / NN_DESC, d = k % NN_DESC;
            for (int a = 0; a < NN_CHUNK; a++) {
                const float* v = sv + a * NN_VEC_STRIDE;
                s = fmaf(v[j], sg[a * NN_DESC + d], s);
                s = fmaf(v[NN_H + j], sr[a * NN_DESC + d], s);
            }
        } else if (k < NN_OFF_W2) {
            const int j = k - NN_OFF_B1;
            for (int a = 0; a < NN_CHUNK; a++) s += sv[a * NN_VEC_STRIDE + j];
        } else if (k < NN_OFF_B2) {
            const int o = (k - NN_OFF_W2) / NN_H, j = (k - NN_OFF_W2) % NN_H;
            for (int a = 0; a < NN_CHUNK; a++) {
                const float* v = sv + a * NN_VEC_STRIDE;
                s = fmaf(v[2 * NN_H + o], v[4 * NN_H + j], s);
                s = fmaf(v[3 * NN_H + o], v[5 * NN_H + j], s);
            }
        } else if (k < NN_OFF_W3) {
            const int o = k - NN_OFF_B2;
            for (int a = 0; a < NN_CHUNK; a++) s += sv[a * NN_VEC_STRIDE + 2 * NN_H + o];
        } else if (k < NN_OFF_B3) {
            const int o = k - NN_OFF_W3;
            for (int a = 0; a < NN_CHUNK; a++) s += sv[a * NN_VEC_STRIDE + 6 * NN_H + o];
        } else {
            for (int a = 0; a < NN_CHUNK; a++) s += sv[a * NN_VEC_STRIDE + 7 * NN_H];
        }
        out[k] = s;
    }
}

__global__ void k_nn_wgrad_final(const float* __restrict__ partial, int nchunks, float* __restrict__ grad) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= NN_PARAMS) return;
    double s = 0.0;
    for (int c = 0; c < nchunks; c++) s += (double)partial[(size_t)c * NN_PARAMS + k];
    grad[k] = (float)s;
}

__global__ void k_nn_loss(const float* __restrict__ lossE, int nb, const float* __restrict__ lossF, int na,
                          double* __restrict__ loss) {
    __shared__ double red[256];
    double s = 0.0;
    for (int q = threadIdx.x; q < nb; q += blockDim.x) s += (double)lossE[q];
    for (int q = threadIdx.x; q < na; q += blockDim.x) s += (double)lossF[q];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) loss[0] = red[0];
}

__global__ void k_nn_adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                          float* __restrict__ v, float lr_t, float b1, float b2, float eps) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= NN_PARAMS) return;
    const float gk = g[k];
    const float mk = b1 * m[k] + (1.f - b1) * gk;
    const float vk = b2 * v[k] + (1.f - b2) * gk * gk;
    m[k] = mk;
    v[k] = vk;
    w[k] -= lr_t * mk / (sqrtf(vk) + eps);
}

}  // namespace omdg

// ====================================================================== C ABI
using namespace omdg;

static int nn_fail(omdg_nn* t, int code, const std::string& msg) {
    if (t) t->err = msg;
    return code;
}

static int nn_cuda(omdg_nn* t, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return OMDG_OK;
    return nn_fail(t, OMDG_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

static int nn_status(omdg_nn* t) {
    unsigned st = 0;
    cudaError_t e = cudaMemcpyAsync(&st, t->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, t->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(t->stream);
    if (e != cudaSuccess) return nn_cuda(t, e, "status");
    if (!st) return OMDG_OK;
    unsigned zero = 0;
    cudaMemcpy(t->d_status, &zero, sizeof(unsigned), cudaMemcpyHostToDevice);
    if (st & ERR_TIMEOUT) return nn_fail(t, OMDG_ECUDA, "tensor-core kernel wait timed out");
    if (st & ERR_NBR_OVERFLOW) return nn_fail(t, OMDG_ESTATE, "asymmetric neighbour slots");
    return nn_fail(t, OMDG_ECUDA, "device status word set");
}

static void nn_free_data(omdg_nn* t) {
    cudaFree(t->d_fw);
    cudaFree(t->d_eatom);
    cudaFree(t->d_ewa);
    t->d_fw = t->d_eatom = t->d_ewa = nullptr;
    void* ptrs[] = {t->d_conf_start, t->d_atom_conf, t->d_x,     t->d_L,      t->d_eref,    t->d_fref,   t->d_slot_start,
                    t->d_slot_j,     t->d_slot_rev,  t->d_slot_d, t->d_G,     t->d_Gt,      t->d_J,      t->d_E,
                    t->d_u,          t->d_F,         t->d_rho,   t->d_vvec,   t->d_ew,      t->d_lossE,  t->d_lossF,
                    t->d_vecs,       t->d_partial,   t->d_list,  t->d_clist};
    for (void* p : ptrs) cudaFree(p);
    t->d_conf_start = t->d_atom_conf = t->d_slot_start = t->d_slot_j = t->d_slot_rev = t->d_list = t->d_clist = nullptr;
    t->d_x = t->d_L = nullptr;
    t->d_eref = t->d_fref = t->d_G = t->d_Gt = t->d_J = t->d_E = t->d_u = t->d_F = t->d_rho = t->d_vvec = nullptr;
    t->d_ew = t->d_lossE = t->d_lossF = t->d_vecs = t->d_partial = nullptr;
    t->d_slot_d = nullptr;
    t->nconf = 0;
    t->natoms = t->nslots = 0;
    t->cap_batch_atoms = 0;
}

template <typename T>
static cudaError_t dalloc(T** p, size_t count) {
    return cudaMalloc(reinterpret_cast<void**>(p), sizeof(T) * std::max<size_t>(count, 1));
}

extern "C" {

int omdg_nn_create(omdg_nn** out, int device) {
    if (!out) return OMDG_EINVAL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return OMDG_ECUDA;
    omdg_nn* t = new omdg_nn();
    t->device = device;
    cudaSetDevice(device);
    cudaDeviceGetAttribute(&t->num_sms, cudaDevAttrMultiProcessorCount, device);
    cudaError_t e = cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = dalloc(&t->d_status, 1);
    if (e == cudaSuccess) e = cudaMemset(t->d_status, 0, sizeof(unsigned));
    if (e == cudaSuccess) e = dalloc(&t->d_params, NN_PARAMS);
    if (e == cudaSuccess) e = dalloc(&t->d_adam_m, NN_PARAMS);
    if (e == cudaSuccess) e = dalloc(&t->d_adam_v, NN_PARAMS);
    if (e == cudaSuccess) e = dalloc(&t->d_grad, NN_PARAMS);
    if (e == cudaSuccess) e = dalloc(&t->d_loss, 1);
    if (e != cudaSuccess) {
        delete t;
        return OMDG_ECUDA;
    }
    nn_default_descriptors(t->model.dp);
    for (int d = 0; d < NN_DESC; d++) t->model.sigma[d] = 1.f;
    t->model.w.assign(NN_PARAMS, 0.f);
    *out = t;
    return OMDG_OK;
}

int omdg_nn_destroy(omdg_nn* t) {
    if (!t) return OMDG_EINVAL;
    cudaSetDevice(t->device);
    nn_free_data(t);
    void* ptrs[] = {t->d_status, t->d_params, t->d_adam_m, t->d_adam_v, t->d_grad, t->d_loss};
    for (void* p : ptrs) cudaFree(p);
    nn_net_free(t->net);
    cudaStreamDestroy(t->stream);
    delete t;
    return OMDG_OK;
}

const char* omdg_nn_last_error(omdg_nn* t) { return t ? t->err.c_str() : "null network"; }

int omdg_nn_set_weights(omdg_nn* t, const float* params, long count) {
    if (!t || !params || count != NN_PARAMS) return t ? nn_fail(t, OMDG_EINVAL, "expected 6337 parameters") : OMDG_EINVAL;
    cudaSetDevice(t->device);
    t->model.w.assign(params, params + NN_PARAMS);
    t->have_weights = true;
    t->adam_t = 0;
    cudaError_t e = cudaMemcpyAsync(t->d_params, params, sizeof(float) * NN_PARAMS, cudaMemcpyHostToDevice, t->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(t->d_adam_m, 0, sizeof(float) * NN_PARAMS, t->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(t->d_adam_v, 0, sizeof(float) * NN_PARAMS, t->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(t->stream);
    return nn_cuda(t, e, "set weights");
}

int omdg_nn_get_weights(omdg_nn* t, float* params, long count) {
    if (!t || !params || count != NN_PARAMS) return OMDG_EINVAL;
    cudaSetDevice(t->device);
    cudaError_t e = cudaMemcpy(params, t->d_params, sizeof(float) * NN_PARAMS, cudaMemcpyDeviceToHost);
    return nn_cuda(t, e, "get weights");
}

int omdg_nn_set_normalization(omdg_nn* t, const float* mu, const float* sigma, const float* gmin, const float* gmax) {
    if (!t || !mu || !sigma) return OMDG_EINVAL;
    for (int d = 0; d < NN_DESC; d++) {
        if (!(sigma[d] > 0.f)) return nn_fail(t, OMDG_EINVAL, "sigma must be positive");
        t->model.dp.mu[d] = mu[d];
        t->model.sigma[d] = sigma[d];
        t->model.dp.isig[d] = 1.f / sigma[d];
        t->model.dp.gmin[d] = gmin ? gmin[d] : -INFINITY;
        t->model.dp.gmax[d] = gmax ? gmax[d] : INFINITY;
    }
    if (t->natoms > 0) {
        cudaSetDevice(t->device);
        const long q = t->natoms * NN_DESC;
        k_nn_normalize<<<(unsigned)((q + 255) / 256), 256, 0, t->stream>>>(t->model.dp, t->natoms, t->d_G, t->d_Gt);
        return nn_cuda(t, cudaStreamSynchronize(t->stream), "normalise");
    }
    return OMDG_OK;
}

int omdg_nn_get_normalization(omdg_nn* t, float* mu, float* sigma, float* gmin, float* gmax) {
    if (!t) return OMDG_EINVAL;
    for (int d = 0; d < NN_DESC; d++) {
        if (mu) mu[d] = t->model.dp.mu[d];
        if (sigma) sigma[d] = t->model.sigma[d];
        if (gmin) gmin[d] = t->model.dp.gmin[d];
        if (gmax) gmax[d] = t->model.dp.gmax[d];
    }
    return OMDG_OK;
}

int omdg_nn_save(omdg_nn* t, const char* path) {
    if (!t || !path) return OMDG_EINVAL;
    cudaSetDevice(t->device);
    int rc = omdg_nn_get_weights(t, t->model.w.data(), NN_PARAMS);
    if (rc) return rc;
    return nn_model_save(path, t->model, t->err);
}

int omdg_nn_load(omdg_nn* t, const char* path) {
    if (!t || !path) return OMDG_EINVAL;
    NNModel m;
    int rc = nn_model_load(path, m, t->err);
    if (rc) return rc;
    rc = omdg_nn_set_normalization(t, m.dp.mu, m.sigma, m.dp.gmin, m.dp.gmax);
    if (rc) return rc;
    t->model.dp = m.dp;
    return omdg_nn_set_weights(t, m.w.data(), NN_PARAMS);
}

int omdg_nn_set_descriptors(omdg_nn* t, const float* rs, const float* eta_r, const int* zeta, const float* lambda,
                            const float* eta_a) {
    if (!t || !rs || !eta_r || !zeta || !lambda || !eta_a) return OMDG_EINVAL;
    if (t->natoms > 0) return nn_fail(t, OMDG_ESTATE, "set the descriptors before the dataset");
    NNDescParams& p = t->model.dp;
    for (int k = 0; k < NN_RAD; k++) {
        if (!(eta_r[k] >= 0.f)) return nn_fail(t, OMDG_EINVAL, "radial eta must be >= 0");
        p.rs[k] = rs[k];
        p.eta_r[k] = eta_r[k];
    }
    for (int m = 0; m < NN_ANG; m++) {
        if (zeta[m] < 1 || zeta[m] > 16) return nn_fail(t, OMDG_EINVAL, "zeta must be an integer in [1, 16]");
        if (!(eta_a[m] >= 0.f)) return nn_fail(t, OMDG_EINVAL, "angular eta must be >= 0");
        p.zeta[m] = zeta[m];
        p.lam[m] = lambda[m];
        p.eta_a[m] = eta_a[m];
        p.pref[m] = (float)std::pow(2.0, 1.0 - zeta[m]);
    }
    return OMDG_OK;
}

int omdg_nn_set_cutoff(omdg_nn* t, float rc, float rin) {
    if (!t) return OMDG_EINVAL;
    if (t->natoms > 0) return nn_fail(t, OMDG_ESTATE, "set the cutoff before the dataset");
    if (!nn_set_cutoff(t->model.dp, rc, rin)) return nn_fail(t, OMDG_EINVAL, "the cutoff needs 0 <= rin < rc");
    return OMDG_OK;
}

int omdg_nn_set_dataset(omdg_nn* t, int nconf, const int* natoms, const double* x, const double* box_len,
                        const double* energy, const double* forces) {
    if (!t || nconf <= 0 || !natoms || !x || !box_len || !energy || !forces) return OMDG_EINVAL;
    cudaSetDevice(t->device);
    nn_free_data(t);
    const double rc = t->model.dp.rc;
    std::vector<int> start(nconf + 1, 0), atom_conf;
    for (int c = 0; c < nconf; c++) {
        if (natoms[c] <= 0) return nn_fail(t, OMDG_EINVAL, "configuration without atoms");
        for (int a = 0; a < 3; a++)
            if (!(box_len[3 * c + a] >= 2.0 * rc))
                return nn_fail(t, OMDG_EINVAL, "every box length must be at least twice the descriptor cutoff");
        start[c + 1] = start[c] + natoms[c];
        atom_conf.insert(atom_conf.end(), natoms[c], c);
    }
    const long n = start[nconf];
    std::vector<float> eref(nconf), fref(3 * (size_t)n);
    for (int c = 0; c < nconf; c++) eref[c] = (float)energy[c];
    for (long q = 0; q < 3 * n; q++) fref[q] = (float)forces[q];
    cudaError_t e = dalloc(&t->d_conf_start, nconf + 1);
    if (e == cudaSuccess) e = dalloc(&t->d_atom_conf, n);
    if (e == cudaSuccess) e = dalloc(&t->d_x, 3 * n);
    if (e == cudaSuccess) e = dalloc(&t->d_L, 3 * (size_t)nconf);
    if (e == cudaSuccess) e = dalloc(&t->d_eref, nconf);
    if (e == cudaSuccess) e = dalloc(&t->d_fref, 3 * n);
    if (e == cudaSuccess) e = dalloc(&t->d_fw, nconf);
    if (e == cudaSuccess) e = dalloc(&t->d_slot_start, n + 1);
    if (e == cudaSuccess) e = dalloc(&t->d_G, n * NN_DESC);
    if (e == cudaSuccess) e = dalloc(&t->d_Gt, n * NN_DESC);
    if (e == cudaSuccess) e = dalloc(&t->d_E, n);
    if (e == cudaSuccess) e = dalloc(&t->d_u, n * NN_DESC);
    if (e == cudaSuccess) e = dalloc(&t->d_F, 3 * n);
    if (e == cudaSuccess) e = dalloc(&t->d_rho, 3 * n);
    if (e == cudaSuccess) e = dalloc(&t->d_vvec, n * NN_DESC);
    if (e == cudaSuccess) e = dalloc(&t->d_ew, nconf);
    if (e == cudaSuccess) e = dalloc(&t->d_list, n);
    if (e == cudaSuccess) e = dalloc(&t->d_clist, nconf);
    if (e != cudaSuccess) return nn_cuda(t, e, "dataset allocation");
    cudaStream_t s = t->stream;
    cudaMemcpyAsync(t->d_conf_start, start.data(), sizeof(int) * (nconf + 1), cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(t->d_atom_conf, atom_conf.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(t->d_x, x, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(t->d_L, box_len, sizeof(double) * 3 * nconf, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(t->d_eref, eref.data(), sizeof(float) * nconf, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(t->d_fref, fref.data(), sizeof(float) * 3 * n, cudaMemcpyHostToDevice, s);
    t->fms.assign(nconf, 0.f);
    for (int c = 0; c < nconf; c++) {
        double q = 0;
        for (long a = 3L * start[c]; a < 3L * start[c + 1]; a++) q += (double)forces[a] * forces[a];
        t->fms[c] = (float)(q / (3.0 * natoms[c]));
    }
    std::vector<float> ones(nconf, 1.f);
    cudaMemcpyAsync(t->d_fw, ones.data(), sizeof(float) * nconf, cudaMemcpyHostToDevice, s);
    const unsigned blocks = (unsigned)((n + 127) / 128);
    int* d_count = t->d_slot_start;  // counts first, then converted to starts on the host
    k_nn_count<<<blocks, 128, 0, s>>>(n, t->d_atom_conf, t->d_conf_start, t->d_x, t->d_L, rc * rc, d_count);
    std::vector<int> cnt(n + 1, 0);
    e = cudaMemcpyAsync(cnt.data(), d_count, sizeof(int) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return nn_cuda(t, e, "neighbour count");
    std::vector<int> sstart(n + 1, 0);
    for (long i = 0; i < n; i++) {
        if (cnt[i] > NN_MAXN) return nn_fail(t, OMDG_ESTATE, "an atom has more than 24 neighbours inside the cutoff");
        sstart[i + 1] = sstart[i] + cnt[i];
    }
    const long ns = sstart[n];
    e = dalloc(&t->d_slot_j, ns);
    if (e == cudaSuccess) e = dalloc(&t->d_slot_rev, ns);
    if (e == cudaSuccess) e = dalloc(&t->d_slot_d, ns);
    if (e == cudaSuccess) e = dalloc(&t->d_J, (size_t)ns * 3 * NN_DESC);
    if (e != cudaSuccess) return nn_cuda(t, e, "slot allocation");
    cudaMemcpyAsync(t->d_slot_start, sstart.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s);
    k_nn_fill<<<blocks, 128, 0, s>>>(n, t->d_atom_conf, t->d_conf_start, t->d_x, t->d_L, rc * rc, t->d_slot_start,
                                     t->d_slot_j, t->d_slot_d);
    k_nn_rev<<<blocks, 128, 0, s>>>(n, t->d_slot_start, t->d_slot_j, t->d_slot_rev, t->d_status);
    k_nn_train_desc<<<blocks, 128, 0, s>>>(t->model.dp, n, t->d_slot_start, t->d_slot_d, t->d_G, t->d_J);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return nn_cuda(t, e, "descriptors");
    t->nconf = nconf;
    t->natoms = n;
    t->nslots = ns;
    t->conf_start = start;
    int rc2 = nn_status(t);
    if (rc2) return rc2;
    return omdg_nn_set_normalization(t, t->model.dp.mu, t->model.sigma, t->model.dp.gmin, t->model.dp.gmax);
}

// relative != 0: each configuration's force residual is weighted by the mean
// square reference force over the dataset divided by its own, so that every
// configuration counts by its relative force error; 0: plain mean square.
int omdg_nn_set_force_weighting(omdg_nn* t, int relative) {
    if (!t || t->nconf == 0) return OMDG_EINVAL;
    cudaSetDevice(t->device);
    std::vector<float> w(t->nconf, 1.f);
    if (relative) {
        double mean = 0;
        for (float q : t->fms) mean += q;
        mean /= t->nconf;
        for (int c = 0; c < t->nconf; c++) w[c] = t->fms[c] > 0.f ? (float)(mean / t->fms[c]) : 1.f;
    }
    cudaError_t e = cudaMemcpyAsync(t->d_fw, w.data(), sizeof(float) * t->nconf, cudaMemcpyHostToDevice, t->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(t->stream);
    return nn_cuda(t, e, "force weights");
}

// Per-atom reference energies: the energy term of the loss becomes
// wE mean_i (E_i - E_i^ref)^2 over the batch atoms; NULL returns to the
// per-configuration total-energy term.
int omdg_nn_set_atom_energies(omdg_nn* t, const double* e_atom) {
    if (!t || t->natoms == 0) return OMDG_EINVAL;
    cudaSetDevice(t->device);
    cudaFree(t->d_eatom);
    cudaFree(t->d_ewa);
    t->d_eatom = t->d_ewa = nullptr;
    if (!e_atom) return OMDG_OK;
    std::vector<float> h(e_atom, e_atom + t->natoms);
    cudaError_t e = dalloc(&t->d_eatom, t->natoms);
    if (e == cudaSuccess) e = dalloc(&t->d_ewa, t->natoms);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(t->d_eatom, h.data(), sizeof(float) * t->natoms, cudaMemcpyHostToDevice, t->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(t->stream);
    return nn_cuda(t, e, "atom energies");
}

int omdg_nn_descriptors(omdg_nn* t, float* G, long count) {
    if (!t || !G || count != t->natoms * NN_DESC) return OMDG_EINVAL;
    cudaSetDevice(t->device);
    return nn_cuda(t, cudaMemcpy(G, t->d_G, sizeof(float) * count, cudaMemcpyDeviceToHost), "descriptors");
}

// Mean, standard deviation and range of every descriptor over the dataset.
int omdg_nn_normalize_from_dataset(omdg_nn* t) {
    if (!t || t->natoms == 0) return OMDG_EINVAL;
    std::vector<float> G(t->natoms * NN_DESC);
    int rc = omdg_nn_descriptors(t, G.data(), (long)G.size());
    if (rc) return rc;
    float mu[NN_DESC], sg[NN_DESC], lo[NN_DESC], hi[NN_DESC];
    for (int d = 0; d < NN_DESC; d++) {
        double s = 0, s2 = 0;
        float a = INFINITY, b = -INFINITY;
        for (long i = 0; i < t->natoms; i++) {
            const double v = G[i * NN_DESC + d];
            s += v;
            s2 += v * v;
            a = std::min(a, (float)v);
            b = std::max(b, (float)v);
        }
        const double m = s / t->natoms;
        const double var = std::max(0.0, s2 / t->natoms - m * m);
        mu[d] = (float)m;
        // a descriptor that does not vary over the dataset keeps scale 1
        const double sd = std::sqrt(var);
        sg[d] = (float)(sd > 1e-6 * std::max(std::fabs(m), 1e-30) ? sd : 1.0);
        lo[d] = a;
        hi[d] = b;
    }
    return omdg_nn_set_normalization(t, mu, sg, lo, hi);
}

static int ensure_batch(omdg_nn* t, long atoms) {
    if (atoms <= t->cap_batch_atoms) return OMDG_OK;
    cudaFree(t->d_lossE);
    cudaFree(t->d_lossF);
    cudaFree(t->d_vecs);
    cudaFree(t->d_partial);
    const long chunks = (atoms + NN_CHUNK - 1) / NN_CHUNK;
    cudaError_t e = dalloc(&t->d_lossE, std::max<long>(t->nconf, atoms));
    if (e == cudaSuccess) e = dalloc(&t->d_lossF, atoms);
    if (e == cudaSuccess) e = dalloc(&t->d_vecs, (size_t)atoms * NN_VEC_STRIDE);
    if (e == cudaSuccess) e = dalloc(&t->d_partial, (size_t)chunks * NN_PARAMS);
    if (e != cudaSuccess) return nn_cuda(t, e, "batch allocation");
    t->cap_batch_atoms = atoms;
    return OMDG_OK;
}

// Loss and gradient over the configurations clist[c0 .. c0 + nb) whose atoms
// are list[a0 .. a0 + na); leaves dL/dw in d_grad and L in d_loss.
static int nn_loss_grad(omdg_nn* t, int c0, int nb, long a0, long na, double wE, double wF) {
    int rc = ensure_batch(t, na);
    if (rc) return rc;
    cudaStream_t s = t->stream;
    const NNDescParams& p = t->model.dp;
    const size_t wsm = sizeof(float) * NN_PARAMS;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_nn_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wsm);
        cudaFuncSetAttribute(k_nn_atom_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wsm);
        cudaFuncSetAttribute(k_nn_wgrad_partial, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(float) * NN_CHUNK * (NN_VEC_STRIDE + 2 * NN_DESC)));
        attr = true;
    }
    const unsigned gb = (unsigned)((na + 127) / 128);
    k_nn_fwd<<<gb, 128, wsm, s>>>(t->d_params, t->d_Gt, p, t->d_list, (int)a0, (int)na, t->d_E, t->d_u);
    if (t->d_eatom)
        k_nn_atom_energy<<<gb, 128, 0, s>>>(t->d_list, (int)a0, (int)na, t->d_E, t->d_eatom, (float)wE, t->d_ewa,
                                            t->d_lossE);
    else
        k_nn_conf_energy<<<nb, 256, 0, s>>>(t->d_clist, c0, nb, t->d_conf_start, t->d_E, t->d_eref, (float)wE,
                                            t->d_ew, t->d_lossE);
    k_nn_force<<<gb, 128, 0, s>>>(t->d_list, (int)a0, (int)na, t->d_slot_start, t->d_slot_j, t->d_slot_rev, t->d_J,
                                  t->d_u, t->d_fref, (float)(wF / (3.0 * na)), t->d_fw, t->d_atom_conf, t->d_F,
                                  t->d_rho, t->d_lossF);
    k_nn_vvec<<<gb, 128, 0, s>>>(t->d_list, (int)a0, (int)na, t->d_slot_start, t->d_slot_j, t->d_J, t->d_rho,
                                 t->d_vvec);
    k_nn_atom_grad<<<gb, 128, wsm, s>>>(t->d_params, t->d_Gt, t->d_vvec, p, t->d_list, t->d_atom_conf,
                                        t->d_eatom ? t->d_ewa : t->d_ew, t->d_eatom ? nullptr : t->d_atom_conf,
                                        (int)a0, (int)na, t->d_vecs);
    const int chunks = (int)((na + NN_CHUNK - 1) / NN_CHUNK);
    k_nn_wgrad_partial<<<chunks, 256, sizeof(float) * NN_CHUNK * (NN_VEC_STRIDE + 2 * NN_DESC), s>>>(
        t->d_vecs, t->d_Gt, t->d_vvec, p, t->d_list, (int)a0, (int)na, t->d_partial);
    k_nn_wgrad_final<<<(NN_PARAMS + 255) / 256, 256, 0, s>>>(t->d_partial, chunks, t->d_grad);
    k_nn_loss<<<1, 256, 0, s>>>(t->d_lossE, t->d_eatom ? (int)na : nb, t->d_lossF, (int)na, t->d_loss);
    return nn_cuda(t, cudaGetLastError(), "training step");
}

static int upload_order(omdg_nn* t, const std::vector<int>& confs, std::vector<long>& conf_atoms0) {
    std::vector<int> list;
    list.reserve(t->natoms);
    conf_atoms0.assign(confs.size() + 1, 0);
    for (size_t k = 0; k < confs.size(); k++) {
        const int c = confs[k];
        for (int a = t->conf_start[c]; a < t->conf_start[c + 1]; a++) list.push_back(a);
        conf_atoms0[k + 1] = (long)list.size();
    }
    cudaError_t e = cudaMemcpyAsync(t->d_list, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice,
                                    t->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(t->d_clist, confs.data(), sizeof(int) * confs.size(), cudaMemcpyHostToDevice, t->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(t->stream);
    return nn_cuda(t, e, "batch order");
}

int omdg_nn_gradient(omdg_nn* t, int conf0, int nconf, double wE, double wF, double* loss, float* grad) {
    if (!t || conf0 < 0 || nconf <= 0 || conf0 + nconf > t->nconf) return OMDG_EINVAL;
    cudaSetDevice(t->device);
    std::vector<int> confs(nconf);
    std::iota(confs.begin(), confs.end(), conf0);
    std::vector<long> ca;
    int rc = upload_order(t, confs, ca);
    if (rc) return rc;
    if ((rc = nn_loss_grad(t, 0, nconf, 0, ca[nconf], wE, wF))) return rc;
    cudaError_t e = cudaSuccess;
    if (loss) e = cudaMemcpyAsync(loss, t->d_loss, sizeof(double), cudaMemcpyDeviceToHost, t->stream);
    if (grad && e == cudaSuccess)
        e = cudaMemcpyAsync(grad, t->d_grad, sizeof(float) * NN_PARAMS, cudaMemcpyDeviceToHost, t->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(t->stream);
    if (e != cudaSuccess) return nn_cuda(t, e, "gradient");
    return nn_status(t);
}

int omdg_nn_train(omdg_nn* t, int epochs, int batch_confs, double lr, double lr_final, double wE, double wF,
                  unsigned seed, double* epoch_loss) {
    if (!t || epochs <= 0 || batch_confs <= 0 || !(lr > 0) || !(lr_final > 0) || t->nconf == 0) return OMDG_EINVAL;
    cudaSetDevice(t->device);
    std::mt19937 rng(seed);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    std::vector<int> confs(t->nconf);
    std::iota(confs.begin(), confs.end(), 0);
    for (int ep = 0; ep < epochs; ep++) {
        // cosine decay from lr (first epoch) to lr_final (last epoch)
        const double lr_ep =
            epochs > 1 ? lr_final + 0.5 * (lr - lr_final) * (1.0 + std::cos(M_PI * ep / (epochs - 1))) : lr;
        std::shuffle(confs.begin(), confs.end(), rng);
        std::vector<long> ca;
        int rc = upload_order(t, confs, ca);
        if (rc) return rc;
        double sum = 0.0;
        int nbatch = 0;
        for (int c0 = 0; c0 < t->nconf; c0 += batch_confs) {
            const int nb = std::min(batch_confs, t->nconf - c0);
            if ((rc = nn_loss_grad(t, c0, nb, ca[c0], ca[c0 + nb] - ca[c0], wE, wF))) return rc;
            t->adam_t++;
            const double bc1 = 1.0 - std::pow((double)b1, (double)t->adam_t);
            const double bc2 = 1.0 - std::pow((double)b2, (double)t->adam_t);
            const float lr_t = (float)(lr_ep * std::sqrt(bc2) / bc1);
            k_nn_adam<<<(NN_PARAMS + 255) / 256, 256, 0, t->stream>>>(t->d_params, t->d_grad, t->d_adam_m,
                                                                      t->d_adam_v, lr_t, b1, b2, eps);
            if (epoch_loss) {
                double l = 0;
                cudaMemcpyAsync(&l, t->d_loss, sizeof(double), cudaMemcpyDeviceToHost, t->stream);
                cudaStreamSynchronize(t->stream);
                sum += l;
            }
            nbatch++;
        }
        cudaError_t e = cudaStreamSynchronize(t->stream);
        if (e != cudaSuccess) return nn_cuda(t, e, "training");
        if (epoch_loss) epoch_loss[ep] = sum / std::max(1, nbatch);
    }
    int rc = nn_status(t);
    if (rc) return rc;
    return omdg_nn_get_weights(t, t->model.w.data(), NN_PARAMS);
}

// Energies per atom and forces of configurations [conf0, conf0 + nconf) with
// the tensor-core network (BF16 weights and activations, FP32 accumulation).
int omdg_nn_predict(omdg_nn* t, int conf0, int nconf, int fp32, double* energy_per_atom, double* forces) {
    if (!t || conf0 < 0 || nconf <= 0 || conf0 + nconf > t->nconf) return OMDG_EINVAL;
    cudaSetDevice(t->device);
    int rc = omdg_nn_get_weights(t, t->model.w.data(), NN_PARAMS);
    if (rc) return rc;
    if ((rc = nn_net_upload(t->net, t->model, t->stream, t->err))) return rc;
    std::vector<int> confs(nconf);
    std::iota(confs.begin(), confs.end(), conf0);
    std::vector<long> ca;
    if ((rc = upload_order(t, confs, ca))) return rc;
    const long a0 = t->conf_start[conf0], na = t->conf_start[conf0 + nconf] - a0;
    const unsigned gb = (unsigned)((na + 127) / 128);
    cudaError_t e = cudaSuccess;
    if (fp32) {
        const size_t wsm = sizeof(float) * NN_PARAMS;
        cudaFuncSetAttribute(k_nn_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wsm);
        k_nn_fwd<<<gb, 128, wsm, t->stream>>>(t->d_params, t->d_Gt, t->model.dp, t->d_list, 0, (int)na, t->d_E,
                                              t->d_u);
        e = cudaGetLastError();
    } else {
        e = nn_mlp_launch(t->net, t->d_Gt + a0 * NN_DESC, (int)na, t->d_E + a0, t->d_u + a0 * NN_DESC, t->d_status,
                          t->num_sms, t->stream);
    }
    if (e != cudaSuccess) return nn_cuda(t, e, "network");
    k_nn_force<<<gb, 128, 0, t->stream>>>(t->d_list, 0, (int)na, t->d_slot_start, t->d_slot_j, t->d_slot_rev, t->d_J,
                                          t->d_u, nullptr, 0.f, nullptr, nullptr, t->d_F, nullptr, nullptr);
    std::vector<float> E(na), F(3 * na);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(E.data(), t->d_E + a0, sizeof(float) * na, cudaMemcpyDeviceToHost, t->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(F.data(), t->d_F + 3 * a0, sizeof(float) * 3 * na, cudaMemcpyDeviceToHost, t->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(t->stream);
    if (e != cudaSuccess) return nn_cuda(t, e, "predict");
    if ((rc = nn_status(t))) return rc;
    for (long i = 0; i < na; i++) {
        if (energy_per_atom) energy_per_atom[i] = E[i];
        if (forces)
            for (int c = 0; c < 3; c++) forces[3 * i + c] = F[3 * i + c];
    }
    return OMDG_OK;
}

}  // extern "C"
