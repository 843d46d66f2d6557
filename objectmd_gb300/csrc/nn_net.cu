// The surrogate's network on the 5th-generation tensor cores, plus the model
// file.  No reference counterpart.
//
// k_nn_mlp evaluates, for 128 atoms per tile (one row per thread, 4 warps):
//   z1 = G~ W1^T        (MMA M=128 N=64 K=32)   a1 = tanh(z1 + b1)
//   z2 = a1 W2^T        (MMA M=128 N=64 K=64)   a2 = tanh(z2 + b2)
//   E  = w3 . a2 + b3   d2 = w3 (1 - a2^2)
//   g1 = d2 W2          (MMA M=128 N=64 K=64)   d1 = g1 (1 - a1^2)
//   u~ = d1 W1          (MMA M=128 N=32 K=32)   u  = u~ * isig  (dE/dG)
// with BF16 operands in shared memory and FP32 accumulators in TMEM.  The
// four weight tiles (24 KB) and the FP32 vectors come in by one bulk copy per
// CTA; the CTA then walks tiles (persistent).  One thread issues the MMAs;
// every wait is bounded and an expired wait aborts the CTA with ERR_TIMEOUT.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>

#include "nn_internal.h"
#include "nn_md.cuh"
#include "tc_common.cuh"

namespace omdg {

// ------------------------------------------------------------------ model
bool nn_set_cutoff(NNDescParams& dp, float rc, float rin) {
    if (!(rin >= 0.f && rin < rc && std::isfinite(rc))) return false;
    dp.rc = rc;
    dp.rin = rin;
    dp.pi_rc = (float)(M_PI / ((double)rc - (double)rin));
    return true;
}

void nn_default_descriptors(NNDescParams& dp) {
    const double rc = 3.2, r0 = 1.6;
    const double h = (rc - r0) / (NN_RAD - 1);
    for (int k = 0; k < NN_RAD; k++) {
        dp.rs[k] = (float)(r0 + k * h);
        dp.eta_r[k] = (float)(1.0 / (2.0 * h * h));
    }
    const double eta[2] = {0.0, 0.3};
    const int zeta[4] = {1, 2, 4, 8};
    const double lam[2] = {1.0, -1.0};
    int m = 0;
    for (int e = 0; e < 2; e++)
        for (int z = 0; z < 4; z++)
            for (int l = 0; l < 2; l++, m++) {
                dp.eta_a[m] = (float)eta[e];
                dp.zeta[m] = zeta[z];
                dp.lam[m] = (float)lam[l];
                dp.pref[m] = (float)std::pow(2.0, 1.0 - zeta[z]);
            }
    nn_set_cutoff(dp, (float)rc, 0.f);
    for (int d = 0; d < NN_DESC; d++) {
        dp.mu[d] = 0.f;
        dp.isig[d] = 1.f;
        dp.gmin[d] = -INFINITY;
        dp.gmax[d] = INFINITY;
    }
}

static void put(std::ostream& o, const char* name, const float* v, int n) {
    o << name;
    char b[32];
    for (int k = 0; k < n; k++) {
        snprintf(b, sizeof(b), " %.9g", (double)v[k]);
        o << b;
    }
    o << "\n";
}

int nn_model_save(const std::string& path, const NNModel& m, std::string& err) {
    std::ofstream o(path);
    if (!o) {
        err = "cannot write " + path;
        return OMDG_EFILE;
    }
    const NNDescParams& p = m.dp;
    o << "omdg-nn 1\n";
    put(o, "rc", &p.rc, 1);
    put(o, "rin", &p.rin, 1);
    put(o, "rs", p.rs, NN_RAD);
    put(o, "eta_r", p.eta_r, NN_RAD);
    float z[NN_ANG];
    for (int k = 0; k < NN_ANG; k++) z[k] = (float)p.zeta[k];
    put(o, "zeta", z, NN_ANG);
    put(o, "lambda", p.lam, NN_ANG);
    put(o, "eta_a", p.eta_a, NN_ANG);
    put(o, "mu", p.mu, NN_DESC);
    put(o, "sigma", m.sigma, NN_DESC);
    put(o, "gmin", p.gmin, NN_DESC);
    put(o, "gmax", p.gmax, NN_DESC);
    o << "params " << NN_PARAMS << "\n";
    put(o, "w", m.w.data(), NN_PARAMS);
    return o ? OMDG_OK : (err = "write failed: " + path, OMDG_EFILE);
}

int nn_model_load(const std::string& path, NNModel& m, std::string& err) {
    std::ifstream in(path);
    if (!in) {
        err = "cannot open " + path;
        return OMDG_EFILE;
    }
    std::string magic;
    int version = 0;
    in >> magic >> version;
    if (magic != "omdg-nn" || version != 1) {
        err = path + ": not an omdg-nn version 1 model";
        return OMDG_EFILE;
    }
    nn_default_descriptors(m.dp);
    m.w.assign(NN_PARAMS, 0.f);
    std::string key;
    auto read = [&](float* v, int n) {
        for (int k = 0; k < n; k++)
            if (!(in >> v[k])) return false;
        return true;
    };
    bool have_w = false;
    while (in >> key) {
        bool ok = true;
        NNDescParams& p = m.dp;
        if (key == "rc") ok = read(&p.rc, 1);
        else if (key == "rin") ok = read(&p.rin, 1);
        else if (key == "rs") ok = read(p.rs, NN_RAD);
        else if (key == "eta_r") ok = read(p.eta_r, NN_RAD);
        else if (key == "zeta") {
            float z[NN_ANG];
            ok = read(z, NN_ANG);
            for (int k = 0; ok && k < NN_ANG; k++) {
                p.zeta[k] = (int)z[k];
                if (p.zeta[k] < 1 || p.zeta[k] > 16 || (float)p.zeta[k] != z[k]) ok = false;
                p.pref[k] = (float)std::pow(2.0, 1.0 - p.zeta[k]);
            }
        } else if (key == "lambda") ok = read(p.lam, NN_ANG);
        else if (key == "eta_a") ok = read(p.eta_a, NN_ANG);
        else if (key == "mu") ok = read(p.mu, NN_DESC);
        else if (key == "sigma") ok = read(m.sigma, NN_DESC);
        else if (key == "gmin") ok = read(p.gmin, NN_DESC);
        else if (key == "gmax") ok = read(p.gmax, NN_DESC);
        else if (key == "params") {
            int np = 0;
            ok = (bool)(in >> np) && np == NN_PARAMS;
        } else if (key == "w") {
            ok = read(m.w.data(), NN_PARAMS);
            have_w = ok;
        } else {
            err = path + ": unknown key " + key;
            return OMDG_EFILE;
        }
        if (!ok) {
            err = path + ": bad values for " + key;
            return OMDG_EFILE;
        }
    }
    if (!have_w) {
        err = path + ": no parameters";
        return OMDG_EFILE;
    }
    if (!nn_set_cutoff(m.dp, m.dp.rc, m.dp.rin)) {
        err = path + ": the cutoff needs 0 <= rin < rc";
        return OMDG_EFILE;
    }
    for (int d = 0; d < NN_DESC; d++) {
        if (!(m.sigma[d] > 0.f)) {
            err = path + ": sigma must be positive";
            return OMDG_EFILE;
        }
        m.dp.isig[d] = 1.f / m.sigma[d];
    }
    return OMDG_OK;
}

// ------------------------------------------------------------------ device image
static uint16_t bf16_bits(float f) {  // round to nearest even
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

int nn_net_upload(NNDevNet& net, const NNModel& m, cudaStream_t s, std::string& err) {
    if ((int)m.w.size() != NN_PARAMS) {
        err = "network parameters missing";
        return OMDG_ESTATE;
    }
    std::vector<uint16_t> img(NN_IMG_ELEMS, 0);
    const float* W1 = m.w.data() + NN_OFF_W1;
    const float* W2 = m.w.data() + NN_OFF_W2;
    for (int j = 0; j < NN_H; j++)
        for (int d = 0; d < NN_DESC; d++) {
            img[NN_IMG_W1 + tc_tile_off(j, d, NN_DESC)] = bf16_bits(W1[j * NN_DESC + d]);
            img[NN_IMG_W1T + tc_tile_off(d, j, NN_H)] = bf16_bits(W1[j * NN_DESC + d]);
        }
    for (int o = 0; o < NN_H; o++)
        for (int j = 0; j < NN_H; j++) {
            img[NN_IMG_W2 + tc_tile_off(o, j, NN_H)] = bf16_bits(W2[o * NN_H + j]);
            img[NN_IMG_W2T + tc_tile_off(j, o, NN_H)] = bf16_bits(W2[o * NN_H + j]);
        }
    std::vector<float> vec(NN_VEC_FLOATS, 0.f);
    for (int k = 0; k < NN_H; k++) {
        vec[NN_VEC_B1 + k] = m.w[NN_OFF_B1 + k];
        vec[NN_VEC_B2 + k] = m.w[NN_OFF_B2 + k];
        vec[NN_VEC_W3 + k] = m.w[NN_OFF_W3 + k];
    }
    vec[NN_VEC_B3] = m.w[NN_OFF_B3];
    for (int d = 0; d < NN_DESC; d++) vec[NN_VEC_ISIG + d] = m.dp.isig[d];
    cudaError_t e = cudaSuccess;
    if (!net.img) e = cudaMalloc(&net.img, sizeof(uint16_t) * NN_IMG_ELEMS);
    if (e == cudaSuccess && !net.vec) e = cudaMalloc(&net.vec, sizeof(float) * NN_VEC_FLOATS);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(net.img, img.data(), sizeof(uint16_t) * NN_IMG_ELEMS, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(net.vec, vec.data(), sizeof(float) * NN_VEC_FLOATS, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        err = std::string("network upload: ") + cudaGetErrorString(e);
        return OMDG_ECUDA;
    }
    return OMDG_OK;
}

void nn_net_free(NNDevNet& net) {
    cudaFree(net.img);
    cudaFree(net.vec);
    net.img = nullptr;
    net.vec = nullptr;
}

// ------------------------------------------------------------------ tensor-core kernel
constexpr int MLP_ROWS = 128;
constexpr int MLP_TMEM_COLS = 128;

struct MLPSmem {
    // weight tiles in the device-image order (one bulk copy)
    __nv_bfloat16 w1t[NN_DESC * NN_H];
    __nv_bfloat16 w1[NN_H * NN_DESC];
    __nv_bfloat16 w2[NN_H * NN_H];
    __nv_bfloat16 w2t[NN_H * NN_H];
    float vec[NN_VEC_FLOATS];
    __nv_bfloat16 x[MLP_ROWS * NN_DESC];
    __nv_bfloat16 h[MLP_ROWS * NN_H];
    uint64_t bar_load, bar_mma;
    uint32_t tmem_base;
    int abort;
};
static_assert(sizeof(__nv_bfloat16) * NN_IMG_ELEMS == offsetof(MLPSmem, vec), "image order");
static_assert(offsetof(MLPSmem, x) % 16 == 0 && offsetof(MLPSmem, h) % 16 == 0, "operand alignment");
static_assert(sizeof(MLPSmem::h) >= sizeof(float) * MLP_ROWS * NN_DESC, "dE/dG rows staged in h");

// tanh x = 1 - 2 / (e^{2x} + 1), branch-free with the hardware exponential
// and reciprocal: an absolute error of a few 1e-7 (the activations then round
// to BF16); the limits come out exactly (e^{2x} -> inf gives 1, -> 0 gives -1).
__device__ __forceinline__ float nn_tanh(float x) { return 1.f - __fdividef(2.f, __expf(2.f * x) + 1.f); }

// one row of 8 BF16 values -> 16 bytes
__device__ __forceinline__ uint4 pack8(const float* v) {
    uint4 r;
    __nv_bfloat162 p0 = __floats2bfloat162_rn(v[0], v[1]);
    __nv_bfloat162 p1 = __floats2bfloat162_rn(v[2], v[3]);
    __nv_bfloat162 p2 = __floats2bfloat162_rn(v[4], v[5]);
    __nv_bfloat162 p3 = __floats2bfloat162_rn(v[6], v[7]);
    r.x = *reinterpret_cast<uint32_t*>(&p0);
    r.y = *reinterpret_cast<uint32_t*>(&p1);
    r.z = *reinterpret_cast<uint32_t*>(&p2);
    r.w = *reinterpret_cast<uint32_t*>(&p3);
    return r;
}

// four values -> 8 bytes (the pairs pack8 makes)
__device__ __forceinline__ uint2 pack4(const float4& v) {
    uint2 r;
    __nv_bfloat162 p0 = __floats2bfloat162_rn(v.x, v.y);
    __nv_bfloat162 p1 = __floats2bfloat162_rn(v.z, v.w);
    r.x = *reinterpret_cast<uint32_t*>(&p0);
    r.y = *reinterpret_cast<uint32_t*>(&p1);
    return r;
}

// D = A (128 x K) * B (N x K)^T over K in steps of 16; one thread.
__device__ __forceinline__ void tc_gemm(uint32_t d, uint32_t a, uint32_t b, int K, uint32_t idesc) {
    const uint32_t sbo = (uint32_t)K * 16u;
    for (int kk = 0; kk < K / 16; kk++)
        tc_mma(d, tc_sdesc(a + kk * 256, 128, sbo), tc_sdesc(b + kk * 256, 128, sbo), idesc, kk > 0 ? 1u : 0u);
}

// 64 FP32 columns [col, col + 64) of this thread's lane
__device__ __forceinline__ void tc_ld64(uint32_t taddr, float* v) {
    uint32_t r0[16], r1[16], r2[16], r3[16];
    tc_ld16(taddr, r0);
    tc_ld16(taddr + 16, r1);
    tc_ld16(taddr + 32, r2);
    tc_ld16(taddr + 48, r3);
    tc_wait_ld(r0);
    tc_wait_ld(r1);
    tc_wait_ld(r2);
    tc_wait_ld(r3);
#pragma unroll
    for (int k = 0; k < 16; k++) {
        v[k] = __uint_as_float(r0[k]);
        v[16 + k] = __uint_as_float(r1[k]);
        v[32 + k] = __uint_as_float(r2[k]);
        v[48 + k] = __uint_as_float(r3[k]);
    }
}

__device__ __forceinline__ void tc_ld32(uint32_t taddr, float* v) {
    uint32_t r0[16], r1[16];
    tc_ld16(taddr, r0);
    tc_ld16(taddr + 16, r1);
    tc_wait_ld(r0);
    tc_wait_ld(r1);
#pragma unroll
    for (int k = 0; k < 16; k++) {
        v[k] = __uint_as_float(r0[k]);
        v[16 + k] = __uint_as_float(r1[k]);
    }
}

// generic-proxy tile writes -> visible to the MMA; all threads
__device__ __forceinline__ void tc_handoff() {
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
}

// Where a tile's input rows come from: normalised descriptor rows in global
// memory (training, prediction), or (MD) computed by each thread from the
// Verlet list, so the descriptors never leave the chip and their FP32 work
// overlaps the other resident CTAs' MMA round trips.
struct MLPInput {
    const float* gt;        // rows x 32 normalised descriptors (null: MD)
    NNMD q;
    NNDescParams dp;
    const PosPack* pack;
    const unsigned* nbr;
    const int* nnb;
    int* flag;              // 1: outside the training range (Tersoff fallback)
    int* count;
};

// MD: descriptors from the Verlet list (STD: the default angular layout).
template <bool MD, bool STD = false>
__global__ void __launch_bounds__(MLP_ROWS, 4) k_nn_mlp(const __nv_bfloat16* __restrict__ img,
                                                       const float* __restrict__ vec, const MLPInput in,
                                                       int rows, float* __restrict__ E, float* __restrict__ U,
                                                       unsigned* status, int polls) {
    extern __shared__ uint8_t smem_raw[];
    MLPSmem& S = *reinterpret_cast<MLPSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int t = threadIdx.x, warp = t >> 5;
    if (t == 0) {
        mbar_init(&S.bar_load, 1);
        mbar_init(&S.bar_mma, 1);
        S.abort = 0;
        mbar_fence_init();
    }
    if (warp == 0) {
        tmem_alloc(&S.tmem_base, MLP_TMEM_COLS);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem_base;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    if (t == 0) {
        mbar_expect_tx(&S.bar_load, (uint32_t)(sizeof(__nv_bfloat16) * NN_IMG_ELEMS + sizeof(float) * NN_VEC_FLOATS));
        bulk_g2s(S.w1t, img, (uint32_t)(sizeof(__nv_bfloat16) * NN_IMG_ELEMS), &S.bar_load);
        bulk_g2s(S.vec, vec, (uint32_t)(sizeof(float) * NN_VEC_FLOATS), &S.bar_load);
    }
    mbar_wait_or_drain(&S.bar_load, 0, polls, S.abort);
    __syncthreads();

    const uint32_t sx = smem_u32(S.x), sh = smem_u32(S.h);
    const uint32_t sw1 = smem_u32(S.w1), sw2 = smem_u32(S.w2), sw2t = smem_u32(S.w2t), sw1t = smem_u32(S.w1t);
    constexpr uint32_t ID64 = tc_idesc_bf16(MLP_ROWS, NN_H), ID32 = tc_idesc_bf16(MLP_ROWS, NN_DESC);
    const float* b1 = S.vec + NN_VEC_B1;
    const float* b2 = S.vec + NN_VEC_B2;
    const float* w3 = S.vec + NN_VEC_W3;
    const float* isig = S.vec + NN_VEC_ISIG;
    uint32_t phase = 0;
    const int ntiles = (rows + MLP_ROWS - 1) / MLP_ROWS;

    for (int tile = blockIdx.x; tile < ntiles && !S.abort; tile += gridDim.x) {
        const int row = tile * MLP_ROWS + t;
        const bool valid = row < rows;
        // the warp's rows [r0, r0 + 32): one contiguous run of 256 float4 in
        // the row-major descriptor and dE/dG arrays; lane l moves float4
        // j*32 + l (row (j*32 + l) / 8, quarter (j*32 + l) % 8), so every
        // global access of the warp is 512 contiguous bytes
        const int lane = t & 31, r0 = tile * MLP_ROWS + warp * 32;
        if (MD) {
            float g[NN_DESC];
            if (valid) {
                nn_md_descriptors<STD>(in.q, in.dp, row, in.pack, in.nbr, in.nnb[row], g, status);
                const bool out = nn_out_of_range(in.dp, g);
                in.flag[row] = out ? 1 : 0;
                if (out) atomicAdd(in.count, 1);
#pragma unroll
                for (int k = 0; k < NN_DESC; k++) g[k] = (g[k] - in.dp.mu[k]) * in.dp.isig[k];
            } else {
#pragma unroll
                for (int k = 0; k < NN_DESC; k++) g[k] = 0.f;
            }
#pragma unroll
            for (int k8 = 0; k8 < NN_DESC / 8; k8++)
                *reinterpret_cast<uint4*>(&S.x[tc_tile_off(t, k8 * 8, NN_DESC)]) = pack8(g + 8 * k8);
        } else {
            const float4* src = reinterpret_cast<const float4*>(in.gt) + (size_t)r0 * (NN_DESC / 4);
            float4 v[NN_DESC / 4];
#pragma unroll
            for (int j = 0; j < NN_DESC / 4; j++) {
                const int idx = j * 32 + lane;
                v[j] = r0 + (idx >> 3) < rows ? __ldg(src + idx) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (int j = 0; j < NN_DESC / 4; j++) {
                const int idx = j * 32 + lane;
                *reinterpret_cast<uint2*>(&S.x[tc_tile_off(warp * 32 + (idx >> 3), 4 * (idx & 7), NN_DESC)]) =
                    pack4(v[j]);
            }
        }
        tc_handoff();
        // Epilogues work on 32 TMEM columns at a time, and a1 is not kept
        // across the MMAs: z1 stays in columns [0, 64) until delta1, which
        // recomputes a1 from it (the same values), so no row of 64 floats
        // lives through a round trip.
        // z1 -> TMEM columns [0, 64)
        if (t == 0) {
            tc_gemm(tmem, sx, sw1, NN_DESC, ID64);
            tc_commit(&S.bar_mma);
        }
        mbar_wait_or_drain(&S.bar_mma, phase, polls, S.abort);
        phase ^= 1u;
        tc_fence_after();
#pragma unroll 1
        for (int c = 0; c < NN_H; c += 32) {
            float a1[32];
            tc_ld32(lane_base + c, a1);
#pragma unroll
            for (int k = 0; k < 32; k++) a1[k] = nn_tanh(a1[k] + b1[c + k]);
#pragma unroll
            for (int k8 = 0; k8 < 4; k8++)
                *reinterpret_cast<uint4*>(&S.h[tc_tile_off(t, c + k8 * 8, NN_H)]) = pack8(a1 + 8 * k8);
        }
        tc_handoff();
        if (S.abort) break;
        // z2 -> columns [64, 128)
        if (t == 0) {
            tc_gemm(tmem + 64, sh, sw2, NN_H, ID64);
            tc_commit(&S.bar_mma);
        }
        mbar_wait_or_drain(&S.bar_mma, phase, polls, S.abort);
        phase ^= 1u;
        tc_fence_after();
        float e = S.vec[NN_VEC_B3];
#pragma unroll 1
        for (int c = 0; c < NN_H; c += 32) {
            float z[32];
            tc_ld32(lane_base + 64 + c, z);
#pragma unroll
            for (int k = 0; k < 32; k++) {
                const float a2 = nn_tanh(z[k] + b2[c + k]);
                e = fmaf(w3[c + k], a2, e);
                z[k] = w3[c + k] * (1.f - a2 * a2);  // delta2
            }
#pragma unroll
            for (int k8 = 0; k8 < 4; k8++)
                *reinterpret_cast<uint4*>(&S.h[tc_tile_off(t, c + k8 * 8, NN_H)]) = pack8(z + 8 * k8);
        }
        tc_handoff();
        if (S.abort) break;
        // g1 = delta2 W2 -> columns [64, 128) (z2 is spent; z1 stays)
        if (t == 0) {
            tc_gemm(tmem + 64, sh, sw2t, NN_H, ID64);
            tc_commit(&S.bar_mma);
        }
        mbar_wait_or_drain(&S.bar_mma, phase, polls, S.abort);
        phase ^= 1u;
        tc_fence_after();
#pragma unroll 1
        for (int c = 0; c < NN_H; c += 32) {
            float g1[32], z1[32];
            uint32_t r0[16], r1[16], r2[16], r3[16];
            tc_ld16(lane_base + 64 + c, r0);
            tc_ld16(lane_base + 64 + c + 16, r1);
            tc_ld16(lane_base + c, r2);
            tc_ld16(lane_base + c + 16, r3);
            tc_wait_ld(r0);
            tc_wait_ld(r1);
            tc_wait_ld(r2);
            tc_wait_ld(r3);
#pragma unroll
            for (int k = 0; k < 16; k++) {
                g1[k] = __uint_as_float(r0[k]);
                g1[16 + k] = __uint_as_float(r1[k]);
                z1[k] = __uint_as_float(r2[k]);
                z1[16 + k] = __uint_as_float(r3[k]);
            }
#pragma unroll
            for (int k = 0; k < 32; k++) {
                const float a1 = nn_tanh(z1[k] + b1[c + k]);
                g1[k] *= 1.f - a1 * a1;  // delta1
            }
#pragma unroll
            for (int k8 = 0; k8 < 4; k8++)
                *reinterpret_cast<uint4*>(&S.h[tc_tile_off(t, c + k8 * 8, NN_H)]) = pack8(g1 + 8 * k8);
        }
        tc_handoff();
        if (S.abort) break;
        // u~ = delta1 W1 -> columns [64, 96)
        if (t == 0) {
            tc_gemm(tmem + 64, sh, sw1t, NN_H, ID32);
            tc_commit(&S.bar_mma);
        }
        mbar_wait_or_drain(&S.bar_mma, phase, polls, S.abort);
        phase ^= 1u;
        tc_fence_after();
        {
            float u[NN_DESC];
            tc_ld32(lane_base + 64, u);
            if (valid) E[row] = e;
            // dE/dG rows leave through the warp's quarter of S.h (free: the
            // last MMA has read it), a row's float4 q at slot q ^ (row & 7) so
            // that neither the row-wise writes nor the run-wise reads meet a
            // bank conflict; then the same contiguous runs as the loads
            float4* st = reinterpret_cast<float4*>(S.h) + warp * 32 * (NN_DESC / 4);
#pragma unroll
            for (int q = 0; q < NN_DESC / 4; q++)
                st[lane * (NN_DESC / 4) + (q ^ (lane & 7))] =
                    make_float4(u[4 * q] * isig[4 * q], u[4 * q + 1] * isig[4 * q + 1],
                                u[4 * q + 2] * isig[4 * q + 2], u[4 * q + 3] * isig[4 * q + 3]);
            __syncwarp();
            float4* dst = reinterpret_cast<float4*>(U) + (size_t)r0 * (NN_DESC / 4);
#pragma unroll
            for (int j = 0; j < NN_DESC / 4; j++) {
                const int idx = j * 32 + lane, r = idx >> 3;
                if (r0 + r < rows) dst[idx] = st[r * (NN_DESC / 4) + ((idx & 7) ^ (r & 7))];
            }
        }
        // TMEM reads done before the next tile's MMAs overwrite the columns
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
    }
    if (S.abort && t == 0) atomicOr(status, ERR_TIMEOUT);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, MLP_TMEM_COLS);
}

template <bool MD, bool STD = false>
static cudaError_t mlp_launch(const NNDevNet& net, const MLPInput& in, int rows, float* E, float* u,
                              unsigned* status, int num_sms, cudaStream_t s) {
    if (rows <= 0) return cudaSuccess;
    const size_t smem = sizeof(MLPSmem) + 1024;  // + alignment slack
    cudaError_t e =
        cudaFuncSetAttribute(k_nn_mlp<MD, STD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int tiles = (rows + MLP_ROWS - 1) / MLP_ROWS;
    // 4 CTAs per SM: about 51 KB of shared memory and 128 of the SM's 512
    // TMEM columns each, so the allocations never wait; four MMA chains overlap
    const int grid = std::min(tiles, 4 * std::max(1, num_sms));
    k_nn_mlp<MD, STD><<<grid, MLP_ROWS, smem, s>>>(net.img, net.vec, in, rows, E, u, status, tc_wait_polls());
    return cudaGetLastError();
}

cudaError_t nn_mlp_launch(const NNDevNet& net, const float* gt, int rows, float* E, float* u, unsigned* status,
                          int num_sms, cudaStream_t s) {
    MLPInput in{};
    in.gt = gt;
    return mlp_launch<false>(net, in, rows, E, u, status, num_sms, s);
}

cudaError_t nn_mlp_md_launch(const NNDevNet& net, const NNMD& q, const NNDescParams& dp, bool std_ang,
                             const PosPack* pack, const unsigned* nbr, const int* nnb, int* flag, int* count,
                             float* E, float* u, unsigned* status, int num_sms, cudaStream_t s) {
    MLPInput in{};
    in.q = q;
    in.dp = dp;
    in.pack = pack;
    in.nbr = nbr;
    in.nnb = nnb;
    in.flag = flag;
    in.count = count;
    return std_ang ? mlp_launch<true, true>(net, in, q.n, E, u, status, num_sms, s)
                   : mlp_launch<true, false>(net, in, q.n, E, u, status, num_sms, s);
}

}  // namespace omdg
