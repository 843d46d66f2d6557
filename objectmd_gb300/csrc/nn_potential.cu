// The neural surrogate as a force kernel of a context (no reference
// counterpart).  Per force evaluation:
//   k_nn_md_desc   descriptors of every atom from the Verlet list; an atom
//                  with a descriptor outside the training range is flagged
//   k_nn_mlp       the network on the tensor cores: E_i and u_i = dE_i/dG_i
//   k_nn_md_force  u_i contracted with the descriptor derivatives: the force
//                  on each neighbour goes to i's slot, the rest to i
//   k_tersoff_a    (fallback) plain Tersoff for the flagged centres only
//   k_slot_gather  every atom collects the slots that point at it
// Flagged atoms take their energy and forces from Tersoff; all others from the
// network, so the total is the energy of that mixed per-atom decomposition.
#include <string>

#include "nn_md.cuh"

namespace omdg {

struct NNState {
    NNModel model;
    NNDevNet net;
    float* Gt = nullptr;   // n x 32 normalised descriptors
    float* E = nullptr;    // n
    float* U = nullptr;    // n x 32 dE/dG
    int* flag = nullptr;   // n: 1 = outside the training range
    int* count = nullptr;  // flagged atoms in the last evaluation
    int cap = 0;
    int fallback = -1;     // index of the Tersoff potential in ctx->pots
};

// STD: the default angular layout (zeta and lambda constants of the term loop)
template <bool STD>
__global__ void __launch_bounds__(128) k_nn_md_desc(NNMD q, NNDescParams p, const PosPack* __restrict__ pack,
                                                    const unsigned* __restrict__ nbr, const int* __restrict__ nnb,
                                                    float* __restrict__ Gt, int* __restrict__ flag, int* count,
                                                    unsigned* status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= q.n) return;
    float g[NN_DESC];
    nn_md_descriptors<STD>(q, p, i, pack, nbr, nnb[i], g, status);
    float4* dst = reinterpret_cast<float4*>(Gt + (size_t)i * NN_DESC);
#pragma unroll
    for (int k = 0; k < NN_DESC; k += 4) {
        float4 w;
        w.x = (g[k] - p.mu[k]) * p.isig[k];
        w.y = (g[k + 1] - p.mu[k + 1]) * p.isig[k + 1];
        w.z = (g[k + 2] - p.mu[k + 2]) * p.isig[k + 2];
        w.w = (g[k + 3] - p.mu[k + 3]) * p.isig[k + 3];
        dst[k / 4] = w;
    }
    const bool out = nn_out_of_range(p, g);
    flag[i] = out ? 1 : 0;
    if (out) atomicAdd(count, 1);
}

// STD holds the shared powers of both bases: 80 registers at six blocks per
// SM, where unbounded it takes 96 (five blocks)
template <bool STD>
__global__ void __launch_bounds__(128, STD ? 6 : 7) k_nn_md_force(NNMD q, NNDescParams p, const PosPack* __restrict__ pack,
                                                     const unsigned* __restrict__ nbr, const int* __restrict__ nnb,
                                                     const float* __restrict__ E, const float* __restrict__ U,
                                                     const int* __restrict__ flag, float4* __restrict__ slot,
                                                     float* __restrict__ fx, float* __restrict__ fy,
                                                     float* __restrict__ fz, float* __restrict__ pe,
                                                     float* __restrict__ vir, unsigned* status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= q.n) return;
    const int m = nnb[i];
    for (int s = 0; s < m; s++) slot[nbr_at(i, s, q.hshift, q.maxnb)] = make_float4(0.f, 0.f, 0.f, 0.f);
    float ox = 0.f, oy = 0.f, oz = 0.f, oe = 0.f, ow = 0.f;
    if (!flag[i]) {
        float vx[NN_MAXN], vy[NN_MAXN], vz[NN_MAXN], rr[NN_MAXN], tx[NN_MAXN], ty[NN_MAXN], tz[NN_MAXN];
        int sl[NN_MAXN];
        const int nc = nn_gather(q, p, i, pack[i], pack, nbr, m, vx, vy, vz, rr, sl, status);
        float u[NN_DESC];
        const float4* src = reinterpret_cast<const float4*>(U + (size_t)i * NN_DESC);
#pragma unroll
        for (int k = 0; k < NN_DESC; k += 4) {
            const float4 w = src[k / 4];
            u[k] = w.x;
            u[k + 1] = w.y;
            u[k + 2] = w.z;
            u[k + 3] = w.w;
        }
        // radial: dE/dx_j = (sum_k u_k dG_k/dr) e_j
        for (int a = 0; a < nc; a++) {
            float dfc;
            const float fc = nn_fc(p, rr[a], dfc);
            float c = 0.f;
#pragma unroll
            for (int k = 0; k < NN_RAD; k++) {
                float v, ddr;
                nn_radial(p, rr[a], fc, dfc, k, v, ddr);
                c = fmaf(u[k], ddr, c);
            }
            const float ir = 1.f / rr[a];
            tx[a] = c * vx[a] * ir;
            ty[a] = c * vy[a] * ir;
            tz[a] = c * vz[a] * ir;
        }
        // angular: through r_a, r_b and cos(theta)
        for (int a = 0; a < nc; a++) {
            float dfa;
            const float fa = nn_fc(p, rr[a], dfa);
            const float ia = 1.f / rr[a];
            const float ea[3] = {vx[a] * ia, vy[a] * ia, vz[a] * ia};
            for (int b = a + 1; b < nc; b++) {
                float dfb;
                const float fb = nn_fc(p, rr[b], dfb);
                const float ib = 1.f / rr[b];
                const float eb[3] = {vx[b] * ib, vy[b] * ib, vz[b] * ib};
                const float cs = ea[0] * eb[0] + ea[1] * eb[1] + ea[2] * eb[2];
                float cra = 0.f, crb = 0.f, ccs = 0.f;
                const float s2 = rr[a] * rr[a] + rr[b] * rr[b];
                NNAngExp ex;
#pragma unroll
                for (int mm = 0; mm < NN_ANG; mm++) {
                    float v, d_ra, d_rb, d_cs;
                    nn_angular<STD>(p, mm, rr[a], rr[b], cs, fa, dfa, fb, dfb, ex.get(p.eta_a[mm], s2), v, d_ra,
                                    d_rb, d_cs);
                    const float w = u[NN_RAD + mm];
                    cra = fmaf(w, d_ra, cra);
                    crb = fmaf(w, d_rb, crb);
                    ccs = fmaf(w, d_cs, ccs);
                }
                tx[a] += cra * ea[0] + ccs * (eb[0] - cs * ea[0]) * ia;
                ty[a] += cra * ea[1] + ccs * (eb[1] - cs * ea[1]) * ia;
                tz[a] += cra * ea[2] + ccs * (eb[2] - cs * ea[2]) * ia;
                tx[b] += crb * eb[0] + ccs * (ea[0] - cs * eb[0]) * ib;
                ty[b] += crb * eb[1] + ccs * (ea[1] - cs * eb[1]) * ib;
                tz[b] += crb * eb[2] + ccs * (ea[2] - cs * eb[2]) * ib;
            }
        }
        for (int a = 0; a < nc; a++) {
            slot[nbr_at(i, sl[a], q.hshift, q.maxnb)] = make_float4(-tx[a], -ty[a], -tz[a], 0.f);
            ox += tx[a];
            oy += ty[a];
            oz += tz[a];
            ow -= vx[a] * tx[a] + vy[a] * ty[a] + vz[a] * tz[a];  // (x_i - x_j) . dE_i/dx_j
        }
        oe = E[i];
    }
    if (q.first) {
        fx[i] = ox;
        fy[i] = oy;
        fz[i] = oz;
        pe[i] = oe;
        vir[i] = ow;
    } else {
        fx[i] += ox;
        fy[i] += oy;
        fz[i] += oz;
        pe[i] += oe;
        vir[i] += ow;
    }
}

static int nn_ensure(Context* c, NNState& s) {
    if (s.cap >= c->n) return OMDG_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(c->stream, &cs);
    if (cs != cudaStreamCaptureStatusNone) return set_error(c, OMDG_ESTATE, "surrogate buffers missing in capture");
    cudaFree(s.Gt);
    cudaFree(s.E);
    cudaFree(s.U);
    cudaFree(s.flag);
    const size_t n = (size_t)std::max(c->cap, c->n);
    cudaError_t e = cudaMalloc(&s.Gt, sizeof(float) * n * NN_DESC);
    if (e == cudaSuccess) e = cudaMalloc(&s.E, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&s.U, sizeof(float) * n * NN_DESC);
    if (e == cudaSuccess) e = cudaMalloc(&s.flag, sizeof(int) * n);
    if (e == cudaSuccess && !s.count) e = cudaMalloc(&s.count, sizeof(int));
    if (e != cudaSuccess) return set_error(c, OMDG_ENOMEM, "surrogate buffers");
    s.cap = (int)n;
    invalidate_graph(c);  // a captured step holds the old buffers
    return OMDG_OK;
}

int nn_launch(Context* c, Potential& pot, bool first) {
    if (!c->rev || !c->slot_buf) return set_error(c, OMDG_ESTATE, "three-body buffers missing");
    NNState& s = *pot.nn;
    int rc = nn_ensure(c, s);
    if (rc) return rc;
    NNMD q;
    q.n = c->n;
    q.hshift = c->nbr_hshift;
    q.maxnb = c->maxnb;
    q.first = first ? 1 : 0;
    q.L = make_shift(c->box);
    q.rc2 = s.model.dp.rc * s.model.dp.rc * 1.0001f;
    const unsigned grid = (unsigned)grid_for(c->n, 128);
    const unsigned* nbr = reinterpret_cast<const unsigned*>(c->nbr);
    cudaMemsetAsync(s.count, 0, sizeof(int), c->stream);
    const bool std_ang = nn_std_angular(s.model.dp);
    cudaError_t e;
    if (c->nn_fused) {
        // descriptors computed by the network kernel's own threads
        prof_begin(c, "nn_desc_mlp");
        e = nn_mlp_md_launch(s.net, q, s.model.dp, std_ang, c->pack, nbr, c->nnb, s.flag, s.count, s.E, s.U,
                             c->d_status, c->num_sms, c->stream);
        prof_end(c);
        c->launches -= 1;
    } else {
        prof_begin(c, "nn_descriptors");
        auto desc = std_ang ? k_nn_md_desc<true> : k_nn_md_desc<false>;
        desc<<<grid, 128, 0, c->stream>>>(q, s.model.dp, c->pack, nbr, c->nnb, s.Gt, s.flag, s.count, c->d_status);
        prof_end(c);
        prof_begin(c, "nn_mlp");
        e = nn_mlp_launch(s.net, s.Gt, c->n, s.E, s.U, c->d_status, c->num_sms, c->stream);
        prof_end(c);
    }
    if (e != cudaSuccess) return check_cuda(c, e, "surrogate network");
    prof_begin(c, "nn_force");
    auto force = std_ang ? k_nn_md_force<true> : k_nn_md_force<false>;
    force<<<grid, 128, 0, c->stream>>>(q, s.model.dp, c->pack, nbr, c->nnb, s.E, s.U, s.flag, c->slot_buf, c->fx,
                                       c->fy, c->fz, c->pe, c->vir, c->d_status);
    prof_end(c);
    c->launches += 3;
    if ((rc = check_cuda(c, cudaGetLastError(), "surrogate"))) return rc;
    if (s.fallback >= 0 && (rc = tersoff_centre(c, c->pots[s.fallback], false, s.flag, s.count))) return rc;
    return gather_slots(c, false);
}

void nn_release(Potential& pot) {
    if (!pot.nn) return;
    NNState& s = *pot.nn;
    nn_net_free(s.net);
    cudaFree(s.Gt);
    cudaFree(s.E);
    cudaFree(s.U);
    cudaFree(s.flag);
    cudaFree(s.count);
    delete pot.nn;
    pot.nn = nullptr;
}

}  // namespace omdg

using namespace omdg;

extern "C" {

int omdg_add_nn(omdg_ctx* c, int ta, int tb, const char* model_file, const char* tersoff_fallback) {
    if (!c || !model_file) return OMDG_EINVAL;
    if (ta < 0 || tb < 0 || ta >= MAX_TYPES || tb >= MAX_TYPES) return set_error(c, OMDG_EINVAL, "bad type id");
    if (c->ntypes > 1) return set_error(c, OMDG_EINVAL, "the surrogate handles one atom type");
    if (c->use_f64) return set_error(c, OMDG_EINVAL, "the surrogate cannot be combined with FP64 kernels");
    cudaSetDevice(c->device);
    Potential p;
    p.kind = POT_NN;
    p.ta = ta;
    p.tb = tb;
    p.nn = new NNState();
    std::string err;
    int rc = nn_model_load(model_file, p.nn->model, err);
    if (rc == OMDG_OK) rc = nn_net_upload(p.nn->net, p.nn->model, c->stream, err);
    if (rc) {
        nn_release(p);
        return set_error(c, rc, err);
    }
    p.rc = p.nn->model.dp.rc;
    if (tersoff_fallback) {
        rc = omdg_add_tersoff(c, ta, tb, tersoff_fallback);
        if (rc) {
            nn_release(p);
            return rc;
        }
        c->pots.back().fallback_only = true;
        p.nn->fallback = (int)c->pots.size() - 1;
    }
    c->pots.push_back(p);
    c->need_rev = true;
    update_rc(c);
    return OMDG_OK;
}

int omdg_nn_fallback_atoms(omdg_ctx* c, long* atoms) {
    if (!c || !atoms) return OMDG_EINVAL;
    cudaSetDevice(c->device);
    for (auto& p : c->pots)
        if (p.kind == POT_NN) {
            int h = 0;
            if (!p.nn->count) {  // not evaluated yet
                *atoms = 0;
                return OMDG_OK;
            }
            cudaError_t e = cudaMemcpyAsync(&h, p.nn->count, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
            if (e != cudaSuccess) return check_cuda(c, e, "fallback count");
            *atoms = h;
            return OMDG_OK;
        }
    return set_error(c, OMDG_ESTATE, "no surrogate registered");
}

}  // extern "C"
