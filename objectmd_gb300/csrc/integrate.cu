// Velocity Verlet (MDIntegrator::Integrate, integrator.cpp:225-259) in FP64,
// the energy ledger (MeasurePotential/MeasureKinetic, system.cpp:1060-1094)
// and the Berendsen thermostat (TempController::PostIntegration,
// TempController.h:78-91), all driven by a device-side step state so that a
// captured step replays without host parameters.
//
//   kick_drift  v = lambda v (thermostat of the previous step), v += dt/2 f/m,
//               x += dt v, refresh the FP32 position packs, flag a rebuild
//               when an atom moved more than skin/2 since the last build
//   kick        v += dt/2 f/m, block partials of sum m v^2, sum potential,
//               sum virial (FP32 pairs, fixed order; FP64 for the totals
//               only); the last block writes the ledger row, the
//               thermostat factor and the step counter
//
// GB300's FP64 pipe is about 1/64 of its FP32 pipe: the FP64 instructions
// here are the state updates themselves (fma for v and x); conversions use
// the bit patterns, the pack refresh and the sums use FP32 pairs.
#include <vector>

#include "integrate_dev.cuh"

namespace omdg {

__global__ void __launch_bounds__(256, 8) k_kick_drift(IntParams p, double* __restrict__ x, double* __restrict__ y,
                                                    double* __restrict__ z, double* __restrict__ vx,
                                                    double* __restrict__ vy, double* __restrict__ vz,
                                                    const float* __restrict__ fx, const float* __restrict__ fy,
                                                    const float* __restrict__ fz, const double* __restrict__ f64,
                                                    const int* __restrict__ type, PosPack* __restrict__ pack,
                                                    const float4* __restrict__ xref, unsigned* __restrict__ aflag,
                                                    StepState* st, const int* __restrict__ rep_of,
                                                    int* __restrict__ rflag) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    __shared__ int moved;
    if (threadIdx.x == 0) moved = 0;
    __syncthreads();
    bool self_moved = false;  // replica mode: flag this atom's replica
    unsigned fl = 1u;
    if (i < p.n && aflag) {
        fl = aflag[i];
        // RangeLimiter::PostIntegration of the previous step (positions are
        // unchanged since): a group atom beyond box -/+ border is deactivated,
        // and the list is rebuilt without it
        if (p.range_on && (fl & 1u) && (fl & p.range_group)) {
            const double X0 = x[i], Y0 = y[i], Z0 = z[i];
            if (X0 < p.range_lo[0] || X0 > p.range_hi[0] || Y0 < p.range_lo[1] || Y0 > p.range_hi[1] ||
                Z0 < p.range_lo[2] || Z0 > p.range_hi[2]) {
                fl &= ~1u;
                aflag[i] = fl;
                moved = 1;
                self_moved = true;
            }
        }
    }
    if (i < p.n && (fl & 1u)) {  // inactive atoms: the integrator skips them (integrator.cpp:233, :250)
        const double lam = st->lambda;
        int t = type[i];
        const double h = st->hdtm[t], dt = st->dt;
        double ax, ay, az;
        if (p.use_f64) {
            ax = f64[3 * (size_t)i];
            ay = f64[3 * (size_t)i + 1];
            az = f64[3 * (size_t)i + 2];
        } else {
            ax = f2d_exact(fx[i]);
            ay = f2d_exact(fy[i]);
            az = f2d_exact(fz[i]);
        }
        double ux = vx[i], uy = vy[i], uz = vz[i];
        // a pending thermostat factor (the product by 1.0 is the identity;
        // compared by bits to keep the test off the FP64 pipe)
        if (__double_as_longlong(lam) != 0x3FF0000000000000ll) {
            ux *= lam;
            uy *= lam;
            uz *= lam;
        }
        ux = fma(ax, h, ux);
        uy = fma(ay, h, uy);
        uz = fma(az, h, uz);
        double X = fma(dt, ux, x[i]);
        double Y = fma(dt, uy, y[i]);
        double Z = fma(dt, uz, z[i]);
        vx[i] = ux;
        vy[i] = uy;
        vz[i] = uz;
        x[i] = X;
        y[i] = Y;
        z[i] = Z;
        PosPack pk;
        pack_coord(X, p.Qh[0], p.Ql[0], pk.hi.x, pk.lo.x);
        pack_coord(Y, p.Qh[1], p.Ql[1], pk.hi.y, pk.lo.y);
        pack_coord(Z, p.Qh[2], p.Ql[2], pk.hi.z, pk.lo.z);
        pk.hi.w = __int_as_float(t);
        pk.lo.w = 0.f;
        pack[i] = pk;
        float4 r0 = xref[i];
        float dx = (pk.hi.x - r0.x) + pk.lo.x, dy = (pk.hi.y - r0.y) + pk.lo.y, dz = (pk.hi.z - r0.z) + pk.lo.z;
        if (!(dx * dx + dy * dy + dz * dz <= p.half_skin2)) {  // NaN counts as moved
            moved = 1;
            self_moved = true;
        }
    }
    if (self_moved && rflag) rflag[rep_of[i]] = 1;
    __syncthreads();
    if (threadIdx.x == 0 && moved) st->rebuild = 1;
}


// Second half kick v += dt/2 f/m (kick = 1) and the energy ledger: per
// atom m v^2, the potential and the virial as FP32 pairs, a fixed xor tree
// per warp and over the warps, FP32-pair block partials; the last block to
// finish sums the partials in block order (finalize_block).
__global__ void __launch_bounds__(RED_BLOCK, 2048 / RED_BLOCK) k_kick(IntParams p, FinParams f, double* __restrict__ vx,
                                                    double* __restrict__ vy, double* __restrict__ vz,
                                                    const float* __restrict__ fx, const float* __restrict__ fy,
                                                    const float* __restrict__ fz, const double* __restrict__ f64,
                                                    const int* __restrict__ type, const float* __restrict__ pe,
                                                    const float* __restrict__ vir,
                                                    const unsigned* __restrict__ aflag, BlockPartial* __restrict__ partial,
                                                    double* __restrict__ ledger, StepState* st, int kick) {
    const int i = blockIdx.x * RED_BLOCK + threadIdx.x;
    F2 k = {0.f, 0.f}, e = {0.f, 0.f}, w = {0.f, 0.f};
    unsigned long long vmax = 0ull;  // bits of the largest squared speed
    // inactive atoms: not integrated, not measured (system.cpp:1067, :1085)
    if (i < p.n && (!aflag || (aflag[i] & 1u))) {
        const int t = type[i];
        if (kick && !p.use_f64) {
            kick_atom_terms(p, i, t, fx[i], fy[i], fz[i], pe[i], vir[i], st->hdtm[t], vx, vy, vz, k, e, w, vmax);
        } else {
            double ux = vx[i], uy = vy[i], uz = vz[i];
            if (kick) {
                const double h = st->hdtm[t];
                ux = fma(f64[3 * (size_t)i], h, ux);
                uy = fma(f64[3 * (size_t)i + 1], h, uy);
                uz = fma(f64[3 * (size_t)i + 2], h, uz);
                vx[i] = ux;
                vy[i] = uy;
                vz[i] = uz;
            }
            const F2 sx = f2_from(ux), sy = f2_from(uy), sz = f2_from(uz);
            const F2 v2 = f2_add(f2_add(f2_mul(sx, sx), f2_mul(sy, sy)), f2_mul(sz, sz));
            k = f2_mul(v2, F2{p.mh[t], p.ml[t]});
            e = p.use_f64 ? f2_from(f64[3 * (size_t)p.n + i]) : F2{pe[i], 0.f};
            w = F2{vir[i], 0.f};
            if (p.need_vmax)  // sqrv = vx*vx + vy*vy + vz*vz (system.cpp:1086)
                vmax = (unsigned long long)__double_as_longlong(
                    __dadd_rn(__dadd_rn(__dmul_rn(ux, ux), __dmul_rn(uy, uy)), __dmul_rn(uz, uz)));
        }
    }
    ledger_block(p, f, k, e, w, vmax, partial, ledger, st);
}

struct GhostParams {
    int n;
    double lo[3], hi[3], L[3], rv;
    int periodic[3];
};

__global__ void k_zero_counter(int* c) { *c = 0; }

// Periodic images the reference would hold as ghosts (comhandler.cpp:647-755:
// an atom closer than Rv to a face of a periodic axis is sent across it).
__global__ void k_count_ghosts(GhostParams g, const double* __restrict__ x, const double* __restrict__ y,
                               const double* __restrict__ z, int* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int images = 0;
    if (i < g.n) {
        const double p[3] = {x[i], y[i], z[i]};
        int prod = 1;
        for (int d = 0; d < 3; d++) {
            if (!g.periodic[d]) continue;
            double w = p[d] - floor((p[d] - g.lo[d]) / g.L[d]) * g.L[d];
            prod *= 1 + (w < g.lo[d] + g.rv) + (w > g.hi[d] - g.rv);
        }
        images = prod - 1;
    }
    // integer sums are order independent
    for (int off = 16; off > 0; off >>= 1) images += __shfl_xor_sync(0xffffffffu, images, off);
    if ((threadIdx.x & 31) == 0 && images) atomicAdd(out, images);
}

// One block per replica: kinetic (1/2 sum m v^2) and potential energy of the
// replica's atom range, summed in a fixed order.
__global__ void k_rep_sums(const int* __restrict__ start, const double* __restrict__ vx,
                           const double* __restrict__ vy, const double* __restrict__ vz,
                           const int* __restrict__ type, const double* __restrict__ mass,
                           const float* __restrict__ pe, double* __restrict__ out) {
    __shared__ double sk[256], se[256];
    const int r = blockIdx.x;
    double k = 0.0, e = 0.0;
    for (int i = start[r] + threadIdx.x; i < start[r + 1]; i += blockDim.x) {
        k = fma(mass[type[i]], fma(vx[i], vx[i], fma(vy[i], vy[i], vz[i] * vz[i])), k);
        e += (double)pe[i];
    }
    sk[threadIdx.x] = k;
    se[threadIdx.x] = e;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) {
            sk[threadIdx.x] += sk[threadIdx.x + off];
            se[threadIdx.x] += se[threadIdx.x + off];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[2 * r] = 0.5 * sk[0];
        out[2 * r + 1] = se[0];
    }
}

int replica_sums(Context* c, double* kinetic, double* potential) {
    if (c->nrep == 0 || !c->d_rep_sums || !c->d_rep_start) return set_error(c, OMDG_ESTATE, "no replicas built");
    int rc = resolve_thermostat(c);
    if (rc) return rc;
    k_rep_sums<<<c->nrep, 256, 0, c->stream>>>(c->d_rep_start, c->vx, c->vy, c->vz, c->type, c->d_mass, c->pe,
                                               c->d_rep_sums);
    std::vector<double> h(2 * (size_t)c->nrep);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h.data(), c->d_rep_sums, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return check_cuda(c, e, "replica sums");
    for (int r = 0; r < c->nrep; r++) {
        if (kinetic) kinetic[r] = h[2 * r];
        if (potential) potential[r] = h[2 * r + 1];
    }
    return OMDG_OK;
}

// PostForce modifies of the impact runs, in the order added: ForceDamper
// (ForceDamper.h:30-36: f -= factor v) and CoordClamp (CoordClamp.h:36-42:
// f = v = 0 on the clamped axes), each on its group's atoms.
struct PostOpDev {
    int kind;  // 1 damper, 2 clamp
    unsigned group;
    double factor;
    int axes;
};
constexpr int MAX_POST_OPS = 4;
struct PostParams {
    int n, nops;
    PostOpDev op[MAX_POST_OPS];
};

__global__ void k_post_force(PostParams p, const unsigned* __restrict__ aflag, float* __restrict__ fx,
                             float* __restrict__ fy, float* __restrict__ fz, double* __restrict__ f64,
                             double* __restrict__ vx, double* __restrict__ vy, double* __restrict__ vz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const unsigned fl = aflag[i];
    for (int k = 0; k < p.nops; k++) {
        const PostOpDev& o = p.op[k];
        if (o.group != ~0u && !(fl & o.group)) continue;
        if (o.kind == 1) {
            const double a = __dsub_rn(f64 ? f64[3 * (size_t)i] : (double)fx[i], __dmul_rn(o.factor, vx[i]));
            const double b = __dsub_rn(f64 ? f64[3 * (size_t)i + 1] : (double)fy[i], __dmul_rn(o.factor, vy[i]));
            const double c = __dsub_rn(f64 ? f64[3 * (size_t)i + 2] : (double)fz[i], __dmul_rn(o.factor, vz[i]));
            fx[i] = (float)a;
            fy[i] = (float)b;
            fz[i] = (float)c;
            if (f64) {
                f64[3 * (size_t)i] = a;
                f64[3 * (size_t)i + 1] = b;
                f64[3 * (size_t)i + 2] = c;
            }
        } else {
            if (o.axes & 1) {
                fx[i] = 0.f;
                vx[i] = 0.0;
                if (f64) f64[3 * (size_t)i] = 0.0;
            }
            if (o.axes & 2) {
                fy[i] = 0.f;
                vy[i] = 0.0;
                if (f64) f64[3 * (size_t)i + 1] = 0.0;
            }
            if (o.axes & 4) {
                fz[i] = 0.f;
                vz[i] = 0.0;
                if (f64) f64[3 * (size_t)i + 2] = 0.0;
            }
        }
    }
}

int post_force_modifies(Context* c) {
    if (c->post_ops.empty() || c->n == 0) return OMDG_OK;
    PostParams p;
    p.n = c->n;
    p.nops = (int)c->post_ops.size();
    if (p.nops > MAX_POST_OPS) return set_error(c, OMDG_EINVAL, "at most 4 force modifies");
    for (int k = 0; k < p.nops; k++) {
        const Context::PostOp& o = c->post_ops[k];
        p.op[k].kind = o.kind;
        p.op[k].group = group_bits(o.group);
        p.op[k].factor = o.factor;
        p.op[k].axes = o.axes;
    }
    k_post_force<<<grid_for(c->n, 256), 256, 0, c->stream>>>(p, c->aflag, c->fx, c->fy, c->fz,
                                                             c->use_f64 ? c->f64 : nullptr, c->vx, c->vy, c->vz);
    c->launches++;
    return check_cuda(c, cudaGetLastError(), "force modifies");
}

// EnergySource pulse (EnergySource.h:113-131): every active atom with
// v^2 >= (1e-6 |v|max)^2 gets v *= sqrt(1 + 2 delta / (v^2 m)).
__global__ void k_energy_source(int n, double delta, const int* __restrict__ type, const double* __restrict__ mass,
                                const unsigned* __restrict__ aflag, double* __restrict__ vx, double* __restrict__ vy,
                                double* __restrict__ vz, const StepState* st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !st->src_scale) return;
    if (aflag && !(aflag[i] & 1u)) return;
    // the reference's expressions, without contraction into fma
    const double vmax = __dmul_rn(sqrt(st->sqrmaxv), 1e-6);
    const double small = __dmul_rn(vmax, vmax);
    const double ux = vx[i], uy = vy[i], uz = vz[i];
    const double c2 = __dadd_rn(__dadd_rn(__dmul_rn(ux, ux), __dmul_rn(uy, uy)), __dmul_rn(uz, uz));
    if (c2 < small) return;
    const double chi = sqrt(__dadd_rn(1.0, __ddiv_rn(__ddiv_rn(__dmul_rn(2.0, delta), c2), mass[type[i]])));
    vx[i] = __dmul_rn(ux, chi);
    vy[i] = __dmul_rn(uy, chi);
    vz[i] = __dmul_rn(uz, chi);
}

int energy_source(Context* c) {
    if (!c->src_on || c->n == 0) return OMDG_OK;
    k_energy_source<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->src_delta, c->type, c->d_mass,
                                                                c->flags_used ? c->aflag : nullptr, c->vx, c->vy,
                                                                c->vz, reinterpret_cast<StepState*>(c->d_state));
    c->launches++;
    return check_cuda(c, cudaGetLastError(), "energy source");
}

// ------------------------------------------------------------------ host

static IntParams int_params(Context* c) {
    IntParams p;
    p.n = c->n;
    for (int t = 0; t < MAX_TYPES; t++) {
        p.mh[t] = (float)c->mass[t];
        p.ml[t] = (float)(c->mass[t] - (double)p.mh[t]);
    }
    // RangeLimiter::Init (RangeLimiter.h:21-29): the box -/+ the border
    p.range_on = c->range_on ? 1 : 0;
    p.range_group = group_bits(c->range_group);
    for (int d = 0; d < 3; d++) {
        p.range_lo[d] = c->box.lo[d] - c->range_border;
        p.range_hi[d] = c->box.hi[d] + c->range_border;
    }
    p.need_vmax = (c->dyn_update > 0 || c->src_on) ? 1 : 0;
    for (int d = 0; d < 3; d++) {
        p.org[d] = c->box.org[d];
        p.P[d] = c->box.P[d];
    }
    float hs = (float)(0.5 * c->skin);
    p.half_skin2 = hs * hs;
    p.use_f64 = c->use_f64 ? 1 : 0;
    for (int d = 0; d < 3; d++) {
        p.Q[d] = c->box.P[d] - c->box.org[d];
        p.Qh[d] = (float)p.Q[d];
        p.Ql[d] = (float)(p.Q[d] - (double)p.Qh[d]);
    }
    return p;
}

int integrate_kick_drift(Context* c, int) {
    IntParams p = int_params(c);
    prof_begin(c, "kick_drift");
    k_kick_drift<<<grid_for(c->n, 256), 256, 0, c->stream>>>(p, c->x, c->y, c->z, c->vx, c->vy, c->vz, c->fx, c->fy,
                                                             c->fz, c->f64, c->type, c->pack, c->xref,
                                                             c->flags_used ? c->aflag : nullptr,
                                                             reinterpret_cast<StepState*>(c->d_state),
                                                             c->nrep > 0 ? c->d_rep_of : nullptr,
                                                             c->nrep > 0 ? c->d_rep_flag : nullptr);
    prof_end(c);
    c->launches++;
    return check_cuda(c, cudaGetLastError(), "kick_drift");
}

static FinParams fin_params(Context* c, const IntParams& p, int count_step) {
    FinParams f;
    f.natoms = c->n;
    f.ledger_cap = c->ledger_cap;
    f.count_step = count_step;
    f.tau = c->thermo_tau;
    f.tset = c->thermo_T;
    f.temp_factor = 2.0 / 3.0 / 8.61734279e-05;
    f.ghosts = nullptr;
    f.status = c->d_status;
    f.ticket = reinterpret_cast<unsigned*>(c->d_flags + 4);
    f.need_vmax = p.need_vmax;
    f.dyn_update = c->dyn_update;
    f.dyn_apply = (count_step || c->first_measure) ? 1 : 0;
    f.dyn_maxpath = c->dyn_maxpath;
    f.dyn_maxdt = c->dyn_maxdt;
    for (int t = 0; t < MAX_TYPES; t++) f.mass[t] = c->mass[t];
    f.src_on = c->src_on ? 1 : 0;
    f.src_start = c->src_start;
    f.src_stop = c->src_start + c->src_width;
    return f;
}

// A step's second half-kick can ride in the force kernel's epilogue: FP32
// forces, and no ghost count for the thermostat (its extra launch precedes
// the kick).
bool kick_fusable(const Context* c) {
    return !c->use_f64 && !(c->thermo_count_ghosts && c->thermo_tau > 0.0) && c->post_ops.empty() && !c->ttm &&
           c->nrep == 0;
}

void kick_args(Context* c, KickArgs& ka) {
    ka.p = int_params(c);
    ka.f = fin_params(c, ka.p, 1);
    ka.partial = reinterpret_cast<BlockPartial*>(c->d_red);
    ka.partial_cap = grid_for(std::max(c->cap, c->n), 8) + 1;
    ka.st = reinterpret_cast<StepState*>(c->d_state);
}

__global__ void __launch_bounds__(1024) k_ledger_finalize(FinParams f, int nparts, const BlockPartial* partial,
                                                          double* ledger, StepState* st) {
    finalize_block(f, nparts, partial, ledger, st);
}

void launch_ledger_finalize(Context* c, const KickArgs& ka, int nparts) {
    k_ledger_finalize<<<1, 1024, 0, c->stream>>>(ka.f, nparts, ka.partial, c->d_ledger, ka.st);
    c->launches++;
}

static int reduce_and_finalize(Context* c, int kick, int count_step) {
    if (kick && count_step && c->kick_fused) {  // the force kernel's epilogue took it
        c->kick_fused = false;
        return OMDG_OK;
    }
    IntParams p = int_params(c);
    int nb = grid_for(c->n, RED_BLOCK);
    FinParams f = fin_params(c, p, count_step);
    if (c->thermo_count_ghosts && count_step && c->thermo_tau > 0.0) {
        // TempController::GetSystemTemperature divides by GetTotalAtom(), which
        // on MDSystemGrid is GetNAtom(): owners plus their periodic ghost images
        // (system.h:337, TempController.h:73-76).  Count those images: per
        // periodic axis an atom within Rv of a face has one more image.
        GhostParams g;
        g.n = c->n;
        double rv = c->rc_ref + c->skin;  // the reference's ghost shell
        for (int d = 0; d < 3; d++) {
            g.lo[d] = c->box.lo[d];
            g.hi[d] = c->box.hi[d];
            g.L[d] = c->box.L[d];
            g.periodic[d] = c->box.periodic[d];
        }
        g.rv = rv;
        k_zero_counter<<<1, 1, 0, c->stream>>>(c->d_flags + 2);
        k_count_ghosts<<<grid_for(c->n, 256), 256, 0, c->stream>>>(g, c->x, c->y, c->z, c->d_flags + 2);
        c->launches += 2;
        f.ghosts = c->d_flags + 2;
    }
    prof_begin(c, "kick");
    k_kick<<<nb, RED_BLOCK, 0, c->stream>>>(p, f, c->vx, c->vy, c->vz, c->fx, c->fy, c->fz, c->f64, c->type, c->pe,
                                            c->vir, c->flags_used ? c->aflag : nullptr,
                                            reinterpret_cast<BlockPartial*>(c->d_red), c->d_ledger,
                                            reinterpret_cast<StepState*>(c->d_state), kick);
    prof_end(c);
    c->launches += 1;
    return check_cuda(c, cudaGetLastError(), "kick");
}

int integrate_kick(Context* c, int) { return reduce_and_finalize(c, 1, 1); }

int measure_energies(Context* c, int) { return reduce_and_finalize(c, 0, 0); }

size_t step_state_bytes() { return sizeof(StepState); }

int step_state_reset(Context* c, int reset_row, int rebuild_every) {
    StepState h;
    cudaError_t e = cudaMemcpyAsync(&h, c->d_state, sizeof(StepState), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return check_cuda(c, e, "step state");
    if (reset_row) h.row = 0;
    h.rebuild_every = rebuild_every;
    e = cudaMemcpyAsync(c->d_state, &h, sizeof(StepState), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return check_cuda(c, e, "step state");
}

static void set_dt(StepState& h, const Context* c, double dt) {
    h.dt = dt;
    for (int t = 0; t < MAX_TYPES; t++) h.hdtm[t] = c->mass[t] > 0 ? (0.5 * dt) / c->mass[t] : 0.0;
}

static int state_rw(Context* c, StepState& h, bool write) {
    cudaError_t e = cudaMemcpyAsync(write ? (void*)c->d_state : (void*)&h, write ? (const void*)&h : c->d_state,
                                    sizeof(StepState), write ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost,
                                    c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return check_cuda(c, e, "step state");
}

// Step counter and elapsed time of a resumed run (from a checkpoint).
int step_state_resume(Context* c, long long step, double elapsed) {
    StepState h;
    int rc = state_rw(c, h, false);
    if (rc) return rc;
    h.step = step;
    h.elapsed = elapsed;
    return state_rw(c, h, true);
}

// TimeStep set by the caller (omdg_set_timestep) once the state exists.
int step_state_set_dt(Context* c) {
    StepState h;
    int rc = state_rw(c, h, false);
    if (rc) return rc;
    set_dt(h, c, c->dt);
    return state_rw(c, h, true);
}

int step_state_times(Context* c, double* dt, double* elapsed) {
    StepState h;
    int rc = state_rw(c, h, false);
    if (rc) return rc;
    if (dt) *dt = h.dt;
    if (elapsed) *elapsed = h.elapsed;
    return OMDG_OK;
}

// One round trip after the queued steps: the status word and the step state
// into the pinned staging block and, when rows > 0, the first `rows` ledger
// rows into the pinned ledger copy (what the queued steps write when none
// stopped early), then one stream synchronisation.
int step_state_fetch(Context* c, unsigned* status, long long* step, int* row, double* elapsed, int rows) {
    unsigned char* h = static_cast<unsigned char*>(c->h_sync);
    cudaError_t e = cudaMemcpyAsync(h, c->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h + 16, c->d_state, sizeof(StepState), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && rows > 0)
        e = cudaMemcpyAsync(c->h_ledger, c->d_ledger, sizeof(double) * LEDGER_W * rows, cudaMemcpyDeviceToHost,
                            c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return check_cuda(c, e, "step");
    const StepState* st = reinterpret_cast<const StepState*>(h + 16);
    *status = *reinterpret_cast<const unsigned*>(h);
    *step = st->step;
    *row = st->row;
    *elapsed = st->elapsed;
    return OMDG_OK;
}

__global__ void k_rewind(StepState* st, int rebuild_every) {
    st->row = 0;
    st->rebuild_every = rebuild_every;
}

// Ledger rows restart at 0 for the next omdg_step call (stream ordered, no wait).
// Device address of the step state's ledger row counter (read by kernels
// that fill columns of the current row).
const int* step_state_row(Context* c) { return &reinterpret_cast<StepState*>(c->d_state)->row; }
int* step_state_halted(Context* c) { return &reinterpret_cast<StepState*>(c->d_state)->halted; }

int step_state_rewind(Context* c) {
    k_rewind<<<1, 1, 0, c->stream>>>(reinterpret_cast<StepState*>(c->d_state), c->rebuild_every);
    c->launches++;
    return check_cuda(c, cudaGetLastError(), "step state");
}

int step_state_graph_rebuilds(Context* c, int* nrebuild) {
    StepState h;
    cudaError_t e = cudaMemcpyAsync(&h, c->d_state, sizeof(StepState), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return check_cuda(c, e, "step state");
    *nrebuild = h.nrebuild;
    return OMDG_OK;
}

int step_state_read(Context* c, long long* step, int* row, int* rebuild) {
    StepState h;
    cudaError_t e = cudaMemcpyAsync(&h, c->d_state, sizeof(StepState), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return check_cuda(c, e, "step state");
    if (step) *step = h.step;
    if (row) *row = h.row;
    if (rebuild) *rebuild = h.rebuild;
    return OMDG_OK;
}

int step_state_init(Context* c) {
    StepState h;
    h.step = 0;
    h.row = 0;
    h.rebuild = 0;
    h.lambda = 1.0;
    h.rebuild_every = c->rebuild_every;
    h.nrebuild = 0;
    set_dt(h, c, c->dyn_update > 0 ? c->dyn_maxdt : c->dt);  // DynamicTimeStep::Init with no velocity yet
    h.elapsed = 0.0;
    h.sqrmaxv = 0.0;
    h.src_first = 1;
    h.src_scale = 0;
    h.halted = 0;
    h.rebuild_all = 0;
    cudaError_t e = cudaMemcpyAsync(c->d_state, &h, sizeof(StepState), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return check_cuda(c, e, "step state");
}

__global__ void k_clear_rebuild(StepState* st) {
    st->rebuild = 0;
    st->rebuild_all = 0;  // the eager build that follows is a full one
}

// The reference scales velocities at the end of the step
// (TempController::PostIntegration); here the factor waits in the step state
// until the next kick.  Apply it before the caller reads velocities.
__global__ void k_apply_lambda(int n, double* __restrict__ vx, double* __restrict__ vy, double* __restrict__ vz,
                               const StepState* st) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double lam = st->lambda;
    vx[i] *= lam;
    vy[i] *= lam;
    vz[i] *= lam;
}

__global__ void k_reset_lambda(StepState* st) { st->lambda = 1.0; }

int resolve_thermostat(Context* c) {
    if (!c->lambda_pending) return OMDG_OK;
    StepState* st = reinterpret_cast<StepState*>(c->d_state);
    k_apply_lambda<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->vx, c->vy, c->vz, st);
    k_reset_lambda<<<1, 1, 0, c->stream>>>(st);
    c->launches += 2;
    c->lambda_pending = false;
    return check_cuda(c, cudaGetLastError(), "thermostat factor");
}

int drop_thermostat_factor(Context* c) {
    if (!c->lambda_pending) return OMDG_OK;
    k_reset_lambda<<<1, 1, 0, c->stream>>>(reinterpret_cast<StepState*>(c->d_state));
    c->launches += 1;
    c->lambda_pending = false;
    return check_cuda(c, cudaGetLastError(), "thermostat factor");
}

// Flags a rebuild when positions written by the caller moved an atom more
// than skin/2 from where the list was built.
// Positions and/or velocities from the caller (rows of three in caller
// order, at device-addressable addresses) in one pass: the sorted arrays,
// and for positions the pack in the integrator's frame and the displacement
// check against the last build (the list is kept unless an atom moved more
// than skin/2).
__global__ void __launch_bounds__(IO_BLOCK) k_upload_state(IntParams p, const int* __restrict__ inv,
                                                           const double* __restrict__ in_x,
                                                           const double* __restrict__ in_v, double* __restrict__ x,
                                                           double* __restrict__ y, double* __restrict__ z,
                                                           double* __restrict__ vx, double* __restrict__ vy,
                                                           double* __restrict__ vz, const int* __restrict__ type,
                                                           PosPack* __restrict__ pack,
                                                           const float4* __restrict__ xref, StepState* st) {
    __shared__ double s[2][3 * IO_BLOCK];
    __shared__ int moved;
    const int b0 = blockIdx.x * IO_BLOCK, cnt = min(IO_BLOCK, p.n - b0), t = threadIdx.x;
    if (t == 0) moved = 0;
    if (in_x) io_stage_in<3>(in_x, b0, cnt, s[0]);
    if (in_v) io_stage_in<3>(in_v, b0, cnt, s[1]);
    __syncthreads();
    if (t < cnt) {
        const int i = inv[b0 + t];
        if (in_v) {
            vx[i] = s[1][3 * t];
            vy[i] = s[1][3 * t + 1];
            vz[i] = s[1][3 * t + 2];
        }
        if (in_x) {
            const double X = s[0][3 * t], Y = s[0][3 * t + 1], Z = s[0][3 * t + 2];
            x[i] = X;
            y[i] = Y;
            z[i] = Z;
            PosPack pk;
            pack_coord(X, p.Qh[0], p.Ql[0], pk.hi.x, pk.lo.x);
            pack_coord(Y, p.Qh[1], p.Ql[1], pk.hi.y, pk.lo.y);
            pack_coord(Z, p.Qh[2], p.Ql[2], pk.hi.z, pk.lo.z);
            pk.hi.w = __int_as_float(type[i]);
            pk.lo.w = 0.f;
            pack[i] = pk;
            const float4 r0 = xref[i];
            const float dx = (pk.hi.x - r0.x) + pk.lo.x, dy = (pk.hi.y - r0.y) + pk.lo.y,
                        dz = (pk.hi.z - r0.z) + pk.lo.z;
            if (!(dx * dx + dy * dy + dz * dz <= p.half_skin2)) moved = 1;  // NaN counts as moved
        }
    }
    __syncthreads();
    if (t == 0 && moved) {
        st->rebuild = 1;
        st->rebuild_all = 1;
    }
}

int upload_state(Context* c, const double* in_x, const double* in_v) {
    IntParams p = int_params(c);
    k_upload_state<<<(c->n + IO_BLOCK - 1) / IO_BLOCK, IO_BLOCK, 0, c->stream>>>(
        p, c->inv, in_x, in_v, c->x, c->y, c->z, c->vx, c->vy, c->vz, c->type, c->pack, c->xref,
        reinterpret_cast<StepState*>(c->d_state));
    c->launches++;
    return check_cuda(c, cudaGetLastError(), "state upload");
}

__global__ void k_flag_all_if_requested(const StepState* st, int nrep, int* rflag) {
    if (!st->rebuild_all) return;
    for (int r = threadIdx.x; r < nrep; r += blockDim.x) rflag[r] = 1;
}

// Replica mode, eager steps: a request for every replica flags them all
// before the partial build (as the graph's predicate does).
int step_flag_requested_replicas(Context* c) {
    if (c->nrep == 0) return OMDG_OK;
    k_flag_all_if_requested<<<1, 256, 0, c->stream>>>(reinterpret_cast<StepState*>(c->d_state), c->nrep,
                                                      c->d_rep_flag);
    c->launches++;
    return check_cuda(c, cudaGetLastError(), "replica flags");
}

int step_clear_rebuild(Context* c) {
    k_clear_rebuild<<<1, 1, 0, c->stream>>>(reinterpret_cast<StepState*>(c->d_state));
    c->launches++;
    return check_cuda(c, cudaGetLastError(), "clear rebuild");
}

// Graph-side rebuild predicate: copies the request into the conditional
// handle and clears it.
// In replica mode a request for every replica sets every replica's flag
// (the build then rebuilds the flagged replicas only).
__global__ void k_set_rebuild_cond(StepState* st, cudaGraphConditionalHandle h, int nrep, int* rflag) {
    const bool go = st->rebuild && !st->halted;
    const bool all = st->rebuild_all != 0;
    __syncthreads();
    if (go && all && rflag)
        for (int r = threadIdx.x; r < nrep; r += blockDim.x) rflag[r] = 1;
    if (threadIdx.x == 0) {
        cudaGraphSetConditional(h, go ? 1u : 0u);
        if (go) st->nrebuild += 1;
        st->rebuild = 0;
        if (go) st->rebuild_all = 0;
    }
}

int launch_set_rebuild_cond(Context* c, cudaGraphConditionalHandle h) {
    k_set_rebuild_cond<<<1, 256, 0, c->stream>>>(reinterpret_cast<StepState*>(c->d_state), h, c->nrep,
                                                 c->nrep > 0 ? c->d_rep_flag : nullptr);
    c->launches++;
    return check_cuda(c, cudaGetLastError(), "rebuild predicate");
}

__global__ void k_zero_f(int n, float* fx, float* fy, float* fz, double* f64) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    fx[i] = 0.f;
    fy[i] = 0.f;
    fz[i] = 0.f;
    if (f64) {
        f64[3 * (size_t)i] = 0.0;
        f64[3 * (size_t)i + 1] = 0.0;
        f64[3 * (size_t)i + 2] = 0.0;
    }
}

int zero_forces(Context* c) {
    k_zero_f<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->fx, c->fy, c->fz, c->f64);
    c->launches++;
    return check_cuda(c, cudaGetLastError(), "zero forces");
}

}  // namespace omdg
