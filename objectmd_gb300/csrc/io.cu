// Host<->device state transfer in the caller's atom order.  The device keeps
// atoms in cell order; these kernels permute through the caller-to-sorted
// map on the GPU, so each array crosses the host link once as n rows of
// doubles, which is what an Object-MD application's host mirror of Atom
// x/v/f needs (SyncData points, gadget.h:212-213).  Pinned host arrays are
// read and written by the kernels themselves (no staging copy).
#include <algorithm>

#include "device_common.cuh"

namespace omdg {

// Sorted arrays (C components, SoA of type T) to caller-order rows: thread
// t gathers caller atom b0 + t from its sorted index.
template <int C, typename T>
__global__ void __launch_bounds__(IO_BLOCK) k_soa_to_rows(int n, const int* __restrict__ inv, const T* __restrict__ a,
                                                          const T* __restrict__ b, const T* __restrict__ c,
                                                          double* __restrict__ out) {
    __shared__ double s[C * IO_BLOCK];
    const int b0 = blockIdx.x * IO_BLOCK, cnt = min(IO_BLOCK, n - b0), t = threadIdx.x;
    if (t < cnt) {
        const int i = inv[b0 + t];
        s[C * t] = (double)a[i];
        if (C == 3) {
            s[C * t + 1] = (double)b[i];
            s[C * t + 2] = (double)c[i];
        }
    }
    __syncthreads();
    io_stage_out<C>(s, b0, cnt, out);
}

// Positions, velocities and forces to caller-order rows in one pass (any
// output may be null): a block gathers the nine values of IO_BLOCK atoms,
// then writes the three row segments; blocks stride over the chunks, so a
// small grid can run beside other kernels.  Forces are FP32 arrays, or
// FP64 interleaved.
__global__ void __launch_bounds__(IO_BLOCK) k_state_to_rows(int n, const int* __restrict__ inv,
                                                            const double* __restrict__ x, const double* __restrict__ y,
                                                            const double* __restrict__ z, const double* __restrict__ vx,
                                                            const double* __restrict__ vy,
                                                            const double* __restrict__ vz, const float* __restrict__ fx,
                                                            const float* __restrict__ fy, const float* __restrict__ fz,
                                                            const double* __restrict__ f64, double* __restrict__ ox,
                                                            double* __restrict__ ov, double* __restrict__ of) {
    __shared__ double s[3][3 * IO_BLOCK];
    const int t = threadIdx.x;
    for (int b0 = blockIdx.x * IO_BLOCK; b0 < n; b0 += gridDim.x * IO_BLOCK) {
        const int cnt = min(IO_BLOCK, n - b0);
        if (t < cnt) {
            const int i = inv[b0 + t];
            if (ox) s[0][3 * t] = x[i], s[0][3 * t + 1] = y[i], s[0][3 * t + 2] = z[i];
            if (ov) s[1][3 * t] = vx[i], s[1][3 * t + 1] = vy[i], s[1][3 * t + 2] = vz[i];
            if (of) {
                if (f64) {
                    const double* r = f64 + 3 * (size_t)i;
                    s[2][3 * t] = r[0], s[2][3 * t + 1] = r[1], s[2][3 * t + 2] = r[2];
                } else {
                    s[2][3 * t] = fx[i], s[2][3 * t + 1] = fy[i], s[2][3 * t + 2] = fz[i];
                }
            }
        }
        __syncthreads();
        if (ox) io_stage_out<3>(s[0], b0, cnt, ox);
        if (ov) io_stage_out<3>(s[1], b0, cnt, ov);
        if (of) io_stage_out<3>(s[2], b0, cnt, of);
        __syncthreads();  // the next chunk reuses the staging
    }
}

// Caller-order force rows to the sorted FP32 arrays (and the FP64 forces,
// three interleaved per atom, when the context keeps them)
__global__ void __launch_bounds__(IO_BLOCK) k_rows_to_forces(int n, const int* __restrict__ inv,
                                                             const double* __restrict__ in, float* __restrict__ fx,
                                                             float* __restrict__ fy, float* __restrict__ fz,
                                                             double* __restrict__ f64) {
    __shared__ double s[3 * IO_BLOCK];
    const int b0 = blockIdx.x * IO_BLOCK, cnt = min(IO_BLOCK, n - b0), t = threadIdx.x;
    io_stage_in<3>(in, b0, cnt, s);
    __syncthreads();
    if (t < cnt) {
        const int i = inv[b0 + t];
        fx[i] = (float)s[3 * t];
        fy[i] = (float)s[3 * t + 1];
        fz[i] = (float)s[3 * t + 2];
        if (f64) {
            f64[3 * (size_t)i] = s[3 * t];
            f64[3 * (size_t)i + 1] = s[3 * t + 1];
            f64[3 * (size_t)i + 2] = s[3 * t + 2];
        }
    }
}

// Staging layout (doubles): x [0,3n) v [3n,6n) f [6n,9n) pot [9n,10n) vir [10n,11n).
static int ensure_io(Context* c) {
    size_t need = (size_t)11 * c->cap;
    if (c->d_io && c->io_cap >= need) return OMDG_OK;
    cudaFree(c->d_io);
    c->d_io = nullptr;
    if (cudaMalloc(&c->d_io, sizeof(double) * need) != cudaSuccess) return set_error(c, OMDG_ENOMEM, "io staging");
    c->io_cap = need;
    return OMDG_OK;
}

// p (count doubles) when kernels can read and write it at its own address:
// pinned or registered host memory, both ends inside registered ranges, on
// a device that addresses registered memory by its host pointer.  Else null
// (pageable memory takes a copy through the staging buffer).
const double* host_view(Context* c, const double* p, size_t count) {
    if (!p || count == 0) return nullptr;
    if (c->host_ptr_ok < 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrCanUseHostPointerForRegisteredMem, c->device) != cudaSuccess) {
            cudaGetLastError();
            v = 0;
        }
        c->host_ptr_ok = v ? 1 : 0;
    }
    if (!c->host_ptr_ok) return nullptr;
    for (const double* q : {p, p + count - 1}) {
        cudaPointerAttributes a;
        if (cudaPointerGetAttributes(&a, q) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        if (a.type != cudaMemoryTypeHost || a.devicePointer != static_cast<const void*>(q)) return nullptr;
    }
    return p;
}

// Per requested array one kernel, writing the caller's rows in place when
// its memory is addressable, else into the staging buffer and one copy;
// the caller synchronizes.
int io_get_state(Context* c, double* x, double* v, double* f, double* pot, double* vir) {
    int rc = ensure_io(c);
    if (rc) return rc;
    const int n = c->n, g = (n + IO_BLOCK - 1) / IO_BLOCK;
    cudaStream_t s = c->stream;
    const size_t n3 = 3 * (size_t)n;
    // destination of one array: the caller's memory or its staging slot
    auto dest = [&](double* h, size_t count, double* stage) { return host_view(c, h, count) ? h : stage; };
    auto finish = [&](double* h, double* d, size_t count) {
        if (d != h) cudaMemcpyAsync(h, d, sizeof(double) * count, cudaMemcpyDeviceToHost, s);
    };
    double* st = c->d_io;
    if (x || v || f) {
        double* dx = x ? dest(x, n3, st) : nullptr;
        double* dv = v ? dest(v, n3, st + n3) : nullptr;
        double* df = f ? dest(f, n3, st + 2 * n3) : nullptr;
        k_state_to_rows<<<g, IO_BLOCK, 0, s>>>(n, c->inv, c->x, c->y, c->z, c->vx, c->vy, c->vz, c->fx, c->fy, c->fz,
                                               c->use_f64 ? c->f64 : nullptr, dx, dv, df);
        if (x) finish(x, dx, n3);
        if (v) finish(v, dv, n3);
        if (f) finish(f, df, n3);
    }
    if (pot) {
        double* d = dest(pot, n, st + 3 * n3);
        if (c->use_f64)
            k_soa_to_rows<1, double><<<g, IO_BLOCK, 0, s>>>(n, c->inv, c->f64 + n3, nullptr, nullptr, d);
        else k_soa_to_rows<1, float><<<g, IO_BLOCK, 0, s>>>(n, c->inv, c->pe, nullptr, nullptr, d);
        finish(pot, d, n);
    }
    if (vir) {
        double* d = dest(vir, n, st + 3 * n3 + n);
        k_soa_to_rows<1, float><<<g, IO_BLOCK, 0, s>>>(n, c->inv, c->vir, nullptr, nullptr, d);
        finish(vir, d, n);
    }
    return check_cuda(c, cudaGetLastError(), "state read-back");
}

// Positions, velocities and/or forces written by one kernel on stream s
// straight into the caller's pinned host arrays (every non-null pointer
// must pass host_view); the step graph's download branches use it.
int io_rows_to_host(Context* c, cudaStream_t s, double* x, double* v, double* f) {
    const int n = c->n;
    // a bounded grid: the link, not the SMs, sets the pace, and the force
    // and kick kernels running beside it keep the rest of the GPU
    const int g = std::min((n + IO_BLOCK - 1) / IO_BLOCK, c->io_blocks);
    k_state_to_rows<<<g, IO_BLOCK, 0, s>>>(n, c->inv, c->x, c->y, c->z, c->vx, c->vy, c->vz, c->fx, c->fy, c->fz,
                                           c->use_f64 ? c->f64 : nullptr, x, v, f);
    return check_cuda(c, cudaGetLastError(), "state download");
}

// Upload positions and/or velocities given in caller order (positions also
// refresh the pack and the displacement check).
int io_set_state(Context* c, const double* x, const double* v) {
    int rc = ensure_io(c);
    if (rc) return rc;
    cudaStream_t s = c->stream;
    const size_t n3 = 3 * (size_t)c->n;
    // source of one array: the caller's memory or its staging slot
    auto source = [&](const double* h, double* stage) -> const double* {
        if (!h) return nullptr;
        if (host_view(c, h, n3)) return h;
        cudaMemcpyAsync(stage, h, sizeof(double) * n3, cudaMemcpyHostToDevice, s);
        return stage;
    };
    const double* sx = source(x, c->d_io);
    const double* sv = source(v, c->d_io + n3);
    if (!sx && !sv) return OMDG_OK;
    return upload_state(c, sx, sv);
}

__global__ void k_flags_from_caller(int n, const int* __restrict__ id, const unsigned* __restrict__ in,
                                    unsigned keep, unsigned* __restrict__ flag) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    flag[k] = (flag[k] & keep) | (in[id[k]] & ~keep);
}

__global__ void k_flags_to_caller(int n, const int* __restrict__ id, const unsigned* __restrict__ flag,
                                  unsigned* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    out[id[k]] = flag[k];
}

// Per-atom flag words in caller order; bits in keep_mask keep their device
// values.  Synchronous (the staging is a temporary device buffer).
int io_set_flags(Context* c, const unsigned* flags, unsigned keep_mask) {
    unsigned* d = nullptr;
    const int n = c->n;
    if (cudaMalloc(&d, sizeof(unsigned) * n) != cudaSuccess) return set_error(c, OMDG_ENOMEM, "flag staging");
    cudaMemcpyAsync(d, flags, sizeof(unsigned) * n, cudaMemcpyHostToDevice, c->stream);
    k_flags_from_caller<<<grid_for(n, 256), 256, 0, c->stream>>>(n, c->id, d, keep_mask, c->aflag);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    cudaFree(d);
    return check_cuda(c, e == cudaSuccess ? cudaGetLastError() : e, "flag upload");
}

int io_get_flags(Context* c, unsigned* flags) {
    unsigned* d = nullptr;
    const int n = c->n;
    if (cudaMalloc(&d, sizeof(unsigned) * n) != cudaSuccess) return set_error(c, OMDG_ENOMEM, "flag staging");
    k_flags_to_caller<<<grid_for(n, 256), 256, 0, c->stream>>>(n, c->id, c->aflag, d);
    cudaMemcpyAsync(flags, d, sizeof(unsigned) * n, cudaMemcpyDeviceToHost, c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    cudaFree(d);
    return check_cuda(c, e == cudaSuccess ? cudaGetLastError() : e, "flag read-back");
}

// Upload forces given in caller order (n*3 FP64; the FP32 arrays get their
// rounding, the FP64 block of the FP64 pair mode the values themselves).
int io_set_forces(Context* c, const double* f) {
    int rc = ensure_io(c);
    if (rc) return rc;
    const int n = c->n;
    cudaStream_t s = c->stream;
    const size_t n3 = 3 * (size_t)n;
    cudaMemcpyAsync(c->d_io + 2 * n3, f, sizeof(double) * n3, cudaMemcpyHostToDevice, s);
    k_rows_to_forces<<<(n + IO_BLOCK - 1) / IO_BLOCK, IO_BLOCK, 0, s>>>(n, c->inv, c->d_io + 2 * n3, c->fx, c->fy,
                                                                       c->fz, c->use_f64 ? c->f64 : nullptr);
    return check_cuda(c, cudaGetLastError(), "force upload");
}

}  // namespace omdg
