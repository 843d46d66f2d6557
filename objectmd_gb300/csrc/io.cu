// Host<->device state transfer in the caller's atom order.  The device keeps
// atoms in cell order; these kernels permute through the id/inv maps on the
// GPU so a transfer is one contiguous copy of n*3 doubles per array, which
// is what an Object-MD application's host mirror of Atom x/v/f needs
// (SyncData points, gadget.h:212-213).
#include "device_common.cuh"

namespace omdg {

__global__ void k_to_caller3(int n, const int* __restrict__ id, const double* __restrict__ a,
                             const double* __restrict__ b, const double* __restrict__ c, double* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    size_t o = 3 * (size_t)id[k];
    out[o] = a[k];
    out[o + 1] = b[k];
    out[o + 2] = c[k];
}

__global__ void k_to_caller3f(int n, const int* __restrict__ id, const float* __restrict__ a,
                              const float* __restrict__ b, const float* __restrict__ c, double* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    size_t o = 3 * (size_t)id[k];
    out[o] = a[k];
    out[o + 1] = b[k];
    out[o + 2] = c[k];
}

__global__ void k_to_caller3d(int n, const int* __restrict__ id, const double* __restrict__ f64,
                              double* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    size_t o = 3 * (size_t)id[k];
    out[o] = f64[3 * (size_t)k];
    out[o + 1] = f64[3 * (size_t)k + 1];
    out[o + 2] = f64[3 * (size_t)k + 2];
}

__global__ void k_to_caller1f(int n, const int* __restrict__ id, const float* __restrict__ a,
                              double* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    out[id[k]] = a[k];
}

__global__ void k_to_caller1d(int n, const int* __restrict__ id, const double* __restrict__ a,
                              double* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    out[id[k]] = a[k];
}

__global__ void k_from_caller3(int n, const int* __restrict__ id, const double* __restrict__ in,
                               double* __restrict__ a, double* __restrict__ b, double* __restrict__ c) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    size_t o = 3 * (size_t)id[k];
    a[k] = in[o];
    b[k] = in[o + 1];
    c[k] = in[o + 2];
}

__global__ void k_from_caller3f(int n, const int* __restrict__ id, const double* __restrict__ in,
                                float* __restrict__ a, float* __restrict__ b, float* __restrict__ c,
                                double* __restrict__ f64) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    size_t o = 3 * (size_t)id[k];
    a[k] = (float)in[o];
    b[k] = (float)in[o + 1];
    c[k] = (float)in[o + 2];
    if (f64) {
        f64[3 * (size_t)k] = in[o];
        f64[3 * (size_t)k + 1] = in[o + 1];
        f64[3 * (size_t)k + 2] = in[o + 2];
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

// One contiguous async copy per requested array; the caller synchronizes.
int io_get_state(Context* c, double* x, double* v, double* f, double* pot, double* vir) {
    int rc = ensure_io(c);
    if (rc) return rc;
    int n = c->n, g = grid_for(n, 256);
    cudaStream_t s = c->stream;
    double* st = c->d_io;
    size_t n3 = 3 * (size_t)n;
    if (x) {
        k_to_caller3<<<g, 256, 0, s>>>(n, c->id, c->x, c->y, c->z, st);
        cudaMemcpyAsync(x, st, sizeof(double) * n3, cudaMemcpyDeviceToHost, s);
    }
    if (v) {
        k_to_caller3<<<g, 256, 0, s>>>(n, c->id, c->vx, c->vy, c->vz, st + n3);
        cudaMemcpyAsync(v, st + n3, sizeof(double) * n3, cudaMemcpyDeviceToHost, s);
    }
    if (f) {
        if (c->use_f64) k_to_caller3d<<<g, 256, 0, s>>>(n, c->id, c->f64, st + 2 * n3);
        else k_to_caller3f<<<g, 256, 0, s>>>(n, c->id, c->fx, c->fy, c->fz, st + 2 * n3);
        cudaMemcpyAsync(f, st + 2 * n3, sizeof(double) * n3, cudaMemcpyDeviceToHost, s);
    }
    if (pot) {
        if (c->use_f64) k_to_caller1d<<<g, 256, 0, s>>>(n, c->id, c->f64 + n3, st + 3 * n3);
        else k_to_caller1f<<<g, 256, 0, s>>>(n, c->id, c->pe, st + 3 * n3);
        cudaMemcpyAsync(pot, st + 3 * n3, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
    }
    if (vir) {
        k_to_caller1f<<<g, 256, 0, s>>>(n, c->id, c->vir, st + 3 * n3 + n);
        cudaMemcpyAsync(vir, st + 3 * n3 + n, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
    }
    return check_cuda(c, cudaGetLastError(), "state read-back");
}

// Upload positions and/or velocities given in caller order.
int io_set_state(Context* c, const double* x, const double* v) {
    int rc = ensure_io(c);
    if (rc) return rc;
    int n = c->n, g = grid_for(n, 256);
    cudaStream_t s = c->stream;
    size_t n3 = 3 * (size_t)n;
    if (x) {
        cudaMemcpyAsync(c->d_io, x, sizeof(double) * n3, cudaMemcpyHostToDevice, s);
        k_from_caller3<<<g, 256, 0, s>>>(n, c->id, c->d_io, c->x, c->y, c->z);
    }
    if (v) {
        cudaMemcpyAsync(c->d_io + n3, v, sizeof(double) * n3, cudaMemcpyHostToDevice, s);
        k_from_caller3<<<g, 256, 0, s>>>(n, c->id, c->d_io + n3, c->vx, c->vy, c->vz);
    }
    return check_cuda(c, cudaGetLastError(), "state upload");
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
    int n = c->n, g = grid_for(n, 256);
    cudaStream_t s = c->stream;
    const size_t n3 = 3 * (size_t)n;
    cudaMemcpyAsync(c->d_io + 2 * n3, f, sizeof(double) * n3, cudaMemcpyHostToDevice, s);
    k_from_caller3f<<<g, 256, 0, s>>>(n, c->id, c->d_io + 2 * n3, c->fx, c->fy, c->fz, c->use_f64 ? c->f64 : nullptr);
    return check_cuda(c, cudaGetLastError(), "force upload");
}

}  // namespace omdg
