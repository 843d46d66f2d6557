// Device helpers shared by the kernels: neighbour entry encoding, the
// mixed-precision relative vector, FP32/FP64 spline reads with TableReader
// semantics and compensated accumulation.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "omdg_internal.h"

namespace omdg {

// Neighbour entry: bits 0..25 atom index, then (s+1) for x, y, z in two bits each.
__host__ __device__ __forceinline__ unsigned nbr_encode(int j, int sx, int sy, int sz) {
    return (unsigned)j | ((unsigned)(sx + 1) << 26) | ((unsigned)(sy + 1) << 28) | ((unsigned)(sz + 1) << 30);
}
__host__ __device__ __forceinline__ int nbr_index(unsigned e) { return (int)(e & (unsigned)INDEX_MASK); }
__host__ __device__ __forceinline__ int nbr_sx(unsigned e) { return (int)((e >> 26) & 3u) - 1; }
__host__ __device__ __forceinline__ int nbr_sy(unsigned e) { return (int)((e >> 28) & 3u) - 1; }
__host__ __device__ __forceinline__ int nbr_sz(unsigned e) { return (int)((e >> 30) & 3u) - 1; }
// The caller-facing image code (sx+1) + 3(sy+1) + 9(sz+1).
__host__ __device__ __forceinline__ int nbr_code(unsigned e) {
    return (nbr_sx(e) + 1) + 3 * (nbr_sy(e) + 1) + 9 * (nbr_sz(e) + 1);
}

// Sliced-ELL neighbour layout: atoms are grouped in slices of H = 2^hshift
// consecutive (cell-sorted) atoms and a slice stores its rows slot-major, so
// a warp that covers 32/H slots of H atoms reads one contiguous 128-byte line.
__host__ __device__ __forceinline__ size_t nbr_at(int i, int s, int hshift, int maxnb) {
    return ((((size_t)(i >> hshift)) * (size_t)maxnb + (size_t)s) << hshift) + (size_t)(i & ((1 << hshift) - 1));
}

// Periodic lengths split into float hi + lo parts.
struct ShiftF {
    float hx, hy, hz, lx, ly, lz;
};

__host__ inline ShiftF make_shift(const BoxGeom& b) {
    ShiftF s;
    s.hx = b.Lh[0];
    s.hy = b.Lh[1];
    s.hz = b.Lh[2];
    s.lx = b.Ll[0];
    s.ly = b.Ll[1];
    s.lz = b.Ll[2];
    return s;
}

__device__ __forceinline__ float sel_shift(int s, float v) { return s == 0 ? 0.0f : (s > 0 ? v : -v); }

// d = x_i - (x_j + s L) from the packs.  hi_i - hi_j is exact (one binade),
// and so is subtracting the hi part of the periodic length (Sterbenz, since
// |hi_i - hi_j| >= L/2 whenever s != 0 and L >= 2 Rv); the lo parts carry the
// remaining bits, so d is the FP32 rounding of the FP64 difference.
__device__ __forceinline__ float3 pair_delta(const float4& hi_i, const float4& lo_i, const float4& hi_j,
                                             const float4& lo_j, unsigned e, const ShiftF& L) {
    int sx = nbr_sx(e), sy = nbr_sy(e), sz = nbr_sz(e);
    float3 d;
    d.x = __fadd_rn(__fsub_rn(__fsub_rn(hi_i.x, hi_j.x), sel_shift(sx, L.hx)),
                    __fsub_rn(__fsub_rn(lo_i.x, lo_j.x), sel_shift(sx, L.lx)));
    d.y = __fadd_rn(__fsub_rn(__fsub_rn(hi_i.y, hi_j.y), sel_shift(sy, L.hy)),
                    __fsub_rn(__fsub_rn(lo_i.y, lo_j.y), sel_shift(sy, L.ly)));
    d.z = __fadd_rn(__fsub_rn(__fsub_rn(hi_i.z, hi_j.z), sel_shift(sz, L.hz)),
                    __fsub_rn(__fsub_rn(lo_i.z, lo_j.z), sel_shift(sz, L.lz)));
    return d;
}

__device__ __forceinline__ int pack_type(const float4& hi) { return __float_as_int(hi.w); }

// One 256-bit read-only load (a whole 32-byte sector) for a neighbour's pack
// or an interleaved pair of spline knots.  The data must not be written by
// the same kernel.
__device__ __forceinline__ void ldg256(const void* p, float4& a, float4& b) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

// Coherent 256-bit load, for kernels that also write other words of the
// same array.
__device__ __forceinline__ void ld256(const void* p, float4& a, float4& b) {
    asm volatile("ld.global.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
                 : "l"(p));
}

// Compensated (Kahan) accumulator; the intrinsics keep the compiler from
// contracting or reassociating the correction.
struct Kahan {
    float s, c;
    __device__ __forceinline__ Kahan() : s(0.f), c(0.f) {}
    __device__ __forceinline__ void add(float v) {
        float y = __fsub_rn(v, c);
        float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    __device__ __forceinline__ float value() const { return s; }
};

// Error reports with their details (the status block in omdg_internal.h):
// the first report of each kind keeps its pair or value.
__device__ __forceinline__ void report_overlap(unsigned* status, int i, int j) {
    atomicOr(status, ERR_OVERLAP);
    if (atomicCAS(status + ST_OV_I, 0xffffffffu, (unsigned)i) == 0xffffffffu) status[ST_OV_J] = (unsigned)j;
}
__device__ __forceinline__ void report_range(unsigned* status, float v, int src) {
    atomicOr(status, ERR_TABLE_RANGE);
    if (atomicCAS(status + ST_RANGE_SRC, 0xffffffffu, (unsigned)src) == 0xffffffffu)
        status[ST_RANGE_V] = __float_as_uint(v);
}

// Grid barrier for kernels whose CTAs are all resident (one CTA per SM or
// fewer): each CTA's thread 0 adds one arrival, then polls until the count
// reaches `target` or `polls` polls have passed.  Returns false (and sets
// ERR_TIMEOUT) when it gave up; the caller then leaves its loop.
__device__ __forceinline__ bool grid_barrier(unsigned* counter, unsigned target, int polls, unsigned* status) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(counter, 1u);
        int k = 0;
        for (; k < polls; k++) {
            unsigned v;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(counter) : "memory");
            if (v >= target) break;
        }
        ok = k < polls;
        if (!ok) atomicOr(status, ERR_TIMEOUT);
    }
    __syncthreads();
    return ok != 0;
}

// ------------------------------------------------------------ spline reads
// TableReader::read (treader.cpp:193-229): index by truncation, the two
// edge rules, cubic value and derivative, RMULT division.  Returns false
// (and sets the status bit) where the reference would die.
__device__ __forceinline__ bool tab_read(const DevTable& t, const float4* __restrict__ coef, float r, float rinv,
                                         float& v, float& dv, unsigned* status) {
    float rval = r - t.off;
    int x = (int)(rval * t.inv_dr);
    float dx = fmaf(-(float)x, t.dr, rval);
    if (x > t.n - 1) {
        if (t.allow_hi) {
            v = dv = t.out_hi;
            return true;
        }
        report_range(status, r, t.src);
        v = dv = 0.f;
        return false;
    }
    if (x < -1) {
        if (t.allow_lo) {
            v = dv = t.out_lo;
            return true;
        }
        report_range(status, r, t.src);
        v = dv = 0.f;
        return false;
    }
    if (x == t.n - 1) {
        dx += t.dr;
        x--;
    }
    if (x == -1) x = 0;
    float4 cf = coef[x];  // (a, b, c, d)
    v = fmaf(dx, fmaf(dx, fmaf(dx, cf.x, cf.y), cf.z), cf.w);
    dv = fmaf(dx, fmaf(3.0f * dx, cf.x, 2.0f * cf.y), cf.z);
    if (t.rmult) {
        v = v * rinv;
        dv = (dv - v) * rinv;
    }
    return true;
}

// Value only (TableReader::read(double), treader.cpp:231-264).
__device__ __forceinline__ bool tab_value(const DevTable& t, const float4* __restrict__ coef, float r, float& v,
                                          float& dv, unsigned* status) {
    float rinv = t.rmult ? 1.0f / r : 0.f;
    return tab_read(t, coef, r, rinv, v, dv, status);
}

// FP64 variant with the reference's exact operation order.
__device__ __forceinline__ bool tab_read64(const DevTable& t, double r, double& v, double& dv, unsigned* status) {
    double rval = __dsub_rn(r, t.off64);
    int x = (int)__ddiv_rn(rval, t.dr64);
    double dx = __dsub_rn(rval, __dmul_rn((double)x, t.dr64));
    if (x > t.n - 1) {
        if (t.allow_hi) {
            v = dv = t.out_hi;
            return true;
        }
        report_range(status, (float)r, t.src);
        v = dv = 0.0;
        return false;
    }
    if (x < -1) {
        if (t.allow_lo) {
            v = dv = t.out_lo;
            return true;
        }
        report_range(status, (float)r, t.src);
        v = dv = 0.0;
        return false;
    }
    if (x == t.n - 1) {
        dx = __dadd_rn(dx, t.dr64);
        x--;
    }
    if (x == -1) x = 0;
    double4_32a cf = t.coef64[x];
    v = __dadd_rn(cf.w, __dmul_rn(dx, __dadd_rn(cf.z, __dmul_rn(dx, __dadd_rn(cf.y, __dmul_rn(dx, cf.x))))));
    dv = __dadd_rn(cf.z, __dmul_rn(dx, __dadd_rn(__dmul_rn(2.0, cf.y), __dmul_rn(__dmul_rn(3.0, dx), cf.x))));
    if (t.rmult) {
        v = __ddiv_rn(v, r);
        dv = __ddiv_rn(__dsub_rn(dv, v), r);
    }
    return true;
}

// ------------------------------------------------------------------
// FP64 work on GB300 runs on a pipe about 1/64 of the FP32 one, so the
// integration and reduction kernels keep FP64 instructions for the state
// updates only.  Conversions go through the bit patterns and sums through
// FP32 pairs (hi + lo, about 44 significant bits).

// Rare cases convert through the FP64 pipe out of line: a call is never
// if-converted, so its FP64 instructions do not issue for the common case.
static __device__ __noinline__ double f2d_slow(float f) { return (double)f; }

// float -> double exactly, by the bit pattern (zero, infinities and NaN
// included); subnormal floats convert out of line.
__device__ __forceinline__ double f2d_exact(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xFFu;
    const unsigned m = u & 0x7FFFFFu;
    if (e == 0u && m != 0u) return f2d_slow(f);
    const unsigned long long de = e == 0u ? 0ull : (e == 0xFFu ? 0x7FFull : (unsigned long long)(e + 896u));
    const unsigned long long d =
        ((unsigned long long)(u & 0x80000000u) << 32) | (de << 52) | ((unsigned long long)m << 29);
    return __longlong_as_double((long long)d);
}

struct F2 {
    float hi, lo;
};

static __device__ __noinline__ F2 split_slow(double X) {
    F2 r;
    r.hi = __double2float_rn(X);
    r.lo = __double2float_rn(__dsub_rn(X, (double)r.hi));
    return r;
}

// X = hi + lo with hi = X rounded to 24 significant bits (half away from
// zero on the bit pattern) and lo = the FP32 rounding of X - hi, from the
// integer bits; zero gives zeros.  Outside 2^-60 <= |X| < 2^100 (tiny,
// huge, non-finite) the FP64 conversions decide, out of line.
__device__ __forceinline__ void split_bits(double X, float& hi, float& lo) {
    const long long b = __double_as_longlong(X);
    const long long a = b & 0x7FFFFFFFFFFFFFFFll;
    const int E = (int)(a >> 52) - 1023;
    if (a == 0) {
        hi = 0.f;
        lo = 0.f;
        return;
    }
    if (E < -60 || E >= 100) {
        const F2 r = split_slow(X);
        hi = r.hi;
        lo = r.lo;
        return;
    }
    const long long hb = (a + (1ll << 28)) & ~((1ll << 29) - 1);
    const int eh = (int)(hb >> 52) - 1023 + 127;
    const int sgn = (int)((unsigned long long)b >> 32) & (int)0x80000000;
    hi = __int_as_float(sgn | (eh << 23) | (int)((hb >> 29) & 0x7FFFFF));
    const int diff = (int)(a - hb);  // units of the last bit of |X|, |diff| <= 2^28
    const float l = __int2float_rn(diff) * __int_as_float((E - 52 + 127) << 23);
    lo = b < 0 ? -l : l;
}

__device__ __forceinline__ F2 f2_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
    const F2 s = f2_two_sum(a.hi, b.hi);
    const float t = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    const float h = __fadd_rn(s.hi, t);
    return {h, __fsub_rn(t, __fsub_rn(h, s.hi))};
}

// a * b for a, b given as pairs (the lo * lo term dropped)
__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    const float h = __fadd_rn(p, e);
    return {h, __fsub_rn(e, __fsub_rn(h, p))};
}

// The pack coordinate X = x + Q as FP32 hi + lo without FP64 arithmetic:
// x split by bits, Q given as a pair (qh, ql); TwoSum of the hi parts is
// exact, the remainder is rounded once and the pair renormalised, so
// |lo| <= ulp(hi)/2 and hi + lo is X to about 2^-47 relative.  Every pack
// writer uses this one function.
__device__ __forceinline__ void pack_coord(double x, float qh, float ql, float& hi, float& lo) {
    float xh, xl;
    split_bits(x, xh, xl);
    const F2 s = f2_two_sum(xh, qh);
    const float t = __fadd_rn(s.lo, __fadd_rn(xl, ql));
    hi = __fadd_rn(s.hi, t);
    lo = __fsub_rn(t, __fsub_rn(hi, s.hi));
}

__device__ __forceinline__ F2 f2_from(double x) {
    F2 r;
    split_bits(x, r.hi, r.lo);
    return r;
}

__device__ __forceinline__ double f2_to_double(F2 a) { return __dadd_rn(f2d_exact(a.hi), f2d_exact(a.lo)); }

__device__ __forceinline__ F2 f2_shfl_xor(F2 a, int o) {
    return {__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
}

// Caller-order transfers move blocks of IO_BLOCK atoms.  A block's rows of C
// doubles are contiguous in the caller's array, so they pass through shared
// memory with coalesced accesses on the caller's side (host memory over the
// chip-to-chip link, or the device staging buffer); the sorted side is
// gathered or scattered through the caller-to-sorted map.
constexpr int IO_BLOCK = 256;

// rows [b0, b0 + cnt) of an n x C caller array into s[0, C*cnt)
template <int C>
__device__ __forceinline__ void io_stage_in(const double* __restrict__ in, int b0, int cnt, double* s) {
    const double* src = in + (size_t)C * b0;
    for (int q = threadIdx.x; q < C * cnt; q += IO_BLOCK) s[q] = src[q];
}

// s[0, C*cnt) out to rows [b0, b0 + cnt) of an n x C caller array
template <int C>
__device__ __forceinline__ void io_stage_out(const double* s, int b0, int cnt, double* __restrict__ out) {
    double* dst = out + (size_t)C * b0;
    for (int q = threadIdx.x; q < C * cnt; q += IO_BLOCK) dst[q] = s[q];
}

}  // namespace omdg
