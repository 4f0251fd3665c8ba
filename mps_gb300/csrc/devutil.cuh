// Device helpers shared by the kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "engine.cuh"
#include "exact64.cuh"

namespace mpsg {

// FP64 operations that are never contracted into a fused multiply-add, so
// that every rounding matches the reference's (x86 builds of it have no FMA).
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// The FP32 starting points of the integer-pipe square root and division:
// the hardware approximations (2 ulp each, documented).
struct Fp32Approx {
    static __host__ __device__ __forceinline__ float rsqrt(float x) {
#ifdef __CUDA_ARCH__
        return rsqrtf(x);
#else
        return 1.0f / sqrtf(x);
#endif
    }
    static __host__ __device__ __forceinline__ float rcp(float x) {
#ifdef __CUDA_ARCH__
        return __fdividef(1.0f, x);
#else
        return 1.0f / x;
#endif
    }
};

// The FP64 instructions for the operands outside the integer paths below.
// They are separate functions so that the compiler branches to them instead
// of issuing them, predicated off, on every call.
static __device__ __noinline__ double ddiv_fp64(double a, double b) { return __ddiv_rn(a, b); }
static __device__ __noinline__ double dsqrt_fp64(double a) { return __dsqrt_rn(a); }
static __device__ __noinline__ double dsub_fp64(double a, double b) { return __dsub_rn(a, b); }
static __device__ __noinline__ float f32_fp64(double x) { return __double2float_rn(x); }

// Correctly rounded FP64 division and square root.  Normal operands with a
// normal result (all of the sweeps' distances and weights) are computed on
// the integer and FP32 pipes (exact64.cuh), the rest by the FP64 instruction
// sequence; both give the IEEE round-to-nearest result.
__device__ __forceinline__ double ddiv(double a, double b) {
    double q;
    if (x64::div_rn<Fp32Approx>(a, b, q)) return q;
    return ddiv_fp64(a, b);
}
__device__ __forceinline__ double dsqrt(double a) {
    double r;
    if (x64::sqrt_rn<Fp32Approx>(a, r)) return r;
    return dsqrt_fp64(a);
}

// FP32 rounding of a double (nearest, ties to even) without the conversion
// instruction, which runs on the FP64 pipe: the same value as (float)x.
__device__ __forceinline__ float f32(double x) {
    float f;
    if (x64::to_f32(x, f)) return f;
    return f32_fp64(x);
}

// v < cut for a cut > 0 and a v that is >= 0 or NaN (squared distances and
// distances), on the integer pipe: the same result as the FP64 comparison.
__device__ __forceinline__ bool lt_cut(double v, double cut) { return x64::lt_cut(v, cut); }

// weight(): src/mps.cpp:9-16.  re / dist >= 1 when dist < re, so the
// subtraction of 1 is exact and done on the integer pipe (the FP64 one only
// for re / dist >= 2^53).
__device__ __forceinline__ double weight(double dist, double re) {
    if (!lt_cut(dist, re)) return 0.0;
    const double q = ddiv(re, dist);
    double w;
    if (x64::sub_one(q, w)) return w;
    return dsub_fp64(q, 1.0);
}

// Cell coordinate int((x - lo) / len) + 1 (src/bucket.cpp:40-42,
// src/mps.cpp:595-597), clamped to [1, cells - 2] where the reference
// would index outside its padded grid.
__device__ __forceinline__ int cell_coord(double x, double lo, double len, int cells) {
    double q = ddiv(dsub(x, lo), len);
    if (!(q >= 0.0)) return 1;
    if (q >= (double)(cells - 2)) return cells - 2;
    return (int)q + 1;
}

__device__ __forceinline__ int32_t cell_key(const Consts& c, double x, double y, double z) {
    int ix = cell_coord(x, c.dmin[0], c.len, c.numX);
    int iy = cell_coord(y, c.dmin[1], c.len, c.numY);
    if (c.planar) return ix * c.numY + iy;
    int iz = cell_coord(z, c.dmin[2], c.len, c.numZ);
    return (ix * c.numY + iy) * c.numZ + iz;
}

// Visits the candidate slots of the 3x3(x3) cells around `key` in the
// reference's order: jx outer, jy, jz inner (src/mps.cpp:599-601), and
// ascending id inside a cell.  Keys are x-major, so the cells of one jx
// column (planar) or one (jx, jy) row (3-D) form one contiguous slot range.
template <bool PLANAR, class F>
__device__ __forceinline__ void for_each_candidate(const Consts& c, const int32_t* __restrict__ cs,
                                                   int32_t key, F&& f) {
    if (PLANAR) {
        int ix = key / c.numY;
        int iy = key - ix * c.numY;
#pragma unroll 1
        for (int jx = ix - 1; jx <= ix + 1; jx++) {
            int kk = jx * c.numY + iy - 1;
            int b = __ldg(cs + kk), e = __ldg(cs + kk + 3);
#pragma unroll 1
            for (int j = b; j < e; j++) f(j);
        }
    } else {
        int iz = key % c.numZ;
        int t = key / c.numZ;
        int iy = t % c.numY;
        int ix = t / c.numY;
#pragma unroll 1
        for (int jx = ix - 1; jx <= ix + 1; jx++)
#pragma unroll 1
            for (int jy = iy - 1; jy <= iy + 1; jy++) {
                int kk = (jx * c.numY + jy) * c.numZ + iz - 1;
                int b = __ldg(cs + kk), e = __ldg(cs + kk + 3);
#pragma unroll 1
                for (int j = b; j < e; j++) f(j);
            }
    }
}

// Exact squared distance in the reference's order, (dx^2 + dy^2) + dz^2.
template <bool PLANAR>
__device__ __forceinline__ double dist2(const StateBuf& s, int i, int j, double xi, double yi,
                                        double zi) {
    double dx = dsub(s.x[j], xi), dy = dsub(s.y[j], yi);
    double r = dadd(dmul(dx, dx), dmul(dy, dy));
    if (!PLANAR) {
        double dz = dsub(s.z[j], zi);
        r = dadd(r, dmul(dz, dz));
    }
    return r;
}

// FP32 pre-filter: true if candidate j is certainly farther from (fx, fy,
// fz) than the radius whose FP32 bound is `bound` (see Consts::ft_max).
template <bool PLANAR>
__device__ __forceinline__ bool far32(const StateBuf& s, int j, float fx, float fy, float fz,
                                      float bound) {
    const float2 q = s.xyf[j];
    const float dx = q.x - fx, dy = q.y - fy;
    float r = dx * dx + dy * dy;
    if (!PLANAR) {
        const float dz = s.zf[j] - fz;
        r += dz * dz;
    }
    return r > bound;
}

// Symmetry fingerprint of a matrix (the test of solvePoissonEquation,
// src/mps.cpp:418-442): the term of stored off-diagonal entry (ri, ci) with
// value v is sgn(ci - ri) H(min, max) bits(v) mod 2^64, H an odd 64-bit
// hash of the unordered pair (the SplitMix64 finaliser of Steele, Lea and
// Flood, 2014) and bits() the IEEE pattern (zeros canonical).  Integer sums
// of these are exact and order-free: 0 for a bitwise symmetric matrix, and
// not 0 for any other with probability 1 - 2^-64.
__host__ __device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ unsigned long long entry_term(int ri, int ci, double v) {
    const unsigned lo = (unsigned)min(ri, ci), hi = (unsigned)max(ri, ci);
    const unsigned long long h = mix64(((unsigned long long)lo << 32) | hi) | 1ull;
    const unsigned long long b = v == 0.0 ? 0ull : (unsigned long long)__double_as_longlong(v);
    const unsigned long long t = h * b;
    return ri < ci ? t : 0ull - t;
}

__device__ __forceinline__ unsigned long long warp_sum64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ void atomic_max_nonneg_double(unsigned long long* a, double v) {
    atomicMax(a, (unsigned long long)__double_as_longlong(v));
}

}  // namespace mpsg
