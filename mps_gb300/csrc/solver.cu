// Pressure Poisson solve (src/mps.cpp:417-470).
//
// Both solvers are persistent cooperative kernels: one launch per solve, the
// blocks stay resident and meet at grid barriers between the phases of an
// iteration, and the convergence test runs on the device.  A dot product is
// reduced per block, written as one partial per block, and summed in a fixed
// order by the last block to reach the barrier, which publishes the total
// before it releases the others; results are therefore run-to-run
// deterministic and every block takes the same branch.
//
//  * FP64 (k_cg64): the Jacobi-preconditioned CG that Eigen's
//    ConjugateGradient runs with its defaults (zero start, stop when
//    ||r||^2 < max(tol^2 ||b||^2, DBL_MIN) on the recursive residual, cap 2n),
//    over the SELL-32 FP64 matrix; three phases per iteration as Eigen's loop
//    is written.  Roofline: HBM (12 B per stored entry and iteration) and FP64
//    issue (one DFMA per entry).
//  * MIXED (k_cg_mixed): iterative refinement.  x and the residual
//    r = b - A x stay FP64 (FP64 matrix); each correction A d = r is solved
//    by Jacobi CG in the Chronopoulos-Gear arrangement (one fused reduction
//    and two barriers per iteration) on an FP32 form of the operator with
//    FP32 vectors and FP64-accurate dot products (error-free FP32 products
//    accumulated with compensation per thread, FP64 across threads and
//    blocks).  On planar scenes the FP32 matrix is stored with one index
//    byte per entry (range of the neighbour sweep + offset), 5 B per entry.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <utility>
#include <vector>

#include "devutil.cuh"
#include "engine.cuh"

namespace mpsg {

namespace {

// Single-scene solves: one 1024-thread block per SM, 152 blocks meet at
// each grid barrier.  Batched solves (many scenes in one launch) run the same
// code on groups of blocks, each group with its own barrier and partials.
constexpr int kBlock = 1024;
constexpr int kMixedBlock = 1024;  // k_cg_mixed: one block per SM
// Polls before a barrier wait gives up: one poll (an acquire load plus the
// back-off) takes ~0.28 us on GB300 (measured by mps_selftest_wait_limit),
// so ~2.4 s, far above any legitimate wait (tens of microseconds).
constexpr long long kSpinLimit = 1ll << 23;

struct SolveArgs {
    int32_t n;          // rows (slots)
    int32_t nslices;
    int32_t K;
    double tol;
    int64_t max_iter;
    double inner_tol;
    int32_t max_refine;
    int32_t warm;       // x holds an initial guess (else the solve zeroes it)
};

// ---------------------------------------------------------------- barriers
// Grid barrier on one monotonically increasing arrival counter: block b's
// e-th barrier adds 1 (a release reduction, no reply) and waits until the
// counter reaches e * (blocks in the group).  No block resets anything, so there is no
// reset race, and the arrivals do not serialise on returning atomics.  The
// wait is bounded: the blocks of a cooperative launch are co-resident, so it
// always completes; if it somehow does not, the block raises ST_TIMEOUT and
// every block leaves at its next barrier.
struct GridBar {
    unsigned int* count;
    unsigned int epoch;  // barriers passed by this block (same in every block)
    int parity;          // which half of the partials buffer the next reduction uses
    int rank;            // this block's index within its group
    int size;            // blocks in the group (the whole grid for a single scene)
    double* partials;    // 2 x size x 8 per-block partial sums of the group
    long long spin_limit = kSpinLimit;  // polls before a barrier wait gives up
};

__device__ __forceinline__ GridBar whole_grid(const Krylov& kv) {
    return GridBar{kv.barrier, 0u, 0, (int)blockIdx.x, (int)gridDim.x, kv.partials};
}

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void red_release_add(unsigned int* p, unsigned int v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Block-level barrier of a thread group: NT = 0 is the whole block
// (__syncthreads), else the block's first NT threads (named barrier 1, NT a
// multiple of 32); the rest of the block runs on meanwhile.
template <int NT>
__device__ __forceinline__ void group_bar() {
    if constexpr (NT == 0)
        __syncthreads();
    else
        asm volatile("bar.sync 1, %0;" ::"n"(NT) : "memory");
}

// A grid barrier passed by a thread group of every block (NT as above):
// thread 0 arrives for the block.  Only thread 0's epoch and warp 0's partials
// parity matter, and thread 0 belongs to every group.
template <int NT = 0>
__device__ __forceinline__ bool grid_sync(GridBar& gb, DevStats* ds) {
    __shared__ int s_ok;
    group_bar<NT>();
    gb.epoch++;
    if (threadIdx.x == 0) {
        const unsigned int target = gb.epoch * (unsigned int)gb.size;
        red_release_add(gb.count, 1u);
        bool ok = true;
        long long it = 0;
        // Passing needs every block's arrival, so a block that gave up never
        // lets the others past the next barrier: they learn of it here, on
        // the slow path, from the status flag (no extra load when passing).
        while ((int)(ld_acquire(gb.count) - target) < 0) {
            if (++it > 256) {
                __nanosleep(16);
                if ((it & 1023) == 0 && (*(volatile int*)&ds->status & ST_TIMEOUT)) {
                    ok = false;
                    break;
                }
                if (it > gb.spin_limit) {
                    atomicOr(&ds->status, ST_TIMEOUT);
                    ok = false;
                    break;
                }
            }
        }
        s_ok = ok;
    }
    group_bar<NT>();
    return s_ok != 0;
}

// Barrier that also sums M per-thread doubles over the whole grid: each
// block reduces its threads through shared memory (one warp, fixed order),
// publishes one partial, and after the barrier every block sums the partials
// in block order, so all blocks hold bitwise the same totals.  Partials are
// double-buffered so that a fast block's next reduction never overwrites
// values a slow block is still reading.
// The two halves of that: publish_partials reduces the block's M values
// and writes its partials into the next buffer (returned); sum_partials,
// after a grid barrier that every block passed after publishing, sums the
// partials in block order.  Between the two any number of phases and
// barriers may run (the pipelined solve overlaps its reduction with the
// preconditioner that way).
template <int M, int BS>
__device__ __forceinline__ const double* publish_partials(GridBar& gb, const double (&v)[M]) {
    constexpr int kW = BS / 32;
    __shared__ double sh[M][BS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double* part = gb.partials + (size_t)gb.parity * gb.size * 8;
    gb.parity ^= 1;
#pragma unroll
    for (int m = 0; m < M; m++) sh[m][threadIdx.x] = v[m];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int m = 0; m < M; m++) {
            double a = 0.0;
#pragma unroll 8
            for (int t = 0; t < kW; t++) a += sh[m][lane + 32 * t];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
            if (lane == 0) part[gb.rank * 8 + m] = a;
        }
    }
    return part;
}

template <int M>
__device__ __forceinline__ void sum_partials(const GridBar& gb, const double* part, double (&tot)[M]) {
    __shared__ double s_tot[M];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp == 0) {
#pragma unroll
        for (int m = 0; m < M; m++) {
            double a = 0.0;
            for (int b = lane; b < gb.size; b += 32) a += __ldcg(part + b * 8 + m);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
            if (lane == 0) s_tot[m] = a;
        }
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < M; m++) tot[m] = s_tot[m];
}

template <int M, int BS>
__device__ __forceinline__ bool reduce_sync(GridBar& gb, const double (&v)[M], double (&tot)[M],
                                            DevStats* ds) {
    const double* part = publish_partials<M, BS>(gb, v);
    if (!grid_sync(gb, ds)) return false;
    sum_partials<M>(gb, part, tot);
    return true;
}

// Double-float (hi + lo, FP32 pair) sums: the per-iteration dot products of
// the mixed solver are reduced with FP32 instructions only.  This part issues
// FP64 at 1/64 of the FP32 rate (one FP64 warp instruction holds its SM
// quarter's FP64 unit for ~80 cycles), so the ~120 dependent FP64 additions
// of a block-and-grid reduction in FP64 cost ~7 us per iteration on the
// critical path; the pair sums keep ~44 bits, far more than an FP32 Krylov
// iteration needs.
struct F2 {
    float hi, lo;
};

// Knuth's two-sum of the high parts, low parts added, renormalised.
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
    const float s = a.hi + b.hi;
    const float bb = s - a.hi;
    const float err = (a.hi - (s - bb)) + (b.hi - bb);
    const float lo = (a.lo + b.lo) + err;
    const float hi = s + lo;
    return F2{hi, lo - (hi - s)};
}

__device__ __forceinline__ F2 f2_shfl_down(F2 v, int o) {
    return F2{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
}

// As publish_partials / sum_partials, on pairs: every warp reduces its lanes
// by a shuffle tree, warp 0 the warps' results, and each block's M pairs go
// to the partials buffer; after the barrier every block sums the partials in
// the same order (bitwise the same totals everywhere) and rounds each total
// to FP32.
template <int M, int BS>
__device__ __forceinline__ const F2* publish_partials_f2(GridBar& gb, const F2 (&v)[M]) {
    constexpr int kW = BS / 32;
    static_assert(kW <= 32 && M <= 8, "one warp reduces the warps' pairs");
    __shared__ F2 sh[M][kW];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    F2* part = reinterpret_cast<F2*>(gb.partials + (size_t)gb.parity * gb.size * 8);
    gb.parity ^= 1;
#pragma unroll
    for (int m = 0; m < M; m++) {
        F2 a = v[m];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a = f2_add(a, f2_shfl_down(a, o));
        if (lane == 0) sh[m][warp] = a;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int m = 0; m < M; m++) {
            F2 a = lane < kW ? sh[m][lane] : F2{0.f, 0.f};
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a = f2_add(a, f2_shfl_down(a, o));
            if (lane == 0) part[gb.rank * 8 + m] = a;
        }
    }
    return part;
}

template <int M>
__device__ __forceinline__ void sum_partials_f2(const GridBar& gb, const F2* part, float (&tot)[M]) {
    __shared__ float s_tot[M];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp == 0) {
        // each lane sums blocks lane, lane + 32, ... in that order; the loads
        // of five of them for every m are issued before any is used
        F2 a[M];
#pragma unroll
        for (int m = 0; m < M; m++) a[m] = F2{0.f, 0.f};
        for (int b0 = lane; b0 < gb.size; b0 += 32 * 5) {
            float2 q[M][5];
#pragma unroll
            for (int u = 0; u < 5; u++) {
                const int b = b0 + 32 * u;
#pragma unroll
                for (int m = 0; m < M; m++)
                    q[m][u] = b < gb.size ? __ldcg(reinterpret_cast<const float2*>(part + b * 8 + m))
                                          : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < 5; u++)
#pragma unroll
                for (int m = 0; m < M; m++)
                    if (b0 + 32 * u < gb.size) a[m] = f2_add(a[m], F2{q[m][u].x, q[m][u].y});
        }
#pragma unroll
        for (int m = 0; m < M; m++) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a[m] = f2_add(a[m], f2_shfl_down(a[m], o));
            if (lane == 0) s_tot[m] = a[m].hi + a[m].lo;
        }
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < M; m++) tot[m] = s_tot[m];
}

template <int M, int BS>
__device__ __forceinline__ bool reduce_sync_f2(GridBar& gb, const F2 (&v)[M], float (&tot)[M],
                                               DevStats* ds) {
    const F2* part = publish_partials_f2<M, BS>(gb, v);
    if (!grid_sync(gb, ds)) return false;
    sum_partials_f2<M>(gb, part, tot);
    return true;
}

// ------------------------------------------------------------------ SpMV
// y_i = sum over the SELL-32 row (padding entries are (i, 0)) + diag_i x_i,
// loads batched four at a time so that gathers overlap.
__device__ __forceinline__ double spmv64_row(const Ppe& A, int K, int sl, int lane, int row,
                                             const double* __restrict__ x, double xi) {
    const int w = __ldg(A.slice_w + sl);
    const int32_t* cp = A.col + (size_t)sl * K * 32 + lane;
    const double* vp = A.val + (size_t)sl * K * 32 + lane;
    double s0 = 0.0, s1 = 0.0;
    int m = 0;
    for (; m + 4 <= w; m += 4) {
        int c0 = __ldg(cp + (m + 0) * 32), c1 = __ldg(cp + (m + 1) * 32);
        int c2 = __ldg(cp + (m + 2) * 32), c3 = __ldg(cp + (m + 3) * 32);
        double v0 = __ldg(vp + (m + 0) * 32), v1 = __ldg(vp + (m + 1) * 32);
        double v2 = __ldg(vp + (m + 2) * 32), v3 = __ldg(vp + (m + 3) * 32);
        double x0 = __ldcg(x + c0), x1 = __ldcg(x + c1), x2 = __ldcg(x + c2), x3 = __ldcg(x + c3);
        s0 = fma(v0, x0, s0);
        s1 = fma(v1, x1, s1);
        s0 = fma(v2, x2, s0);
        s1 = fma(v3, x3, s1);
    }
    for (; m < w; m++) s0 = fma(__ldg(vp + m * 32), __ldcg(x + __ldg(cp + m * 32)), s0);
    return fma(A.diag[row], xi, s0 + s1);
}

// The FP32 operator rows below return the off-diagonal part in difference
// form, sum_j a_ij (u_j - u_i), given the row's own value u_i; the caller
// adds rsum32_i u_i (the row sum times u_i).  For a smooth u the differences
// are small and exact to within their own rounding, so the product does not
// lose the row's small sum to cancellation, and the FP32 rounding of the
// entries no longer shifts the row sum (the operator's smooth modes).
// Padding entries (value 0) add 0.

// FP32 SELL row (rows without a compact form): int32 columns of the FP64
// matrix, FP32 values in the quad layout.
__device__ __forceinline__ float spmv32_sell_row(const Ppe& A, int K, int row,
                                                 const float* __restrict__ u, float ui) {
    const int sl = row >> 5, lane = row & 31;
    const int w = __ldg(A.slice_w + sl);
    const int32_t* cp = A.col + (size_t)sl * K * 32 + lane;
    const float* vq = A.val32 + qsell_index(row, 0, K);
    float s = 0.f;
    for (int m = 0; m < w; m++)
        s = fmaf(__ldg(vq + (m >> 2) * 128 + (m & 3)), __ldcg(u + __ldg(cp + m * 32)) - ui, s);
    return s;
}

// Compact FP32 row: per group of four entries one 16-byte value word and one
// 4-byte word of index bytes (2 bits: which of the row's three candidate
// ranges, 6 bits: offset in it); the range starts are stored per row.  The
// loads of kGroups groups are issued before any of their gathers and those
// before the multiply-adds, so that a warp keeps several groups' memory
// traffic in flight (a warp issues in order: it stalls at the first use of
// a load).  Summation order is per group (a0: entries 0, 2; a1: 1, 3), the
// same for any kGroups.
constexpr int kGroups = 4;
__device__ __forceinline__ float compact_row_sum(const Ppe& A, const MatFree& mf, int K, int row,
                                                 const float* __restrict__ u, float ui) {
    const int sl = row >> 5;
    const int w = __ldg(A.slice_w + sl);
    const int s0 = __ldg(mf.rs + row), s1 = __ldg(mf.rs + mf.rs_stride + row),
              s2 = __ldg(mf.rs + 2 * mf.rs_stride + row);
    const size_t q0 = qsell_index(row, 0, K) >> 2;  // in 16-byte words
    const float4* vp = reinterpret_cast<const float4*>(A.val32) + q0;
    const uint32_t* ip = reinterpret_cast<const uint32_t*>(mf.idx8) + q0;
    auto col = [&](uint32_t b4, int t) {
        const uint32_t b = (b4 >> (8 * t)) & 255u;
        const uint32_t r = b >> 6;
        return (r == 0 ? s0 : (r == 1 ? s1 : s2)) + (int)(b & 63u);
    };
    float a0 = 0.f, a1 = 0.f;
    const int groups = (w + 3) >> 2;
    int g = 0;
    for (; g + kGroups <= groups; g += kGroups) {
        float4 v[kGroups];
        uint32_t b4[kGroups];
#pragma unroll
        for (int q = 0; q < kGroups; q++) {
            v[q] = __ldg(vp + (g + q) * 32);
            b4[q] = __ldg(ip + (g + q) * 32);
        }
        float x[kGroups][4];
#pragma unroll
        for (int q = 0; q < kGroups; q++)
#pragma unroll
            for (int t = 0; t < 4; t++) x[q][t] = __ldcg(u + col(b4[q], t)) - ui;
#pragma unroll
        for (int q = 0; q < kGroups; q++) {
            a0 = fmaf(v[q].x, x[q][0], a0);
            a1 = fmaf(v[q].y, x[q][1], a1);
            a0 = fmaf(v[q].z, x[q][2], a0);
            a1 = fmaf(v[q].w, x[q][3], a1);
        }
    }
    for (; g < groups; g++) {
        const float4 v = __ldg(vp + g * 32);
        const uint32_t b4 = __ldg(ip + g * 32);
        float x[4];
#pragma unroll
        for (int t = 0; t < 4; t++) x[t] = __ldcg(u + col(b4, t)) - ui;
        a0 = fmaf(v.x, x[0], a0);
        a1 = fmaf(v.y, x[1], a1);
        a0 = fmaf(v.z, x[2], a0);
        a1 = fmaf(v.w, x[3], a1);
    }
    return a0 + a1;
}

// Compact sums of two rows of different slices at once (their groups'
// loads interleaved: twice the memory traffic in flight per thread), given
// both rows' slice widths (both > 0) and range starts.  One loop over the wider row's
// groups, two groups of each row per pass; past a row's own groups it
// re-reads its last group with weight 0, which adds exactly +0, so each
// row's sum equals compact_row_sum's (group by group, a0: entries 0, 2;
// a1: 1, 3) without a serial tail per row.
__device__ __forceinline__ void compact_pair(const Ppe& A, const MatFree& mf, int K, int ra, int rb,
                                             int wa, int wb, const int (&sa)[3], const int (&sb)[3],
                                             const float* __restrict__ u, float ua, float ub, float& oa,
                                             float& ob) {
    const float4* vpa = reinterpret_cast<const float4*>(A.val32) + (qsell_index(ra, 0, K) >> 2);
    const float4* vpb = reinterpret_cast<const float4*>(A.val32) + (qsell_index(rb, 0, K) >> 2);
    const uint32_t* ipa = reinterpret_cast<const uint32_t*>(mf.idx8) + (qsell_index(ra, 0, K) >> 2);
    const uint32_t* ipb = reinterpret_cast<const uint32_t*>(mf.idx8) + (qsell_index(rb, 0, K) >> 2);
    auto col = [](const int (&st)[3], uint32_t b4, int t) {
        const uint32_t b = (b4 >> (8 * t)) & 255u;
        const uint32_t r = b >> 6;
        return (r == 0 ? st[0] : (r == 1 ? st[1] : st[2])) + (int)(b & 63u);
    };
    const int ga = (wa + 3) >> 2, gb = (wb + 3) >> 2, gmax = max(ga, gb);
    float a0 = 0.f, a1 = 0.f, b0 = 0.f, b1 = 0.f;
    for (int g = 0; g < gmax; g += 2) {
        const int ha0 = min(g, ga - 1), ha1 = min(g + 1, ga - 1);
        const int hb0 = min(g, gb - 1), hb1 = min(g + 1, gb - 1);
        float4 va0 = __ldg(vpa + ha0 * 32), va1 = __ldg(vpa + ha1 * 32);
        float4 vb0 = __ldg(vpb + hb0 * 32), vb1 = __ldg(vpb + hb1 * 32);
        const uint32_t ia0 = __ldg(ipa + ha0 * 32), ia1 = __ldg(ipa + ha1 * 32);
        const uint32_t ib0 = __ldg(ipb + hb0 * 32), ib1 = __ldg(ipb + hb1 * 32);
        float xa[8], xb[8];
#pragma unroll
        for (int t = 0; t < 4; t++) {
            xa[t] = __ldcg(u + col(sa, ia0, t)) - ua;
            xa[4 + t] = __ldcg(u + col(sa, ia1, t)) - ua;
            xb[t] = __ldcg(u + col(sb, ib0, t)) - ub;
            xb[4 + t] = __ldcg(u + col(sb, ib1, t)) - ub;
        }
        const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        if (g >= ga) va0 = z;
        if (g + 1 >= ga) va1 = z;
        if (g >= gb) vb0 = z;
        if (g + 1 >= gb) vb1 = z;
        a0 = fmaf(va0.x, xa[0], a0);
        a1 = fmaf(va0.y, xa[1], a1);
        a0 = fmaf(va0.z, xa[2], a0);
        a1 = fmaf(va0.w, xa[3], a1);
        a0 = fmaf(va1.x, xa[4], a0);
        a1 = fmaf(va1.y, xa[5], a1);
        a0 = fmaf(va1.z, xa[6], a0);
        a1 = fmaf(va1.w, xa[7], a1);
        b0 = fmaf(vb0.x, xb[0], b0);
        b1 = fmaf(vb0.y, xb[1], b1);
        b0 = fmaf(vb0.z, xb[2], b0);
        b1 = fmaf(vb0.w, xb[3], b1);
        b0 = fmaf(vb1.x, xb[4], b0);
        b1 = fmaf(vb1.y, xb[5], b1);
        b0 = fmaf(vb1.z, xb[6], b0);
        b1 = fmaf(vb1.w, xb[7], b1);
    }
    oa = a0 + a1;
    ob = b0 + b1;
}

// Off-diagonal parts of rows i and i2 (i2 < 0: none), paired when both are
// compact.  Both rows' format flags, slice widths and range starts are loaded
// in one batch, before the branch that needs the flags.
__device__ __forceinline__ void off_rows(const Ppe& A, const MatFree& mf, int K, int i, int i2,
                                         const float* __restrict__ v, float vi, float vi2, float& o,
                                         float& o2) {
    if (!mf.enabled) {
        o = spmv32_sell_row(A, K, i, v, vi);
        o2 = i2 >= 0 ? spmv32_sell_row(A, K, i2, v, vi2) : 0.f;
        return;
    }
    const int j2 = i2 >= 0 ? i2 : i;  // a lone row is paired with itself
    const int8_t fa = mf.sell_row[i], fb = mf.sell_row[j2];
    const int wa = __ldg(A.slice_w + (i >> 5)), wb = __ldg(A.slice_w + (j2 >> 5));
    const int sa[3] = {__ldg(mf.rs + i), __ldg(mf.rs + mf.rs_stride + i), __ldg(mf.rs + 2 * mf.rs_stride + i)};
    const int sb[3] = {__ldg(mf.rs + j2), __ldg(mf.rs + mf.rs_stride + j2), __ldg(mf.rs + 2 * mf.rs_stride + j2)};
    // pairs need a group in each row (a slice of rows without off-diagonals
    // has width 0 and no stored groups at all)
    if (!fa && !fb && wa > 0 && wb > 0) {
        compact_pair(A, mf, K, i, j2, wa, wb, sa, sb, v, vi, i2 >= 0 ? vi2 : vi, o, o2);
        if (i2 < 0) o2 = 0.f;
        return;
    }
    o = fa ? spmv32_sell_row(A, K, i, v, vi) : compact_row_sum(A, mf, K, i, v, vi);
    o2 = i2 < 0 ? 0.f : (fb ? spmv32_sell_row(A, K, i2, v, vi2) : compact_row_sum(A, mf, K, i2, v, vi2));
}

// ----------------------------------------------------------------- FP64 CG
// A step whose matrix failed the symmetry test skips its solve (the
// reference exits there); every block reads the flag, set before the launch.
__device__ __forceinline__ bool solve_skipped(DevStats* ds) {
    if (!(*(volatile int32_t*)&ds->status & ST_ASYMMETRIC)) return false;
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        ds->cg_iterations = 0;
        ds->refinements = 0;
        ds->cg_rel_residual = -1.0;
    }
    return true;
}

__global__ void __launch_bounds__(kBlock, 1) k_cg64(Ppe A, Krylov kv, SolveArgs a, DevStats* ds) {
    if (solve_skipped(ds)) return;
    GridBar gb = whole_grid(kv);
    const int lane = threadIdx.x & 31;
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;

    double acc[1] = {0.0}, tot[1];
    for (int sl = gwarp; sl < a.nslices; sl += nwarps) {
        int i = sl * 32 + lane;
        if (i >= a.n) continue;
        double d = A.diag[i];
        kv.inv_diag[i] = d != 0.0 ? 1.0 / d : 1.0;
        double b = A.src[i];
        kv.x[i] = 0.0;
        kv.r[i] = b;
        acc[0] = fma(b, b, acc[0]);
    }
    if (!reduce_sync<1, kBlock>(gb, acc, tot, ds)) return;
    const double rhs2 = tot[0];
    int64_t it = 0;
    double rn2 = rhs2;
    bool conv = true;
    if (rhs2 > 0.0) {
        const double thr = fmax(a.tol * a.tol * rhs2, DBL_MIN);
        if (!(rn2 < thr)) {
            double a1[1] = {0.0}, t1[1];
            for (int sl = gwarp; sl < a.nslices; sl += nwarps) {
                int i = sl * 32 + lane;
                if (i >= a.n) continue;
                double r = kv.r[i];
                double p = kv.inv_diag[i] * r;
                kv.p[i] = p;
                a1[0] = fma(r, p, a1[0]);
            }
            if (!reduce_sync<1, kBlock>(gb, a1, t1, ds)) return;
            double abs_new = t1[0];
            while (it < a.max_iter) {
                double a2[1] = {0.0}, t2[1];
                for (int sl = gwarp; sl < a.nslices; sl += nwarps) {
                    int i = sl * 32 + lane;
                    if (i >= a.n) continue;
                    double pi = kv.p[i];
                    double q = spmv64_row(A, a.K, sl, lane, i, kv.p, pi);
                    kv.q[i] = q;
                    a2[0] = fma(pi, q, a2[0]);
                }
                if (!reduce_sync<1, kBlock>(gb, a2, t2, ds)) return;
                const double alpha = abs_new / t2[0];
                double a3[2] = {0.0, 0.0}, t3[2];
                for (int sl = gwarp; sl < a.nslices; sl += nwarps) {
                    int i = sl * 32 + lane;
                    if (i >= a.n) continue;
                    kv.x[i] = fma(alpha, kv.p[i], kv.x[i]);
                    double r = fma(-alpha, kv.q[i], kv.r[i]);
                    kv.r[i] = r;
                    double z = kv.inv_diag[i] * r;
                    kv.z[i] = z;
                    a3[0] = fma(r, r, a3[0]);
                    a3[1] = fma(r, z, a3[1]);
                }
                if (!reduce_sync<2, kBlock>(gb, a3, t3, ds)) return;
                rn2 = t3[0];
                if (rn2 < thr) break;
                const double beta = t3[1] / abs_new;
                abs_new = t3[1];
                for (int sl = gwarp; sl < a.nslices; sl += nwarps) {
                    int i = sl * 32 + lane;
                    if (i >= a.n) continue;
                    kv.p[i] = fma(beta, kv.p[i], kv.z[i]);
                }
                it++;
                if (!grid_sync(gb, ds)) return;
            }
        }
        conv = rn2 < thr;
    } else {
        rn2 = 0.0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ds->cg_iterations = it;
        ds->refinements = 0;
        ds->cg_rel_residual = rhs2 > 0.0 ? sqrt(rn2 / rhs2) : 0.0;
        if (!conv) atomicOr(&ds->status, ST_NOT_CONVERGED);
    }
}

// --------------------------------------------------------------- mixed IR
// Error-free FP32 product accumulated with compensation (hi, lo).
__device__ __forceinline__ void acc_prod(F2& a, float x, float y) {
    float p = x * y;
    float e = fmaf(x, y, -p);
    float s = a.hi + p;
    float bb = s - a.hi;
    float err = (a.hi - (s - bb)) + (p - bb);
    a.hi = s;
    a.lo += err + e;
}

// Loads of multigrid data: the vectors change during the solve (L2), the
// stencils and inverse diagonals do not (read-only cache).
__device__ __forceinline__ float ldv(const float* p, int i) { return __ldcg(p + i); }
__device__ __forceinline__ float ldc(const float* p, size_t i) { return __ldg(p + i); }

constexpr bool kPrefetchStencil = true;
__device__ __forceinline__ void prefetch_l2(const void* p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// Tap (dx, dy) of a 9-point stencil at (x, y): the neighbour's index,
// clamped into the grid so that its loads are always legal (no branch, so the
// compiler can issue every tap's loads at once), and whether it exists.
__device__ __forceinline__ int tap(const MgLevel& L, int x, int y, int d, bool& ok) {
    const int nx = x + d / 3 - 1, ny = y + d % 3 - 1;
    ok = nx >= 0 && ny >= 0 && nx < L.nx && ny < L.ny;
    return min(max(nx, 0), L.nx - 1) * L.ny + min(max(ny, 0), L.ny - 1);
}

// Pre-smoothed residual of fine level F restricted to cell I = (X, Y) of
// level C: the 4x4 stencil C.rw on r_F (the children's residual after one
// Jacobi step from zero, folded at setup).  Taps are clamped into the grid
// (their weights are 0 there), so all 32 loads are unconditional and in
// flight together: one memory round trip per coarse cell, which after a
// grid barrier is an L2 access, often on the other die.
__device__ __forceinline__ float restrict_cell(const MgLevel& F, const MgLevel& C, int I, int X,
                                               int Y) {
    const int nc = C.nx * C.ny;
    if (kPrefetchStencil) {
        // the up pass reads the children's 9-point stencils: start moving
        // them into L2 now (no register or stall cost), since nothing on the
        // way down reads them any more
        const size_t nf = (size_t)F.nx * F.ny;
#pragma unroll
        for (int a = 0; a < 2; a++) {
            const size_t c = (size_t)min(2 * X + a, F.nx - 1) * F.ny + min(2 * Y, F.ny - 1);
#pragma unroll
            for (int d = 0; d < 9; d++) prefetch_l2(F.st + d * nf + c);
        }
    }
    int xs[4], ys[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        xs[k] = min(max(2 * X - 1 + k, 0), F.nx - 1) * F.ny;
        ys[k] = min(max(2 * Y - 1 + k, 0), F.ny - 1);
    }
    float w[16], v[16];
#pragma unroll
    for (int k = 0; k < 16; k++) {
        w[k] = ldc(C.rw, (size_t)k * nc + I);
        v[k] = ldv(F.r, xs[k >> 2] + ys[k & 3]);
    }
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < 16; k++) acc = fmaf(w[k], v[k], acc);
    return acc;
}

// Post-smoothing of a level with the prolongation folded in: the corrected
// value of a cell is e + s * e_parent, computed on the fly for the cell and
// its 8 neighbours, so prolongation needs no pass or barrier of its own.
// Taps clamped and masked: all loads in one batch.
__device__ __forceinline__ float smooth_up_cell(const Mg& mg, const MgLevel& L, const MgLevel& C,
                                                int I) {
    const int n = L.nx * L.ny;
    const int x = I / L.ny, y = I - x * L.ny;
    const float ei = fmaf(mg.scale, ldv(C.e, (x / 2) * C.ny + y / 2), ldv(L.e, I));
    float st[9], ej[9];
    bool ok[9];
#pragma unroll
    for (int d = 0; d < 9; d++) {
        const int j = tap(L, x, y, d, ok[d]);
        const int jx = j / L.ny, jy = j - jx * L.ny;
        st[d] = ldc(L.st, (size_t)d * n + I);
        ej[d] = fmaf(mg.scale, ldv(C.e, (jx / 2) * C.ny + jy / 2), ldv(L.e, j));
    }
    const float iv = ldc(L.invd, I), ri = ldv(L.r, I);
    float acc = 0.f;
#pragma unroll
    for (int d = 0; d < 9; d++)
        if (ok[d]) acc = fmaf(st[d], ej[d], acc);
    return fmaf(mg.omega * iv, ri - acc, ei);
}

// ------------------------------------------------------------ level views
// The hierarchy descriptor (Mg) stays where the launch put it, in read-only
// kernel parameter space: no thread keeps a copy of it.  Each up-smoothing of
// a grid-wide level writes the level's t array, after which the roles of e
// and t swap; a thread tracks the swaps of levels 1..ngrid in a bit mask
// (bit l set: e and t exchanged), the same in every thread that runs the
// cycle.  The first level the block cycle runs, lo = ngrid + 1, never swaps:
// its pre-smoothing is in e, the correction the block cycle hands back in t.
// The levels below lo belong to the block cycle and start from their base
// roles in every cycle.
__device__ __forceinline__ MgLevel lev_view(const Mg& mg, int l, uint32_t swp) {
    MgLevel L = mg.lev[l];
    if ((swp >> l) & 1u) {
        float* t = L.e;
        L.e = L.t;
        L.t = t;
    }
    return L;
}

// Level lo as the coarse level of the up pass at level ngrid: e = its correction.
__device__ __forceinline__ MgLevel lo_corrected(const Mg& mg) {
    MgLevel L = mg.lev[mg.ngrid + 1];
    L.e = L.t;
    return L;
}

// Level 1's correction after a cycle, and the array that takes its next
// pre-smoothing (the same array once level 1 is grid-wide: the correction is
// consumed first).
__device__ __forceinline__ float* level1_correction(const Mg& mg, uint32_t swp) {
    return mg.ngrid >= 1 ? lev_view(mg, 1, swp).e : mg.lev[1].t;
}
__device__ __forceinline__ float* level1_presmooth(const Mg& mg, uint32_t swp) {
    return lev_view(mg, 1, swp).e;
}

// Levels lo..nlev of the V-cycle, run by the group's first block alone (they
// are small): down smoothing + restriction, the dense coarsest solve, up
// smoothing with the prolongation folded in.  Only block-level barriers of
// the group NT inside; the caller brackets it with grid barriers.  Level lo's
// r and pre-smoothing were written by the grid pass; its correction goes to
// its t array.
template <int NT>
__device__ void mg_block_cycle(const Mg& mg, int lo) {
    const int tid = threadIdx.x, nt = NT == 0 ? (int)blockDim.x : NT;
    uint32_t bsw = 0;  // role swaps of the levels below lo in this cycle
    for (int l = lo; l < mg.nlev; l++) {
        const MgLevel L = l == lo ? mg.lev[lo] : lev_view(mg, l, bsw);
        const MgLevel C = lev_view(mg, l + 1, bsw);
        const bool smooth = l + 1 < mg.nlev;
        for (int I = tid; I < C.nx * C.ny; I += nt) {
            const int X = I / C.ny, Y = I - X * C.ny;
            const float iv = ldc(C.invd, I);
            const float rr = iv > 0.f ? restrict_cell(L, C, I, X, Y) : 0.f;
            C.r[I] = rr;
            if (smooth) C.e[I] = mg.omega * iv * rr;
        }
        group_bar<NT>();
    }
    {
        // coarsest level: e = A_c^-1 r, one warp per row (lanes split the
        // row); a warp's rows (up to kDenseRows of them) in one pass, so that
        // all their loads are in flight together
        constexpr int kDenseRows = 6;
        const MgLevel L = lev_view(mg, mg.nlev, bsw);
        float* out = mg.nlev == lo ? L.t : L.e;
        const int n = L.nx * L.ny;
        const int lane = tid & 31, nw = nt >> 5;
        for (int i0 = tid >> 5; i0 < n; i0 += kDenseRows * nw) {
            float acc[kDenseRows];
#pragma unroll
            for (int q = 0; q < kDenseRows; q++) acc[q] = 0.f;
            for (int j = lane; j < n; j += 32) {
                const float rj = ldv(L.r, j);
#pragma unroll
                for (int q = 0; q < kDenseRows; q++) {
                    const int i = i0 + q * nw;
                    if (i < n) acc[q] = fmaf(__ldg(mg.dense + i * n + j), rj, acc[q]);
                }
            }
#pragma unroll
            for (int q = 0; q < kDenseRows; q++) {
                const int i = i0 + q * nw;
                float a = acc[q];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
                if (lane == 0 && i < n) out[i] = ldc(L.invd, i) > 0.f ? a : 0.f;
            }
        }
        group_bar<NT>();
    }
    for (int l = mg.nlev - 1; l >= lo; l--) {
        const MgLevel L = l == lo ? mg.lev[lo] : lev_view(mg, l, bsw);
        const MgLevel C = lev_view(mg, l + 1, bsw);
        const int n = L.nx * L.ny;
        for (int I = tid; I < n; I += nt) L.t[I] = ldc(L.invd, I) > 0.f ? smooth_up_cell(mg, L, C, I) : 0.f;
        group_bar<NT>();
        if (l > lo) bsw ^= 1u << l;
    }
}

// Level 1 of plain aggregation: the sum over each cell's contiguous slots of
// src0, pre-smoothed (e = omega invd r), for the cells with unknowns (the
// others hold 0).  Four of this thread's cells at once, their slots four at
// a time, all loads of a round before any use (predicated: slots past a
// cell's end are not read): each cell still sums its slots in slot order.
// gcell / gsz: this thread's first list entry and the group's stride;
// e_out: the array that receives the pre-smoothing (level1_presmooth).
__device__ __forceinline__ void mg_level1_plain(const Mg& mg, const MatFree& mf,
                                                const float* __restrict__ src0, int gcell, int gsz,
                                                float* __restrict__ e_out) {
    const MgLevel& L1 = mg.lev[1];
    const int na = __ldg(mg.nact + 1);
    for (int a0 = gcell; a0 < na; a0 += 4 * gsz) {
        int b[4], cnt[4], cell[4];
        float iv[4], acc[4];
#pragma unroll
        for (int h = 0; h < 4; h++) {
            const int a = min(a0 + h * gsz, na - 1);
            cell[h] = __ldg(L1.act + a);
            const int2 rg = __ldg(mg.act1_rng + a);
            b[h] = rg.x;
            cnt[h] = rg.y;
            acc[h] = 0.f;
        }
#pragma unroll
        for (int h = 0; h < 4; h++) iv[h] = __ldg(L1.invd + cell[h]);
        const int m = max(max(cnt[0], cnt[1]), max(cnt[2], cnt[3]));
        for (int j = 0; j < m; j += 4) {
            float x[4][4];
#pragma unroll
            for (int h = 0; h < 4; h++)
#pragma unroll
                for (int q = 0; q < 4; q++) x[h][q] = j + q < cnt[h] ? __ldcg(src0 + b[h] + j + q) : 0.f;
#pragma unroll
            for (int h = 0; h < 4; h++)
#pragma unroll
                for (int q = 0; q < 4; q++)
                    if (j + q < cnt[h]) acc[h] += x[h][q];
        }
#pragma unroll
        for (int h = 0; h < 4; h++) {
            if (a0 + h * gsz < na) {
                L1.r[cell[h]] = acc[h];
                e_out[cell[h]] = mg.omega * iv[h] * acc[h];
            }
        }
    }
}

// The cell levels of the V-cycle after level 1's residual and pre-smoothing
// were written: a grid barrier, the grid-wide levels down (restriction
// fused with the next level's pre-smoothing), the small levels in the
// group's first block, the grid-wide levels up (prolongation folded into the post-smoothing), each
// phase closed by a grid barrier of the thread group NT (0: whole blocks).
// Afterwards level 1's correction is complete for every block
// (level1_correction).  sync_first = false skips the first barrier where
// the caller passed one since level 1 was written.  swp: the role swaps.
template <int NT>
__device__ __forceinline__ bool mg_cell_levels(const Mg& mg, uint32_t& swp, GridBar& gb, DevStats* ds,
                                               int gcell, int gsz, bool sync_first = true) {
    if (sync_first && !grid_sync<NT>(gb, ds)) return false;
    const int lo = mg.ngrid + 1;
    // grid-wide levels, down: restrict level l into l+1 and pre-smooth there
    // (every level but the coarsest, whose e comes from its dense inverse),
    // the cells with unknowns only: the others hold 0
    for (int l = 1; l <= mg.ngrid; l++) {
        const MgLevel L = lev_view(mg, l, swp);
        const MgLevel C = l + 1 == lo ? mg.lev[lo] : lev_view(mg, l + 1, swp);
        const bool smooth = l + 1 < mg.nlev;
        const int na = __ldg(mg.nact + l + 1);
        for (int a = gcell; a < na; a += gsz) {
            const int I = __ldg(C.act + a);
            const int X = I / C.ny, Y = I - X * C.ny;
            const float iv = __ldg(C.invd + I);
            const float rr = restrict_cell(L, C, I, X, Y);
            C.r[I] = rr;
            if (smooth) C.e[I] = mg.omega * iv * rr;
        }
        if (!grid_sync<NT>(gb, ds)) return false;
    }
    // small levels in the group's first block
    if (gb.rank == 0) mg_block_cycle<NT>(mg, lo);
    if (!grid_sync<NT>(gb, ds)) return false;
    // grid-wide levels, up: prolongation folded into the post-smoothing
    for (int l = mg.ngrid; l >= 1; l--) {
        const MgLevel L = lev_view(mg, l, swp);
        const MgLevel C = l == mg.ngrid ? lo_corrected(mg) : lev_view(mg, l + 1, swp);
        const int na = __ldg(mg.nact + l);
        for (int a = gcell; a < na; a += gsz) {
            const int I = __ldg(L.act + a);
            L.t[I] = smooth_up_cell(mg, L, C, I);
        }
        if (!grid_sync<NT>(gb, ds)) return false;
        swp ^= 1u << l;
    }
    return true;
}

// u = M r: one symmetric V(1,1) cycle with damped Jacobi smoothing.  The
// caller has already written e0 = omega D^-1 r (level-0 pre-smoothing, local)
// and passed a grid barrier.  Restriction is fused with the next level's
// pre-smoothing, prolongation with the post-smoothing.  Ends after writing u
// (no trailing barrier).  Every block runs the same barrier sequence.
template <int BS>
__device__ __forceinline__ bool mg_vcycle(const Mg& mg, uint32_t& swp, const Ppe& A, const MatFree& mf,
                                          int K, const float* __restrict__ r, float* __restrict__ u,
                                          const float* __restrict__ invd0, int n, GridBar& gb,
                                          DevStats* ds) {
    const int gtid = gb.rank * BS + threadIdx.x;
    const int gsz = gb.size * BS;
    // Cells of the grid levels are dealt to blocks in interleaved 32-cell
    // chunks (coalesced within a warp): the cells with unknowns cover only
    // the fluid's part of the tank, and a contiguous split would hand them all
    // to a few blocks while the rest wait at the next barrier.
    const int gcell = ((threadIdx.x >> 5) * gb.size + gb.rank) * 32 + (threadIdx.x & 31);
    // level 0 residual of the Inner particles (coalesced, one row per thread);
    // the additive form restricts r itself
    const float* src0 = mg.additive ? r : mg.res0;
    if (!mg.additive) {
    for (int i = gtid; i < n; i += 2 * gsz) {
        const int i2 = i + gsz < n ? i + gsz : -1;
        const float ea = __ldcg(mg.e0 + i), eb = i2 >= 0 ? __ldcg(mg.e0 + i2) : 0.f;
        float o, o2;
        off_rows(A, mf, K, i, i2, mg.e0, ea, eb, o, o2);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int row = h == 0 ? i : i2;
            if (row < 0) break;
            const float dg = A.diag32[row];
            mg.res0[row] = dg > 0.f ? __ldcg(r + row) - fmaf(A.rsum32[row], h == 0 ? ea : eb, h == 0 ? o : o2) : 0.f;
        }
    }
    if (!grid_sync(gb, ds)) return false;
    }
    // level 1: sum over each cell's contiguous slots; pre-smooth.  Four of
    // this thread's cells at once, their slots four at a time, all loads of
    // a round before any use (predicated: slots past a cell's end are not
    // read, which also keeps the many empty cells off any one address):
    // each cell still sums its slots in slot order.
    if (mg.smooth) {
        // smoothed transfer: r1 = P^T r = P1^T r - omega B^T D^-1 r, where row i
        // of the 3x3 cells around cell I adds B[d][i] r_i / d_i with d the
        // offset from its cell to I.  A column of three cells is one slot
        // range (rows in cell order), split by the cell starts.
        const MgLevel& L1 = mg.lev[1];
        float* __restrict__ e1pre = level1_presmooth(mg, swp);
        const int n1 = L1.nx * L1.ny, NY = L1.ny;
        const size_t np = (size_t)mg.n_pad;
        for (int I = gcell; I < n1; I += gsz) {
            const float iv = __ldg(L1.invd + I);
            float rr = 0.f;
            if (iv > 0.f) {  // a cell with an unknown: an interior cell of the grid
                const int cx = I / NY, cy = I - cx * NY;
                // the 12 cell starts of the three columns in one batch
                int cb[3][4];
#pragma unroll
                for (int x = 0; x < 3; x++)
#pragma unroll
                    for (int q = 0; q < 4; q++) cb[x][q] = __ldg(mf.cs + (cx - 1 + x) * NY + cy - 1 + q);
                // own cell (column x = 1, cell q = 1), eight slots per batch of
                // predicated loads; sums in slot order
                float acc = 0.f;
                for (int i0 = cb[1][1]; i0 < cb[1][2]; i0 += 8) {
                    float v[8];
#pragma unroll
                    for (int h = 0; h < 8; h++) v[h] = i0 + h < cb[1][2] ? __ldcg(src0 + i0 + h) : 0.f;
#pragma unroll
                    for (int h = 0; h < 8; h++)
                        if (i0 + h < cb[1][2]) acc += v[h];
                }
                float corr = 0.f;
#pragma unroll 1
                for (int x = 0; x < 3; x++) {
                    const int c0 = cb[x][0], c1 = cb[x][1], c2 = cb[x][2], c3 = cb[x][3];
                    for (int i0 = c0; i0 < c3; i0 += 8) {
                        float bv[8], yv[8];
#pragma unroll
                        for (int h = 0; h < 8; h++) {
                            const int i = i0 + h;
                            const int q = (i >= c1) + (i >= c2);
                            const int d = (2 - x) * 3 + (2 - q);  // offset from the row's cell to I
                            const bool in = i < c3;
                            bv[h] = in ? __ldg(mg.rowcell + (size_t)d * np + i) : 0.f;
                            yv[h] = in ? __ldcg(src0 + i) * __ldg(invd0 + i) : 0.f;
                        }
#pragma unroll
                        for (int h = 0; h < 8; h++) corr = fmaf(bv[h], yv[h], corr);
                    }
                }
                rr = acc - mg.omega * corr;
            }
            L1.r[I] = rr;
            e1pre[I] = mg.omega * iv * rr;
        }
    } else {
        mg_level1_plain(mg, mf, src0, gcell, gsz, level1_presmooth(mg, swp));
    }
    if (!mg_cell_levels<0>(mg, swp, gb, ds, gcell, gsz)) return false;
    // level 1's correction
    const float* __restrict__ e1 = level1_correction(mg, swp);
    if (mg.additive && mg.smooth) {
        // u = omega D^-1 r + scale * P e1, P e1 = e1[cell(i)] - omega / d_i sum_d B[d][i] e1[cell(i) + d]
        const MgLevel& L1 = mg.lev[1];
        const int n1 = L1.nx * L1.ny, NY = L1.ny;
        const size_t np = (size_t)mg.n_pad;
        for (int i0 = gtid; i0 < n; i0 += 2 * gsz) {
            float dg[2], ri[2];
            int key[2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int i = min(i0 + h * gsz, n - 1);
                dg[h] = A.diag32[i];
                key[h] = min(__ldg(mf.skey + i), n1 - 1);
                ri[h] = __ldcg(r + i);
            }
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int i = i0 + h * gsz;
                if (i >= n) break;
                float v = 0.f;
                if (dg[h] > 0.f) {  // an unknown: its cell is interior
                    const int k = key[h];
                    const float ec = __ldcg(e1 + k);
                    float bt[9], en[9];
#pragma unroll
                    for (int d = 0; d < 9; d++) {
                        bt[d] = __ldg(mg.rowcell + (size_t)d * np + i);
                        en[d] = __ldcg(e1 + k + (d / 3 - 1) * NY + (d % 3 - 1));
                    }
                    float corr = 0.f;
#pragma unroll
                    for (int d = 0; d < 9; d++) corr = fmaf(bt[d], en[d], corr);
                    const float w = mg.omega / dg[h];
                    v = fmaf(mg.scale, ec - w * corr, w * ri[h]);
                }
                u[i] = v;
            }
        }
        return true;
    }
    if (mg.additive) {
        // u = omega D^-1 r + scale * (level-1 correction of the row's cell)
        const MgLevel& L1 = mg.lev[1];
        const int n1 = L1.nx * L1.ny;
        for (int i0 = gtid; i0 < n; i0 += 4 * gsz) {
            float dg[4], ri[4], ec[4];
            int key[4];
#pragma unroll
            for (int h = 0; h < 4; h++) {
                const int i = min(i0 + h * gsz, n - 1);
                dg[h] = A.diag32[i];
                key[h] = min(__ldg(mf.skey + i), n1 - 1);
                ri[h] = __ldcg(r + i);
            }
#pragma unroll
            for (int h = 0; h < 4; h++) ec[h] = dg[h] > 0.f ? __ldcg(e1 + key[h]) : 0.f;
#pragma unroll
            for (int h = 0; h < 4; h++) {
                const int i = i0 + h * gsz;
                if (i < n) u[i] = dg[h] > 0.f ? fmaf(mg.scale, ec[h], (mg.omega / dg[h]) * ri[h]) : 0.f;
            }
        }
        return true;
    }
    // level 1 -> 0: prolongate to the Inner particles, then post-smooth
    {
        const MgLevel& L1 = mg.lev[1];
        const int n1 = L1.nx * L1.ny;
        // four rows per iteration, loads first and tests after: two round
        // trips per four rows
        for (int i0 = gtid; i0 < n; i0 += 4 * gsz) {
            float dg[4], e0[4], ec[4];
            int key[4];
#pragma unroll
            for (int h = 0; h < 4; h++) {
                const int i = min(i0 + h * gsz, n - 1);
                dg[h] = A.diag32[i];
                key[h] = min(__ldg(mf.skey + i), n1 - 1);  // ghosts: sentinel key
                e0[h] = __ldcg(mg.e0 + i);
            }
#pragma unroll
            for (int h = 0; h < 4; h++) ec[h] = dg[h] > 0.f ? __ldcg(e1 + key[h]) : 0.f;
#pragma unroll
            for (int h = 0; h < 4; h++) {
                const int i = i0 + h * gsz;
                if (i < n && dg[h] > 0.f) mg.e0[i] = fmaf(mg.scale, ec[h], e0[h]);
            }
        }
    }
    if (!grid_sync(gb, ds)) return false;
    for (int i = gtid; i < n; i += 2 * gsz) {
        const int i2 = i + gsz < n ? i + gsz : -1;
        const float ea = __ldcg(mg.e0 + i), eb = i2 >= 0 ? __ldcg(mg.e0 + i2) : 0.f;
        float o, o2;
        off_rows(A, mf, K, i, i2, mg.e0, ea, eb, o, o2);
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int row = h == 0 ? i : i2;
            if (row < 0) break;
            const float dg = A.diag32[row];
            const float e0 = h == 0 ? ea : eb;
            u[row] = dg > 0.f ? fmaf(mg.omega / dg, __ldcg(r + row) - fmaf(A.rsum32[row], e0, h == 0 ? o : o2), e0)
                              : 0.f;
        }
    }
    return true;
}

// The mixed-precision solve of one scene by one group of BS-thread blocks
// (the whole grid for a single scene, or one scene's share of a batch).
template <int BS>
__device__ __forceinline__ void solve_mixed(const Ppe& A, const MatFree& mf, const Mg& mg,
                                            const Krylov& kv, const SolveArgs& a, DevStats* ds,
                                            GridBar& gb) {
    if (*(volatile int32_t*)&ds->status & ST_ASYMMETRIC) {  // the reference exits here
        if (gb.rank == 0 && threadIdx.x == 0) {
            ds->cg_iterations = 0;
            ds->refinements = 0;
            ds->cg_rel_residual = -1.0;
        }
        return;
    }
    const int gtid = gb.rank * BS + threadIdx.x;
    const int gsz = gb.size * BS;
    const int lane = threadIdx.x & 31;
    const int gwarp = gtid >> 5;
    const int nwarps = gsz >> 5;
    uint32_t swp = 0;  // e/t role swaps of the grid-wide levels (lev_view)

    double acc[1] = {0.0}, tot[1];
    for (int sl = gwarp; sl < a.nslices; sl += nwarps) {
        int i = sl * 32 + lane;
        if (i >= a.n) continue;
        if (!a.warm) kv.x[i] = 0.0;
        double b = A.src[i];
        acc[0] = fma(b, b, acc[0]);
    }
    if (!reduce_sync<1, BS>(gb, acc, tot, ds)) return;
    const double rhs2 = tot[0];
    // b = 0 has the solution 0 whatever the guess (the loop below does not run)
    if (a.warm && !(rhs2 > 0.0))
        for (int i = gtid; i < a.n; i += gsz) kv.x[i] = 0.0;
    const double thr = fmax(a.tol * a.tol * rhs2, DBL_MIN);
    int64_t inner_total = 0;
    int refine = 0;
    double rn2 = rhs2;
    while (rhs2 > 0.0) {
        // FP64 residual r = b - A x (x was made complete by the last barrier)
        double a0[1] = {0.0}, t0[1];
        for (int sl = gwarp; sl < a.nslices; sl += nwarps) {
            int i = sl * 32 + lane;
            if (i >= a.n) continue;
            double r = A.src[i] - spmv64_row(A, a.K, sl, lane, i, kv.x, kv.x[i]);
            kv.r[i] = r;
            a0[0] = fma(r, r, a0[0]);
        }
        if (!reduce_sync<1, BS>(gb, a0, t0, ds)) return;
        rn2 = t0[0];
        if (a.warm && refine == 0 && rn2 > rhs2) {
            // a guess worse than zero (a state replaced by mps_upload): start from zero
            for (int i = gtid; i < a.n; i += gsz) {
                kv.x[i] = 0.0;
                kv.r[i] = A.src[i];
            }
            rn2 = rhs2;
            if (!grid_sync(gb, ds)) return;
        }
        if (rn2 < thr || refine >= a.max_refine || inner_total >= a.max_iter) break;
        refine++;
        // inner solve of A d = r / ||r|| (unit right-hand side), to the
        // reduction this refinement still needs (with a 2x margin), but no
        // tighter than FP32 iterations can resolve
        const float ithr = (float)fmax(a.inner_tol * a.inner_tol, 0.25 * thr / rn2);
        const float scale = (float)(1.0 / sqrt(rn2));
        for (int i = gtid; i < a.n; i += gsz) {
            float r = f32(kv.r[i]) * scale;
            kv.r32[i] = r;
            kv.x32[i] = 0.f;
            kv.p32[i] = 0.f;
            kv.s32[i] = 0.f;
            if (mg.enabled)
                mg.e0[i] = mg.omega * kv.inv_diag32[i] * r;
            else
                kv.u32[i] = kv.inv_diag32[i] * r;
        }
        if (!grid_sync(gb, ds)) return;
        if (mg.enabled) {
            if (!mg_vcycle<BS>(mg, swp, A, mf, a.K, kv.r32, kv.u32, kv.inv_diag32, a.n, gb, ds)) return;
            if (!grid_sync(gb, ds)) return;
        }
        float alpha = 0.f, beta = 0.f, gamma_old = 1.f;
        int64_t k = 0;
        for (;;) {
            // phase B: w = A u ; gamma = r.u, delta = w.u, rho = r.r
            F2 g = {0.f, 0.f}, dl = {0.f, 0.f}, rr = {0.f, 0.f};
            // rows i and i + gsz of this thread together (their operator
            // loads interleaved); rows that are not unknowns (diagonal 0:
            // Surface, Ignored, ghosts) get w = +0
            for (int i = gtid; i < a.n; i += 2 * gsz) {
                const int i2 = i + gsz < a.n ? i + gsz : -1;
                // the rows' own words first: in flight with the operator's
                float ui[2], dg[2], rv[2];
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int row = h == 0 || i2 < 0 ? i : i2;
                    ui[h] = __ldcg(kv.u32 + row);
                    dg[h] = A.diag32[row];
                    rv[h] = kv.r32[row];
                }
                float o, o2;
                off_rows(A, mf, a.K, i, i2, kv.u32, ui[0], ui[1], o, o2);
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int row = h == 0 ? i : i2;
                    if (row < 0) break;
                    const float w = dg[h] > 0.f ? fmaf(A.rsum32[row], ui[h], h == 0 ? o : o2) : 0.f;
                    kv.w32[row] = w;
                    acc_prod(g, rv[h], ui[h]);
                    acc_prod(dl, w, ui[h]);
                    acc_prod(rr, rv[h], rv[h]);
                }
            }
            const F2 v3[3] = {g, dl, rr};
            float t3[3];
            if (!reduce_sync_f2<3, BS>(gb, v3, t3, ds)) return;
            if (t3[2] < ithr || inner_total + k >= a.max_iter) break;
            const float gamma = t3[0], delta = t3[1];
            if (k == 0) {
                beta = 0.f;
                alpha = gamma / delta;
            } else {
                beta = gamma / gamma_old;
                float den = delta - beta * gamma / alpha;
                if (!(den > 0.f)) break;  // loss of positive definiteness in FP32
                alpha = gamma / den;
            }
            gamma_old = gamma;
            // phase A: p = u + beta p ; s = w + beta s ; x += alpha p ; r -= alpha s ; u = M r
            // (the additive cycle starts from r alone: no level-0 pre-smoothing here)
            const bool need_id = !mg.enabled || !mg.additive;
            // Four of this thread's rows per iteration, all loads before any
            // store (the compiler cannot move loads above stores to arrays it
            // cannot prove distinct): four rows' memory traffic in flight.
            for (int i0 = gtid; i0 < a.n; i0 += 4 * gsz) {
                float u[4], p[4], s[4], w[4], x[4], r[4], id[4];
#pragma unroll
                for (int h = 0; h < 4; h++) {
                    const int i = min(i0 + h * gsz, a.n - 1);
                    u[h] = __ldcg(kv.u32 + i);
                    p[h] = kv.p32[i];
                    s[h] = kv.s32[i];
                    w[h] = kv.w32[i];
                    x[h] = kv.x32[i];
                    r[h] = kv.r32[i];
                    id[h] = need_id ? kv.inv_diag32[i] : 0.f;
                }
#pragma unroll
                for (int h = 0; h < 4; h++) {
                    const int i = i0 + h * gsz;
                    if (i >= a.n) break;
                    const float pn = fmaf(beta, p[h], u[h]);
                    const float sn = fmaf(beta, s[h], w[h]);
                    kv.p32[i] = pn;
                    kv.s32[i] = sn;
                    kv.x32[i] = fmaf(alpha, pn, x[h]);
                    const float rn = fmaf(-alpha, sn, r[h]);
                    kv.r32[i] = rn;
                    if (!mg.enabled)
                        kv.u32[i] = id[h] * rn;
                    else if (!mg.additive)
                        mg.e0[i] = mg.omega * id[h] * rn;
                }
            }
            k++;
            if (!grid_sync(gb, ds)) return;
            if (mg.enabled) {
                if (!mg_vcycle<BS>(mg, swp, A, mf, a.K, kv.r32, kv.u32, kv.inv_diag32, a.n, gb, ds)) return;
                if (!grid_sync(gb, ds)) return;
            }
        }
        inner_total += k;
        // x += d (FP64)
        const double back = sqrt(rn2);
        for (int i = gtid; i < a.n; i += gsz) kv.x[i] = fma((double)kv.x32[i], back, kv.x[i]);
        if (!grid_sync(gb, ds)) return;
    }
    if (gb.rank == 0 && threadIdx.x == 0) {
        ds->cg_iterations = inner_total;
        ds->refinements = refine;
        ds->cg_rel_residual = rhs2 > 0.0 ? sqrt(rn2 / rhs2) : 0.0;
        if (rhs2 > 0.0 && !(rn2 < thr)) atomicOr(&ds->status, ST_NOT_CONVERGED);
    }
}

// (Parameters are __grid_constant__: read where the launch put them, never
// copied per thread.)
__global__ void __launch_bounds__(kMixedBlock, 1)
    k_cg_mixed(__grid_constant__ const Ppe A, __grid_constant__ const MatFree mf, __grid_constant__ const Mg mg,
               __grid_constant__ const Krylov kv, __grid_constant__ const SolveArgs a, DevStats* ds) {
    GridBar gb = whole_grid(kv);
    solve_mixed<kMixedBlock>(A, mf, mg, kv, a, ds, gb);
}

// ----------------------------------------------- overlapped additive cycle
// Multigrid mode 1 (additive, plain transfer) arranged so that the level-0
// operator pass overlaps the cell levels of the V-cycle.  With y = D^-1 r and
// e1 the level-1 correction, the preconditioned residual is
//     u = omega y + scale P1 e1
// and, since A P1 = B (the rows' 3x3-cell sums, k_mg_rowcell),
//     w = A u = omega (A y) + scale B e1,
// where A y needs only r, not the cycle.  So after the vector update (which
// writes y) and one grid barrier, each block splits: its first kCycleThreads
// threads run the cycle (level-1 sums, the grid-wide levels with grid
// barriers of that group, the small levels in block 0), the other warps
// apply the FP32 operator to y for the block's own rows (z = A y).  The
// block joins, and one pass over its rows forms u, w and the three dot
// products.  The operator pass (most of an iteration's HBM traffic) is thus
// off the cycle's chain of dependent phases, and u and w never leave the
// block (no operator pass reads them).  Same Chronopoulos-Gear recurrences,
// refinement and stopping rules as solve_mixed.
//
// Rows: 32-row slices dealt to blocks 1..G-1 (block 0 runs the small levels).
constexpr int kCycleThreads = 512;
// The vector update of the overlapped solve gives each warp one contiguous
// range of rows that starts and ends at level-1 cell boundaries, walked in
// 64-row batches whose new residuals stay in a 128-row shared ring for the
// cells' sums.
constexpr int kRing = 128;

// The first slot at or after p that starts a level-1 cell (or n).
__device__ __forceinline__ int cell_start_at_or_after(const int32_t* __restrict__ skey, int p, int n) {
    const int lane = threadIdx.x & 31;
    for (; p < n; p += 32) {
        const int i = p + lane;
        const bool st = i < n && (i == 0 || __ldg(skey + i) != __ldg(skey + i - 1));
        const unsigned bal = __ballot_sync(0xffffffffu, st);
        if (bal) return p + __ffs(bal) - 1;
    }
    return n;
}

template <int BS, int NV>
__device__ __forceinline__ void solve_mixed_overlap(const Ppe& A, const MatFree& mf, const Mg& mg,
                                                    const Krylov& kv, const SolveArgs& a, DevStats* ds,
                                                    GridBar& gb) {
    if (*(volatile int32_t*)&ds->status & ST_ASYMMETRIC) {  // the reference exits here
        if (gb.rank == 0 && threadIdx.x == 0) {
            ds->cg_iterations = 0;
            ds->refinements = 0;
            ds->cg_rel_residual = -1.0;
        }
        return;
    }
    constexpr int kW = BS / 32, kVW = NV / 32, kZW = kW - kVW;
    static_assert(kVW > 0 && kZW > 0, "both groups need warps");
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int G = gb.size, b = gb.rank;
    const int gtid = b * BS + tid, gsz = G * BS;
    const int gwarp = gtid >> 5, nwarps = gsz >> 5;
    const int n = a.n, nsl = a.nslices;
    // The rows (32-row slices) of the operator pass, of the pass that forms
    // u and w and of the vector update belong to blocks 1..G-1: slices
    // rb, rb + RB, rb + 2 RB, ...  Block 0 runs the cycle's small levels and
    // does not also stream rows beside them.
    const int RB = G > 1 ? G - 1 : 1;
    const int rb = G > 1 ? b - 1 : 0;
    const bool has_rows = G == 1 || b > 0;
    // per-slot FP32 work vectors of this arrangement (the additive cycle uses
    // neither the level-0 correction nor the level-0 residual arrays)
    float* __restrict__ y = mg.e0;    // D^-1 r
    float* __restrict__ z = mg.res0;  // A y
    const size_t np = (size_t)mg.n_pad;
    const int NY = mg.lev[1].ny, n1 = mg.lev[1].nx * NY;
    // level 1's sums fused into the vector update (cell indices fit 24 bits)
    const bool fuse1 = n1 < (1 << 24);
    __shared__ int s_cycle_ok;
    __shared__ float s_ring[kW][kRing];
    // the e/t role swaps of the grid-wide levels (lev_view): the cycle group
    // makes them, the other warps follow with the same mask after each cycle
    uint32_t swp = 0;
    const uint32_t cycle_swaps = ((1u << (mg.ngrid + 1)) - 1u) & ~1u;  // levels 1..ngrid

    double acc[1] = {0.0}, tot[1];
    for (int sl = gwarp; sl < nsl; sl += nwarps) {
        int i = sl * 32 + lane;
        if (i >= n) continue;
        // the last slots of the level-1 cells with unknowns (fixed for the solve)
        if (fuse1) {
            const int key = __ldg(mf.skey + i);
            int32_t ce = -1;
            if (key < n1 && (i == n - 1 || key != __ldg(mf.skey + i + 1))) {
                const float iv = __ldg(mg.lev[1].invd + key);
                const int len = i + 1 - __ldg(mf.cs + key);
                if (iv > 0.f) ce = key | (min(len, 255) << 24);
            }
            mg.cell_end[i] = ce;
        }
        if (!a.warm) kv.x[i] = 0.0;
        double bb = A.src[i];
        acc[0] = fma(bb, bb, acc[0]);
    }
    if (!reduce_sync<1, BS>(gb, acc, tot, ds)) return;
    // this warp's rows of the vector update: [rlo, rhi), from the first cell
    // start at or after an even split point to the next warp's
    int rlo = 0, rhi = 0;
    if (has_rows) {
        const int nw = RB * kW, wi = rb * kW + warp;
        rlo = wi == 0 ? 0 : cell_start_at_or_after(mf.skey, (int)((int64_t)n * wi / nw), n);
        rhi = wi + 1 == nw ? n : cell_start_at_or_after(mf.skey, (int)((int64_t)n * (wi + 1) / nw), n);
    }
    const double rhs2 = tot[0];
    // b = 0 has the solution 0 whatever the guess (the loop below does not run)
    if (a.warm && !(rhs2 > 0.0))
        for (int i = gtid; i < n; i += gsz) kv.x[i] = 0.0;
    const double thr = fmax(a.tol * a.tol * rhs2, DBL_MIN);
    int64_t inner_total = 0;
    int refine = 0;
    double rn2 = rhs2;
    while (rhs2 > 0.0) {
        // FP64 residual r = b - A x
        double a0[1] = {0.0}, t0[1];
        for (int sl = gwarp; sl < nsl; sl += nwarps) {
            int i = sl * 32 + lane;
            if (i >= n) continue;
            double r = A.src[i] - spmv64_row(A, a.K, sl, lane, i, kv.x, kv.x[i]);
            kv.r[i] = r;
            a0[0] = fma(r, r, a0[0]);
        }
        if (!reduce_sync<1, BS>(gb, a0, t0, ds)) return;
        rn2 = t0[0];
        if (a.warm && refine == 0 && rn2 > rhs2) {
            // a guess worse than zero (a state replaced by mps_upload): start from zero
            for (int i = gtid; i < n; i += gsz) {
                kv.x[i] = 0.0;
                kv.r[i] = A.src[i];
            }
            rn2 = rhs2;
            if (!grid_sync(gb, ds)) return;
        }
        if (rn2 < thr || refine >= a.max_refine || inner_total >= a.max_iter) break;
        refine++;
        const float ithr = (float)fmax(a.inner_tol * a.inner_tol, 0.25 * thr / rn2);
        const float scale = (float)(1.0 / sqrt(rn2));
        for (int i = gtid; i < n; i += gsz) {
            const float r = f32(kv.r[i]) * scale;
            kv.r32[i] = r;
            kv.x32[i] = 0.f;
            kv.p32[i] = 0.f;
            kv.s32[i] = 0.f;
            y[i] = kv.inv_diag32[i] * r;
        }
        if (!grid_sync(gb, ds)) return;
        float alpha = 0.f, beta = 0.f, gamma_old = 1.f;
        int64_t k = 0;
        for (;;) {
            // ---- level 1 of the cycle: every warp sums r over the cells with
            // unknowns into the cycle group's level-1 arrays.  Only the first
            // iteration of a refinement: afterwards the vector update (below)
            // writes them for the next iteration
            if (k == 0 || !fuse1) {
                mg_level1_plain(mg, mf, kv.r32, ((warp * G + b) << 5) + lane, gsz,
                                level1_presmooth(mg, swp));
                if (!grid_sync(gb, ds)) return;
            }
            // ---- split: the cycle's cell levels on r, the operator on y
            if (warp < kVW) {
                const int gcell = ((warp * G + b) << 5) + lane;
                const bool ok = mg_cell_levels<NV>(mg, swp, gb, ds, gcell, G * NV, false);
                if (tid == 0) s_cycle_ok = ok;
            } else {
                for (int q = warp - kVW; has_rows; q += 2 * kZW) {
                    const int sl1 = rb + RB * q;
                    if (sl1 >= nsl) break;
                    const int sl2 = rb + RB * (q + kZW);
                    const int i = sl1 * 32 + lane;
                    int i2 = sl2 < nsl ? sl2 * 32 + lane : -1;
                    if (i2 >= n) i2 = -1;
                    if (i >= n) continue;  // the partial last slice (then i2 < 0 too)
                    const int j2 = i2 >= 0 ? i2 : i;
                    const float dg0 = A.diag32[i], dg1 = A.diag32[j2];
                    const float c0 = A.rsum32[i], c1 = A.rsum32[j2];
                    const float y0 = __ldcg(y + i), y1 = __ldcg(y + j2);
                    float o, o2;
                    off_rows(A, mf, a.K, i, i2, y, y0, y1, o, o2);
                    z[i] = dg0 > 0.f ? fmaf(c0, y0, o) : 0.f;
                    if (i2 >= 0) z[i2] = dg1 > 0.f ? fmaf(c1, y1, o2) : 0.f;
                }
                swp ^= cycle_swaps;
            }
            __syncthreads();
            if (!s_cycle_ok) return;
            const float* __restrict__ e1 = level1_correction(mg, swp);
            // ---- u = omega y + scale e1[cell], w = omega z + scale B e1, dot products
            F2 g = {0.f, 0.f}, dl = {0.f, 0.f}, rr = {0.f, 0.f};
            for (int q = warp; has_rows; q += 2 * kW) {
                const int sla = rb + RB * q;
                if (sla >= nsl) break;
                const int slb = rb + RB * (q + kW);
                int ii[2] = {sla * 32 + lane, slb < nsl ? slb * 32 + lane : n};
                float dg[2], cs[2], ri[2], yi[2], zi[2];
                int key[2];
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int i = min(ii[h], n - 1);
                    dg[h] = A.diag32[i];
                    cs[h] = A.rsum32[i];
                    ri[h] = __ldcg(kv.r32 + i);
                    yi[h] = __ldcg(y + i);
                    zi[h] = __ldcg(z + i);
                    key[h] = min(__ldg(mf.skey + i), n1 - 1);
                }
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    if (ii[h] >= n) break;
                    const int i = ii[h];
                    float u = 0.f, w = 0.f;
                    if (dg[h] > 0.f) {  // an unknown: its cell is interior
                        // B e1 = sum_d B_d e1_d in difference form around the
                        // row's own cell (d = 4): the B_d sum to the row sum
                        float bt[9], en[9];
#pragma unroll
                        for (int d = 0; d < 9; d++) {
                            bt[d] = d == 4 ? 0.f : __ldg(mg.rowcell + (size_t)d * np + i);
                            en[d] = __ldcg(e1 + key[h] + (d / 3 - 1) * NY + (d % 3 - 1));
                        }
                        float corr = 0.f;
#pragma unroll
                        for (int d = 0; d < 9; d++)
                            if (d != 4) corr = fmaf(bt[d], en[d] - en[4], corr);
                        corr = fmaf(cs[h], en[4], corr);
                        u = fmaf(mg.scale, en[4], mg.omega * yi[h]);
                        w = fmaf(mg.scale, corr, mg.omega * zi[h]);
                    }
                    kv.u32[i] = u;
                    kv.w32[i] = w;
                    acc_prod(g, ri[h], u);
                    acc_prod(dl, w, u);
                    acc_prod(rr, ri[h], ri[h]);
                }
            }
            const F2 v3[3] = {g, dl, rr};
            float t3[3];
            if (!reduce_sync_f2<3, BS>(gb, v3, t3, ds)) return;
            if (t3[2] < ithr || inner_total + k >= a.max_iter) break;
            const float gamma = t3[0], delta = t3[1];
            if (k == 0) {
                beta = 0.f;
                alpha = gamma / delta;
            } else {
                beta = gamma / gamma_old;
                float den = delta - beta * gamma / alpha;
                if (!(den > 0.f)) break;  // loss of positive definiteness in FP32
                alpha = gamma / den;
            }
            gamma_old = gamma;
            // ---- p = u + beta p ; s = w + beta s ; x += alpha p ; r -= alpha s ; y = D^-1 r,
            // fused with level 1 of the next cycle: this warp's rows hold whole
            // level-1 cells, so the lane holding a cell's last slot sums the
            // cell's new residuals in slot order and writes the level's residual
            // and pre-smoothing (the same values as the separate level-1 pass)
            {
                float* __restrict__ r1 = mg.lev[1].r;
                float* __restrict__ e1n = level1_presmooth(mg, swp);
                float* ring = s_ring[warp];
                for (int base = rlo; base < rhi; base += 64) {
                    float u[2], p[2], sv[2], w[2], x[2], r[2], id[2];
                    int32_t ce[2];
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const int i = min(base + 32 * h + lane, rhi - 1);
                        u[h] = __ldcg(kv.u32 + i);
                        p[h] = kv.p32[i];
                        sv[h] = kv.s32[i];
                        w[h] = __ldcg(kv.w32 + i);
                        x[h] = kv.x32[i];
                        r[h] = __ldcg(kv.r32 + i);
                        id[h] = kv.inv_diag32[i];
                        ce[h] = fuse1 ? __ldg(mg.cell_end + i) : -1;
                    }
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const int i = base + 32 * h + lane;
                        if (i < rhi) {
                            const float pn = fmaf(beta, p[h], u[h]);
                            const float sn = fmaf(beta, sv[h], w[h]);
                            kv.p32[i] = pn;
                            kv.s32[i] = sn;
                            kv.x32[i] = fmaf(alpha, pn, x[h]);
                            const float rn = fmaf(-alpha, sn, r[h]);
                            kv.r32[i] = rn;
                            y[i] = id[h] * rn;
                            ring[(i - rlo) & (kRing - 1)] = rn;
                        }
                    }
                    __syncwarp();
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const int i = base + 32 * h + lane;
                        if (i < rhi && ce[h] >= 0) {
                            const int key = ce[h] & 0xFFFFFF;
                            const float iv = __ldg(mg.lev[1].invd + key);
                            int len = (int)((unsigned)ce[h] >> 24);
                            if (len == 255) len = i + 1 - __ldg(mf.cs + key);
                            const int j0 = i + 1 - len;
                            float acc = 0.f;
                            // the ring holds this batch and the previous one
                            const int keep = max(base - 64, rlo);
                            for (int j = j0; j <= i; j++)
                                acc += j >= keep ? ring[(j - rlo) & (kRing - 1)] : __ldcg(kv.r32 + j);
                            r1[key] = acc;
                            e1n[key] = mg.omega * iv * acc;
                        }
                    }
                    __syncwarp();
                }
            }
            k++;
            if (!grid_sync(gb, ds)) return;
        }
        inner_total += k;
        // x += d (FP64)
        const double back = sqrt(rn2);
        for (int i = gtid; i < n; i += gsz) kv.x[i] = fma((double)kv.x32[i], back, kv.x[i]);
        if (!grid_sync(gb, ds)) return;
    }
    if (gb.rank == 0 && threadIdx.x == 0) {
        ds->cg_iterations = inner_total;
        ds->refinements = refine;
        ds->cg_rel_residual = rhs2 > 0.0 ? sqrt(rn2 / rhs2) : 0.0;
        if (rhs2 > 0.0 && !(rn2 < thr)) atomicOr(&ds->status, ST_NOT_CONVERGED);
    }
}

__global__ void __launch_bounds__(kMixedBlock, 1)
    k_cg_mixed_ov(__grid_constant__ const Ppe A, __grid_constant__ const MatFree mf, __grid_constant__ const Mg mg,
                  __grid_constant__ const Krylov kv, __grid_constant__ const SolveArgs a, DevStats* ds) {
    GridBar gb = whole_grid(kv);
    solve_mixed_overlap<kMixedBlock, kCycleThreads>(A, mf, mg, kv, a, ds, gb);
}

// Many scenes in one persistent launch: block b belongs to group bmap[b].x
// (one scene) with rank bmap[b].y; each group converges on its own.
struct SceneSolve {
    Ppe A;
    MatFree mf;
    Mg mg;
    Krylov kv;
    SolveArgs a;
    DevStats* ds;
};

template <int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_cg_mixed_batched(const SceneSolve* __restrict__ scenes,
                                                               const int2* __restrict__ bmap,
                                                               const int32_t* __restrict__ gsize,
                                                               unsigned int* bars) {
    const int2 m = bmap[blockIdx.x];
    const SceneSolve& s = scenes[m.x];
    GridBar gb{bars + 32 * m.x, 0u, 0, m.y, gsize[m.x], s.kv.partials};
    solve_mixed<BS>(s.A, s.mf, s.mg, s.kv, s.a, s.ds, gb);
}

// Mixed-solver setup: FP32 values of the matrix and their compact index
// bytes (quad layout, padded to a multiple of four entries with value 0 and
// index 0), the row's three range starts, FP32 diagonal and inverse
// diagonal.  A row whose column lies 64 or more slots into its range keeps
// the int32 columns (sell_row = 1).
__global__ void k_mixed_setup(Consts c, Ppe A, MatFree mf, Krylov kv, const int32_t* __restrict__ ids,
                              int warm, unsigned long long* __restrict__ sym_fp) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long fp = 0;  // this row's terms of the symmetry fingerprint (over slots)
    if (k < c.n) {
        const double d = A.diag[k];
        A.rsum32[k] = f32(A.rsum[k]);
        // initial guess: the particle's solution of the last solve (rows without
        // an unknown stay 0, as the zero start leaves them)
        if (warm) kv.x[k] = d > 0.0 ? kv.x_prev[ids[k]] : 0.0;
        A.diag32[k] = f32(d);
        kv.inv_diag32[k] = d != 0.0 ? f32(ddiv(1.0, d)) : 1.f;
        const size_t base = (size_t)(k >> 5) * c.K * 32 + (k & 31);
        const int w = A.slice_w[k >> 5];
        const int wq = (w + 3) & ~3;
        const int cnt = A.offcnt[k];
        int8_t sell = 1;
        int st[3] = {0, 0, 0};
        if (mf.enabled) {
            sell = 0;
            const int32_t key = mf.skey[k];
            if (key < c.nkeys) {
                const int ix = key / c.numY, iy = key - ix * c.numY;
                for (int r = 0; r < 3; r++) st[r] = mf.cs[(ix - 1 + r) * c.numY + iy - 1];
            }
            for (int r = 0; r < 3; r++) mf.rs[(size_t)r * mf.rs_stride + k] = st[r];
        }
        // four entries per pass: one 16-byte value word and one 4-byte word
        // of index bytes (padding: range 0, offset 0, value 0)
        for (int m0 = 0; m0 < wq; m0 += 4) {
            float v4[4];
            uint32_t b4 = 0;
#pragma unroll
            for (int t = 0; t < 4; t++) {
                const int m = m0 + t;
                const size_t e = base + (size_t)m * 32;
                const double v = m < w ? A.val[e] : 0.0;
                v4[t] = m < w ? f32(v) : 0.f;
                if (m < cnt) {
                    const int j = A.col[e];
                    fp += entry_term(k, j, v);
                    if (mf.enabled) {
                        int r = 2;
                        while (r > 0 && j < st[r]) r--;
                        const int off = j - st[r];
                        if (off >= 0 && off < 64)
                            b4 |= (uint32_t)((r << 6) | off) << (8 * t);
                        else
                            sell = 1;
                    }
                }
            }
            const size_t q = qsell_index(k, m0, c.K);  // a multiple of 4
            reinterpret_cast<float4*>(A.val32)[q >> 2] = make_float4(v4[0], v4[1], v4[2], v4[3]);
            if (mf.enabled) reinterpret_cast<uint32_t*>(mf.idx8)[q >> 2] = b4;
        }
        mf.sell_row[k] = sell;
    }
    fp = warp_sum64(fp);
    if ((threadIdx.x & 31) == 0 && fp) atomicAdd(sym_fp, fp);
}

// Co-resident blocks of a persistent kernel (0 if the configuration does not
// fit, which the launchers report instead of launching).  A kernel that asks
// for dynamic shared memory opts in to it first.
int coop_grid(const void* fn, int device, int block, size_t smem, int max_per_sm) {
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (smem > 0) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, block, smem) != cudaSuccess) {
        cudaGetLastError();
        per = 0;
    }
    return sms * std::min(per, max_per_sm);
}

SolveArgs make_args(const Consts& c, double tol, int64_t max_iter) {
    SolveArgs a;
    a.n = c.n;
    a.nslices = (c.n + 31) / 32;
    a.K = c.K;
    a.tol = tol;
    a.max_iter = max_iter;
    // An inner solve's residual reduction: with the operator in difference
    // form one refinement reaches ~1e-5 of its start on the 1M-particle dam
    // break (FP32 vectors); asking for more costs iterations that the next
    // refinement's FP64 residual does not see.
    a.inner_tol = 1e-5;
    a.max_refine = 40;
    a.warm = 0;
    return a;
}

}  // namespace

void solver_setup(Krylov& k, int32_t /*n_pad*/, int device) {
    int g1 = coop_grid((const void*)k_cg64, device, kBlock, 0, 1);
    int g2 = coop_grid((const void*)k_cg_mixed, device, kMixedBlock, 0, 1);
    int g3 = coop_grid((const void*)k_cg_mixed_ov, device, kMixedBlock, 0, 1);
    k.grid = std::min({g1, g2, g3});
    k.block = kBlock;
}

void launch_mixed_setup(const Consts& c, const SortScratch& sc, const Ppe& A, MatFree& mf,
                        const Krylov& k, const int32_t* ids, bool warm, DevStats* ds, cudaStream_t st) {
    mf.skey = sc.skey;
    mf.cs = sc.cell_start;
    mf.numY = c.numY;
    mf.nkeys = c.nkeys;
    k_mixed_setup<<<(c.n + 255) / 256, 256, 0, st>>>(c, A, mf, k, ids, warm ? 1 : 0, &ds->sym_fp);
    ++g_launches;
}

void launch_solve_fp64(const Consts& c, const Ppe& A, const Krylov& k, double tol,
                       int64_t max_iter, DevStats* ds, cudaStream_t st) {
    SolveArgs a = make_args(c, tol, max_iter);
    Ppe AA = A;
    Krylov kk = k;
    void* args[] = {&AA, &kk, &a, &ds};
    cudaMemsetAsync(k.barrier, 0, sizeof(unsigned int), st);
    cudaLaunchCooperativeKernel((const void*)k_cg64, dim3(k.grid), dim3(kBlock), args, 0, st);
    ++g_launches;
}

// Self-test of the bounded waits: the solver's grid barrier in a group that
// counts one block more than the launch has, so no block can pass.  Every
// block gives up (at its spin limit, here 2^16 polls instead of the solver's
// 2^23, or on the flag of the first that did), records it and ends; nothing
// faults and nothing is left waiting.
namespace {
__global__ void k_selftest_barrier(unsigned int* words, DevStats* ds) {
    GridBar gb{words, 0u, 0, (int)blockIdx.x, (int)gridDim.x + 1, nullptr, 1ll << 16};
    const bool ok = grid_sync(gb, ds);
    if (threadIdx.x == 0 && !ok) atomicAdd(words + 1, 1u);
}
}  // namespace

int selftest_wait_limit(int blocks, int* gave_up, int* status, float* ms) {
    unsigned int* words = nullptr;
    DevStats* ds = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = 0;
    if (cudaMalloc(&words, 2 * sizeof(unsigned int)) != cudaSuccess ||
        cudaMalloc(&ds, sizeof(DevStats)) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess) {
        rc = -1;
    } else {
        cudaMemset(words, 0, 2 * sizeof(unsigned int));
        cudaMemset(ds, 0, sizeof(DevStats));
        cudaEventRecord(e0);
        k_selftest_barrier<<<blocks, 64>>>(words, ds);
        cudaEventRecord(e1);
        unsigned int h[2] = {0, 0};
        DevStats hs{};
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess ||
            cudaMemcpy(h, words, sizeof h, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(&hs, ds, sizeof hs, cudaMemcpyDeviceToHost) != cudaSuccess) {
            rc = -1;
        } else {
            *gave_up = (int)h[1];
            *status = hs.status;
            cudaEventElapsedTime(ms, e0, e1);
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(words);
    cudaFree(ds);
    return rc;
}

// ----------------------------------------------------------- batched solve
namespace {
template <int BS, int MINB>
int resident_grid(int device) {
    return coop_grid((const void*)k_cg_mixed_batched<BS, MINB>, device, BS, 0, MINB);
}
}  // namespace

int batch_resident_grid(int block, int device) {
    switch (block) {
        case 256: return resident_grid<256, 4>(device);
        case 512: return resident_grid<512, 2>(device);
        case 1024: return resident_grid<1024, 1>(device);
        default: return 0;
    }
}

void batch_group_sizes(const std::vector<int32_t>& rows, double alpha, int grid,
                       std::vector<int32_t>& out) {
    const int ns = (int)rows.size();
    out.assign(ns, 1);
    std::vector<double> w(ns);
    double tot = 0.0;
    for (int s = 0; s < ns; s++) tot += (w[s] = std::pow((double)std::max(rows[s], 1), alpha));
    int used = 0;
    std::vector<std::pair<double, int>> frac;
    for (int s = 0; s < ns; s++) {
        const double want = grid * w[s] / tot;
        out[s] = std::max(1, (int)want);
        used += out[s];
        frac.push_back({want - (int)want, s});
    }
    std::sort(frac.begin(), frac.end(), [](auto& a, auto& b) { return a.first > b.first; });
    for (size_t k = 0; used < grid && k < frac.size(); k++, used++) out[frac[k].second]++;
    while (used > grid) {  // the floor of 1 block per scene overshot: trim the largest
        int big = 0;
        for (int s = 1; s < ns; s++)
            if (out[s] > out[big]) big = s;
        if (out[big] <= 1) break;
        out[big]--;
        used--;
    }
}

int batch_solve_setup(const std::vector<BatchScene>& scenes, int block, double alpha, int device,
                      BatchSolve& b) {
    batch_solve_free(b);
    const int ns = (int)scenes.size();
    const int grid = batch_resident_grid(block, device);
    if (grid < ns || ns == 0) return 1;
    std::vector<int32_t> rows(ns), gs;
    for (int s = 0; s < ns; s++) rows[s] = scenes[s].c.n;
    batch_group_sizes(rows, alpha, grid, gs);
    std::vector<SceneSolve> hs(ns);
    std::vector<int2> bmap;
    for (int s = 0; s < ns; s++) {
        const BatchScene& q = scenes[s];
        SolveArgs a = make_args(q.c, q.tol, q.max_iter);
        a.warm = q.warm ? 1 : 0;
        hs[s] = SceneSolve{q.A, q.mf, q.mg, q.kv, a, q.ds};
        for (int r = 0; r < gs[s]; r++) bmap.push_back(make_int2(s, r));
    }
    if (cudaMalloc(&b.scenes, sizeof(SceneSolve) * ns) != cudaSuccess ||
        cudaMalloc(&b.bmap, sizeof(int2) * bmap.size()) != cudaSuccess ||
        cudaMalloc(&b.gsize, sizeof(int32_t) * ns) != cudaSuccess ||
        cudaMalloc(&b.bars, sizeof(unsigned int) * 32 * ns) != cudaSuccess) {
        batch_solve_free(b);
        return 2;
    }
    cudaMemcpy(b.scenes, hs.data(), sizeof(SceneSolve) * ns, cudaMemcpyHostToDevice);
    cudaMemcpy(b.bmap, bmap.data(), sizeof(int2) * bmap.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(b.gsize, gs.data(), sizeof(int32_t) * ns, cudaMemcpyHostToDevice);
    b.n_scenes = ns;
    b.block = block;
    b.grid = (int32_t)bmap.size();
    b.alpha = alpha;
    b.group_blocks = gs;
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

void batch_solve_free(BatchSolve& b) {
    if (b.scenes) cudaFree(b.scenes);
    if (b.bmap) cudaFree(b.bmap);
    if (b.gsize) cudaFree(b.gsize);
    if (b.bars) cudaFree(b.bars);
    b = BatchSolve{};
}

void launch_solve_mixed_batched(const BatchSolve& b, cudaStream_t st) {
    const SceneSolve* sc = (const SceneSolve*)b.scenes;
    const int2* bm = b.bmap;
    const int32_t* gs = b.gsize;
    unsigned int* bars = b.bars;
    void* args[] = {&sc, &bm, &gs, &bars};
    cudaMemsetAsync(b.bars, 0, sizeof(unsigned int) * 32 * b.n_scenes, st);
    const void* fn = b.block == 256   ? (const void*)k_cg_mixed_batched<256, 4>
                     : b.block == 512 ? (const void*)k_cg_mixed_batched<512, 2>
                                      : (const void*)k_cg_mixed_batched<1024, 1>;
    cudaLaunchCooperativeKernel(fn, dim3(b.grid), dim3(b.block), args, 0, st);
    ++g_launches;
}

void launch_solve_mixed(const Consts& c, const Ppe& A, const MatFree& mf, const Mg& mg,
                        const Krylov& k, double tol, int64_t max_iter, bool warm, DevStats* ds,
                        cudaStream_t st) {
    SolveArgs a = make_args(c, tol, max_iter);
    a.warm = warm ? 1 : 0;
    Ppe AA = A;
    MatFree mm = mf;
    Mg gg = mg;
    Krylov kk = k;
    void* args[] = {&AA, &mm, &gg, &kk, &a, &ds};
    cudaMemsetAsync(k.barrier, 0, sizeof(unsigned int), st);
    const bool ov = mg.enabled && mg.overlap;
    const void* fn = ov ? (const void*)k_cg_mixed_ov : (const void*)k_cg_mixed;
    cudaLaunchCooperativeKernel(fn, dim3(k.grid), dim3(kMixedBlock), args, 0, st);
    ++g_launches;
}

}  // namespace mpsg
