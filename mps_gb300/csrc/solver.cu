// Pressure Poisson solve (src/mps.cpp:417-470).
//
// Both solvers are single persistent cooperative kernels: one launch per
// solve, the blocks stay resident and meet at a grid barrier between the
// phases of an iteration, and the convergence test runs on the device, so no
// host round trip is needed per iteration.  Every block reduces the per-block
// partial sums of a dot product in the same fixed order, so all blocks take
// the same branch and the result is run-to-run deterministic.
//
//  * FP64: the Jacobi-preconditioned CG that Eigen::ConjugateGradient runs
//    with its defaults (zero start, tolerance on the recursive residual
//    ||r||^2 < max(tol^2 ||b||^2, DBL_MIN), cap 2n), over the SELL-32 FP64
//    matrix.  Roofline: HBM (12 B per stored entry per iteration) and FP64
//    issue (one DFMA per entry).
//  * MIXED: iterative refinement.  The residual r = b - A x and the solution
//    x stay FP64 (FP64 matrix); each correction A d = r is solved by Jacobi
//    CG on the FP32 copy of the matrix with FP32 vectors and FP64-accurate
//    dot products (error-free FP32 products, compensated per thread, FP64
//    across threads and blocks).
#include <cfloat>
#include <cstdio>

#include "devutil.cuh"
#include "engine.cuh"

namespace mpsg {

namespace {

constexpr int kBlock = 256;
constexpr int kWarps = kBlock / 32;
constexpr long long kBarrierSpinLimit = 1ll << 24;  // ~1 s with the back-off below

struct SolveArgs {
    int32_t n;          // rows (slots)
    int32_t nslices;
    int32_t K;
    double tol;
    int64_t max_iter;
    double inner_tol;
    int32_t max_refine;
};

// Grid barrier with a bounded wait: the blocks of a cooperative launch are
// co-resident, so it always completes; if it somehow does not, the waiting
// block raises ST_TIMEOUT and every block leaves at its next check.
__device__ __forceinline__ bool grid_sync(unsigned int* bar, DevStats* ds) {
    __syncthreads();
    __shared__ int s_abort;
    if (threadIdx.x == 0) {
        volatile unsigned int* vgen = bar + 1;
        unsigned int gen = *vgen;
        __threadfence();
        unsigned int arrived = atomicAdd(bar, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long long it = 0;
            while (*vgen == gen) {
                if (++it > kBarrierSpinLimit) {
                    atomicOr(&ds->status, ST_TIMEOUT);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        s_abort = (*(volatile int*)&ds->status & ST_TIMEOUT) != 0;
    }
    __syncthreads();
    return s_abort == 0;
}

// Block-level sum of up to 3 doubles; writes partials[slot * G + block].
template <int M>
__device__ __forceinline__ void block_partials(double (&v)[M], double* partials) {
    __shared__ double sh[M][kWarps];
#pragma unroll
    for (int m = 0; m < M; m++) {
        double x = v[m];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0) sh[m][threadIdx.x >> 5] = x;
    }
    __syncthreads();
    if (threadIdx.x < M) {
        double s = 0.0;
        for (int w = 0; w < kWarps; w++) s += sh[threadIdx.x][w];
        partials[threadIdx.x * gridDim.x + blockIdx.x] = s;
    }
    __syncthreads();
}

// Every block sums the G partials of slot m in the same order (deterministic).
template <int M>
__device__ __forceinline__ void grid_totals(const double* partials, double (&out)[M]) {
    __shared__ double sh[M][kWarps];
    const int G = gridDim.x;
#pragma unroll
    for (int m = 0; m < M; m++) {
        double x = 0.0;
        for (int b = threadIdx.x; b < G; b += blockDim.x) x += __ldcg(partials + m * G + b);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0) sh[m][threadIdx.x >> 5] = x;
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < M; m++) {
        double s = 0.0;
        for (int w = 0; w < kWarps; w++) s += sh[m][w];
        out[m] = s;
    }
    __syncthreads();
}

// y = A x for the rows of slice `sl`, lane `lane` (FP64 SELL-32).
__device__ __forceinline__ double spmv64_row(const Ppe& A, int K, int sl, int lane, int row,
                                             const double* __restrict__ x, double xi) {
    const int w = A.slice_w[sl];
    const size_t base = (size_t)sl * K * 32 + lane;
    const int cnt = A.offcnt[row];
    double s = 0.0;
    for (int m = 0; m < w; m++) {
        int col = __ldg(A.col + base + (size_t)m * 32);
        double v = __ldg(A.val + base + (size_t)m * 32);
        if (m < cnt) s = fma(v, __ldcg(x + col), s);
    }
    return fma(A.diag[row], xi, s);
}

__device__ __forceinline__ float spmv32_row(const Ppe& A, int K, int sl, int lane, int row,
                                            const float* __restrict__ x, float xi, int cnt) {
    const int w = A.slice_w[sl];
    const size_t base = (size_t)sl * K * 32 + lane;
    float s = 0.f;
    for (int m = 0; m < w; m++) {
        int col = __ldg(A.col + base + (size_t)m * 32);
        float v = __ldg(A.val32 + base + (size_t)m * 32);
        if (m < cnt) s = fmaf(v, __ldcg(x + col), s);
    }
    return fmaf(A.diag32[row], xi, s);
}

// ----------------------------------------------------------------- FP64 CG
__global__ void __launch_bounds__(kBlock) k_cg64(Consts c, Ppe A, Krylov kv, SolveArgs a,
                                                 DevStats* ds) {
    const int lane = threadIdx.x & 31;
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    unsigned int* bar = kv.barrier;
    double* P = kv.partials;

    // setup: x = 0, r = b, inv_diag, ||b||^2
    double acc[1] = {0.0};
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
    block_partials<1>(acc, P);
    if (!grid_sync(bar, ds)) return;
    double tot[1];
    grid_totals<1>(P, tot);
    const double rhs2 = tot[0];
    int64_t it = 0;
    double rn2 = rhs2;
    if (rhs2 == 0.0) {
        rn2 = 0.0;
    } else {
        const double thr = fmax(a.tol * a.tol * rhs2, DBL_MIN);
        if (!(rn2 < thr)) {
            // p = M^-1 r, absNew = r.p
            double a1[1] = {0.0};
            for (int sl = gwarp; sl < a.nslices; sl += nwarps) {
                int i = sl * 32 + lane;
                if (i >= a.n) continue;
                double r = kv.r[i];
                double p = kv.inv_diag[i] * r;
                kv.p[i] = p;
                a1[0] = fma(r, p, a1[0]);
            }
            block_partials<1>(a1, P + 1 * gridDim.x);
            if (!grid_sync(bar, ds)) return;
            double t1[1];
            grid_totals<1>(P + 1 * gridDim.x, t1);
            double abs_new = t1[0];
            while (it < a.max_iter) {
                // q = A p ; p.q
                double a2[1] = {0.0};
                for (int sl = gwarp; sl < a.nslices; sl += nwarps) {
                    int i = sl * 32 + lane;
                    if (i >= a.n) continue;
                    double pi = kv.p[i];
                    double q = spmv64_row(A, a.K, sl, lane, i, kv.p, pi);
                    kv.q[i] = q;
                    a2[0] = fma(pi, q, a2[0]);
                }
                block_partials<1>(a2, P + 2 * gridDim.x);
                if (!grid_sync(bar, ds)) return;
                double t2[1];
                grid_totals<1>(P + 2 * gridDim.x, t2);
                const double alpha = abs_new / t2[0];
                // x += alpha p ; r -= alpha q ; z = M^-1 r ; ||r||^2, r.z
                double a3[2] = {0.0, 0.0};
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
                block_partials<2>(a3, P + 3 * gridDim.x);
                if (!grid_sync(bar, ds)) return;
                double t3[2];
                grid_totals<2>(P + 3 * gridDim.x, t3);
                rn2 = t3[0];
                if (rn2 < thr) break;
                const double abs_old = abs_new;
                abs_new = t3[1];
                const double beta = abs_new / abs_old;
                for (int sl = gwarp; sl < a.nslices; sl += nwarps) {
                    int i = sl * 32 + lane;
                    if (i >= a.n) continue;
                    kv.p[i] = fma(beta, kv.p[i], kv.z[i]);
                }
                it++;
                if (!grid_sync(bar, ds)) return;
            }
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ds->cg_iterations = it;
        ds->refinements = 0;
        ds->cg_rel_residual = rhs2 > 0.0 ? sqrt(rn2 / rhs2) : 0.0;
    }
}

// --------------------------------------------------------------- mixed IR
// Error-free FP32 product accumulated with compensation: (hi, lo) pairs.
struct F2 {
    float hi, lo;
};
__device__ __forceinline__ void acc_prod(F2& a, float x, float y) {
    float p = x * y;
    float e = fmaf(x, y, -p);
    float s = a.hi + p;
    float bb = s - a.hi;
    float err = (a.hi - (s - bb)) + (p - bb);
    a.hi = s;
    a.lo += err + e;
}
__device__ __forceinline__ double f2d(const F2& a) { return (double)a.hi + (double)a.lo; }

__global__ void __launch_bounds__(kBlock) k_cg_mixed(Consts c, Ppe A, Krylov kv, SolveArgs a,
                                                     DevStats* ds) {
    const int lane = threadIdx.x & 31;
    const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    unsigned int* bar = kv.barrier;
    double* P = kv.partials;
    const int G = gridDim.x;

    // setup: x = 0, ||b||^2 (the FP32 matrix copy is made by k_to_fp32)
    double acc[1] = {0.0};
    for (int sl = gwarp; sl < a.nslices; sl += nwarps) {
        int i = sl * 32 + lane;
        if (i >= a.n) continue;
        kv.x[i] = 0.0;
        double b = A.src[i];
        acc[0] = fma(b, b, acc[0]);
    }
    block_partials<1>(acc, P);
    if (!grid_sync(bar, ds)) return;
    double tot[1];
    grid_totals<1>(P, tot);
    const double rhs2 = tot[0];
    int64_t inner_total = 0;
    int refine = 0;
    double rn2 = rhs2;
    const double thr = fmax(a.tol * a.tol * rhs2, DBL_MIN);
    while (rhs2 > 0.0 && refine <= a.max_refine) {
        // FP64 residual r = b - A x and its norm
        double a0[1] = {0.0};
        for (int sl = gwarp; sl < a.nslices; sl += nwarps) {
            int i = sl * 32 + lane;
            if (i >= a.n) continue;
            double r = A.src[i] - spmv64_row(A, a.K, sl, lane, i, kv.x, kv.x[i]);
            kv.r[i] = r;
            a0[0] = fma(r, r, a0[0]);
        }
        block_partials<1>(a0, P + 1 * G);
        if (!grid_sync(bar, ds)) return;
        double t0[1];
        grid_totals<1>(P + 1 * G, t0);
        rn2 = t0[0];
        if (rn2 < thr || refine == a.max_refine || inner_total >= a.max_iter) break;
        refine++;
        // inner Jacobi-CG on the FP32 matrix for A d = r (scaled to unit norm)
        const float scale = (float)(1.0 / sqrt(rn2));
        F2 s1 = {0.f, 0.f};
        for (int sl = gwarp; sl < a.nslices; sl += nwarps) {
            int i = sl * 32 + lane;
            if (i >= a.n) continue;
            float r = (float)(kv.r[i]) * scale;
            float p = kv.inv_diag32[i] * r;
            kv.r32[i] = r;
            kv.p32[i] = p;
            kv.x32[i] = 0.f;
            acc_prod(s1, r, p);
        }
        double v1[1] = {f2d(s1)};
        block_partials<1>(v1, P + 2 * G);
        if (!grid_sync(bar, ds)) return;
        double t1[1];
        grid_totals<1>(P + 2 * G, t1);
        double abs_new = t1[0];
        const double r0n2 = 1.0;  // the scaled residual has unit norm
        const double ithr = a.inner_tol * a.inner_tol * r0n2;
        int64_t k = 0;
        while (inner_total + k < a.max_iter) {
            F2 s2 = {0.f, 0.f};
            for (int sl = gwarp; sl < a.nslices; sl += nwarps) {
                int i = sl * 32 + lane;
                if (i >= a.n) continue;
                float pi = kv.p32[i];
                float q = spmv32_row(A, a.K, sl, lane, i, kv.p32, pi, A.offcnt[i]);
                kv.q32[i] = q;
                acc_prod(s2, pi, q);
            }
            double v2[1] = {f2d(s2)};
            block_partials<1>(v2, P + 3 * G);
            if (!grid_sync(bar, ds)) return;
            double t2[1];
            grid_totals<1>(P + 3 * G, t2);
            const float alpha = (float)(abs_new / t2[0]);
            F2 s3a = {0.f, 0.f}, s3b = {0.f, 0.f};
            for (int sl = gwarp; sl < a.nslices; sl += nwarps) {
                int i = sl * 32 + lane;
                if (i >= a.n) continue;
                kv.x32[i] = fmaf(alpha, kv.p32[i], kv.x32[i]);
                float r = fmaf(-alpha, kv.q32[i], kv.r32[i]);
                kv.r32[i] = r;
                float z = kv.inv_diag32[i] * r;
                kv.z32[i] = z;
                acc_prod(s3a, r, r);
                acc_prod(s3b, r, z);
            }
            double v3[2] = {f2d(s3a), f2d(s3b)};
            block_partials<2>(v3, P + 4 * G);
            if (!grid_sync(bar, ds)) return;
            double t3[2];
            grid_totals<2>(P + 4 * G, t3);
            k++;
            if (t3[0] < ithr) break;
            const double abs_old = abs_new;
            abs_new = t3[1];
            const float beta = (float)(abs_new / abs_old);
            for (int sl = gwarp; sl < a.nslices; sl += nwarps) {
                int i = sl * 32 + lane;
                if (i >= a.n) continue;
                kv.p32[i] = fmaf(beta, kv.p32[i], kv.z32[i]);
            }
            if (!grid_sync(bar, ds)) return;
        }
        inner_total += k;
        // x += d (FP64)
        const double inv_scale = sqrt(rn2);
        for (int sl = gwarp; sl < a.nslices; sl += nwarps) {
            int i = sl * 32 + lane;
            if (i >= a.n) continue;
            kv.x[i] = fma((double)kv.x32[i], inv_scale, kv.x[i]);
        }
        if (!grid_sync(bar, ds)) return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        ds->cg_iterations = inner_total;
        ds->refinements = refine;
        ds->cg_rel_residual = rhs2 > 0.0 ? sqrt(rn2 / rhs2) : 0.0;
    }
}

// FP32 copy of the FP64 matrix and of the inverse diagonal (before the solve).
__global__ void k_to_fp32(Ppe A, Krylov kv, int n, int K) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ((n + 31) & ~31)) return;
    int sl = i >> 5, lane = i & 31;
    const int w = A.slice_w[sl];
    const size_t base = (size_t)sl * K * 32 + lane;
    for (int m = 0; m < w; m++) A.val32[base + (size_t)m * 32] = (float)A.val[base + (size_t)m * 32];
    if (i >= n) return;
    double d = A.diag[i];
    A.diag32[i] = (float)d;
    kv.inv_diag32[i] = d != 0.0 ? (float)(1.0 / d) : 1.f;
}

int coop_grid(const void* fn, int device) {
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, kBlock, 0);
    if (per < 1) per = 1;
    if (per > 4) per = 4;
    return sms * per;
}

}  // namespace

void solver_setup(Krylov& k, int32_t /*n_pad*/, int device) {
    int g1 = coop_grid((const void*)k_cg64, device);
    int g2 = coop_grid((const void*)k_cg_mixed, device);
    k.grid = g1 < g2 ? g1 : g2;
    k.block = kBlock;
}

static SolveArgs make_args(const Consts& c, double tol, int64_t max_iter) {
    SolveArgs a;
    a.n = c.n;
    a.nslices = (c.n + 31) / 32;
    a.K = c.K;
    a.tol = tol;
    a.max_iter = max_iter;
    a.inner_tol = 1e-4;
    a.max_refine = 30;
    return a;
}

void launch_solve_fp64(const Consts& c, const Ppe& A, const Krylov& k, double tol,
                       int64_t max_iter, DevStats* ds, cudaStream_t st) {
    SolveArgs a = make_args(c, tol, max_iter);
    Consts cc = c;
    Ppe AA = A;
    Krylov kk = k;
    void* args[] = {&cc, &AA, &kk, &a, &ds};
    cudaMemsetAsync(k.barrier, 0, 2 * sizeof(unsigned int), st);
    cudaLaunchCooperativeKernel((const void*)k_cg64, dim3(k.grid), dim3(kBlock), args, 0, st);
    ++g_launches;
}

void launch_solve_mixed(const Consts& c, const Ppe& A, const Krylov& k, double tol,
                        int64_t max_iter, DevStats* ds, cudaStream_t st) {
    SolveArgs a = make_args(c, tol, max_iter);
    Consts cc = c;
    Ppe AA = A;
    Krylov kk = k;
    void* args[] = {&cc, &AA, &kk, &a, &ds};
    k_to_fp32<<<(c.n + 31 + 255) / 256, 256, 0, st>>>(A, k, c.n, c.K);
    ++g_launches;
    cudaMemsetAsync(k.barrier, 0, 2 * sizeof(unsigned int), st);
    cudaLaunchCooperativeKernel((const void*)k_cg_mixed, dim3(k.grid), dim3(kBlock), args, 0, st);
    ++g_launches;
}

}  // namespace mpsg
