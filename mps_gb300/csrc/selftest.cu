// Device self-check of the integer-pipe FP64 square root and division
// (exact64.cuh) against the GPU's FP64 instruction sequences (__dsqrt_rn,
// __ddiv_rn), on seeded inputs: random significands and exponents, the
// significands next to 2^52 and 2^53 whose roots and quotients sit next to a
// midpoint, equal and adjacent significands, and the operand ranges of the
// neighbour sweeps (squared distances and radii of 1e-4..1e1).
#include <cuda_runtime.h>

#include <string>

#include "devutil.cuh"
#include "engine_impl.cuh"

namespace mpsg {

namespace {

__device__ __forceinline__ uint64_t splitmix(uint64_t z) {
    // SplitMix64 (Steele, Lea and Flood, 2014)
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ uint64_t test_mant(uint64_t r) {
    switch (r & 7) {
        case 0: return (r >> 8) & 0xff;
        case 1: return x64::kMant - ((r >> 8) & 0xff);
        case 2: return ((r >> 8) & 0xffff) << 36;
        default: return r >> 12;
    }
}

// counts[0]: square-root mismatches, [1]: quotient mismatches, [2]/[3]: the
// cases that took the integer path, [4]: mismatches of the exact subtraction
// of 1, the FP32 rounding and the comparison shortcut; bad[0..2]: the first
// square-root or quotient mismatch's operands (x or a, b) in bit form,
// claimed once.
__global__ void k_exact64_check(uint64_t n, uint64_t seed, unsigned long long* counts,
                                unsigned long long* bad) {
    unsigned long long mis_s = 0, mis_d = 0, fast_s = 0, fast_d = 0, mis_o = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r0 = splitmix(seed ^ (i * 0xD1B54A32D192ED03ull));
        const uint64_t r1 = splitmix(r0), r2 = splitmix(r1), r3 = splitmix(r2);
        double x, a, b;
        if ((r3 & 3) == 0) {
            // the sweeps' ranges: squared distances, radii and distances
            x = 1e-8 + (double)(r0 >> 11) * 0x1p-53 * 1e-2;
            a = 1e-4 + (double)(r1 >> 11) * 0x1p-53 * 1e1;
            b = 1e-4 + (double)(r2 >> 11) * 0x1p-53 * 1e1;
        } else {
            x = x64::double_of(((uint64_t)(1 + (r0 >> 53) % 2046) << 52) | (test_mant(r1) & x64::kMant));
            const uint64_t ea = 1 + (r2 >> 53) % 2046;
            int64_t eb = (int64_t)ea + (int64_t)((r3 >> 40) % 201) - 100;
            eb = eb < 1 ? 1 : (eb > 2046 ? 2046 : eb);
            const uint64_t ma = test_mant(r2), mb = (r3 & 12) == 0 ? ma : test_mant(r3 >> 4);
            a = x64::double_of((ea << 52) | (ma & x64::kMant) | ((r1 & 1) << 63));
            b = x64::double_of(((uint64_t)eb << 52) | (mb & x64::kMant) | ((r1 & 2) << 62));
        }
        double got;
        // the exact subtraction of 1, FP32 rounding and ordering shortcut
        const double q = 1.0 + (double)(r0 >> 11) * 0x1p-53 * 64.0;
        double q1;
        float f;
        if (!x64::sub_one(q, q1) || x64::bits_of(q1) != x64::bits_of(__dsub_rn(q, 1.0))) mis_o++;
        if (x64::to_f32(a, f) && __float_as_uint(f) != __float_as_uint(__double2float_rn(a))) mis_o++;
        if (x64::lt_cut(fabs(a), fabs(b)) != (fabs(a) < fabs(b))) mis_o++;
        if (x64::sqrt_rn<Fp32Approx>(x, got)) {
            fast_s++;
            if (x64::bits_of(got) != x64::bits_of(__dsqrt_rn(x))) {
                mis_s++;
                if (atomicCAS(bad + 3, 0ull, 1ull) == 0ull) {
                    bad[0] = x64::bits_of(x);
                    bad[1] = 0;
                    bad[2] = 1;
                }
            }
        }
        if (x64::div_rn<Fp32Approx>(a, b, got)) {
            fast_d++;
            if (x64::bits_of(got) != x64::bits_of(__ddiv_rn(a, b))) {
                mis_d++;
                if (atomicCAS(bad + 3, 0ull, 1ull) == 0ull) {
                    bad[0] = x64::bits_of(a);
                    bad[1] = x64::bits_of(b);
                    bad[2] = 2;
                }
            }
        }
    }
    if (mis_o) atomicAdd(counts + 4, mis_o);
    if (mis_s) atomicAdd(counts + 0, mis_s);
    if (mis_d) atomicAdd(counts + 1, mis_d);
    atomicAdd(counts + 2, fast_s);
    atomicAdd(counts + 3, fast_d);
}

}  // namespace

}  // namespace mpsg

extern "C" int mps_selftest_exact64(uint64_t n, uint64_t seed, uint64_t* result) {
    using namespace mpsg;
    if (!result) {
        set_last_error("mps_selftest_exact64: null result");
        return MPS_ERR_ARG;
    }
    unsigned long long* d = nullptr;
    cudaError_t ce = cudaMalloc(&d, 9 * sizeof(unsigned long long));
    if (ce == cudaSuccess) ce = cudaMemset(d, 0, 9 * sizeof(unsigned long long));
    if (ce == cudaSuccess) {
        k_exact64_check<<<4 * 152, 256>>>(n, seed, d, d + 5);
        ce = cudaGetLastError();
    }
    unsigned long long h[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (ce == cudaSuccess) ce = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
    if (d) cudaFree(d);
    if (ce != cudaSuccess) {
        set_last_error(std::string("mps_selftest_exact64: ") + cudaGetErrorString(ce));
        return MPS_ERR_CUDA;
    }
    // result: sqrt/div mismatches, fast counts, first bad (3), other mismatches
    for (int k = 0; k < 4; k++) result[k] = h[k];
    for (int k = 0; k < 3; k++) result[4 + k] = h[5 + k];
    result[7] = h[4];
    return MPS_OK;
}
