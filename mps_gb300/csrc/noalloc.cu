// mps_number_density_static: the initial particle-number-density pass of
// MPS::loadInitialState (neighbour search + number density ratio) for callers
// that cannot allocate device memory, working entirely in a fixed scratch
// area that lives in this library's static device memory.
//
// Who needs it: a host application that owns every byte of device memory
// itself (a pre-reserved budget or its own pool) and does not let libraries
// call cudaMalloc/cudaFree, and timing-critical loops where an allocation's
// implicit device synchronisation is not acceptable.  mps_create() allocates
// its buffers once per scene; this entry point allocates nothing: the caller
// passes device pointers for the inputs and the output, and the scratch is
// the file-scope array below.
//
// Limits and behaviour:
//  * at most kMaxParticles particles and kMaxCells bucket cells
//    (numX * numY * numZ of the reference's Bucket); larger requests, and a
//    non-finite or inverted domain (max < min on an axis), return
//    MPS_ERR_ARG without touching the GPU;
//  * the scratch array is resident on every GPU that loads the library, for
//    the life of the process (about 5 MB);
//  * the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current) and caches it for the
//    life of the process; make that first call before any stream capture.
//    The cached address belongs to the device's primary context: after
//    cudaDeviceReset (or anything else that destroys that context) it is
//    stale, so this entry point must not be called again in that process;
//  * every call reuses the same scratch and keeps nothing between calls (the
//    cell counters are cleared on each call); calls whose work overlaps on
//    the GPU race on the scratch, so issue them on one stream or order them;
//  * results are bit-identical to the number density ratios mps_create
//    computes (the same FP64 operation order), including Ghost particles
//    (ratio 0); a particle with a non-finite position gets ratio NaN and is
//    left out of the other particles' neighbourhoods.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <limits>
#include <mutex>
#include <string>

#include "../../include/mps_gb300.h"
#include "devutil.cuh"
#include "engine.cuh"
#include "engine_impl.cuh"

using namespace mpsg;

namespace {

constexpr int32_t kMaxParticles = 1 << 16;
constexpr int32_t kMaxCells = 1 << 18;
constexpr size_t kScanTmpInts = (size_t)(kMaxCells + 2) / 2048 + 64;

// scratch layout (byte offsets, each 256-aligned)
constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kOffCount = 0;
constexpr size_t kOffStart = kOffCount + align256(sizeof(int32_t) * (kMaxCells + 2));
constexpr size_t kOffKey = kOffStart + align256(sizeof(int32_t) * (kMaxCells + 2));
constexpr size_t kOffRank = kOffKey + align256(sizeof(int32_t) * kMaxParticles);
constexpr size_t kOffPerm = kOffRank + align256(sizeof(int32_t) * kMaxParticles);
constexpr size_t kOffId = kOffPerm + align256(sizeof(int32_t) * kMaxParticles);
constexpr size_t kOffSkey = kOffId + align256(sizeof(int32_t) * kMaxParticles);
constexpr size_t kOffX = kOffSkey + align256(sizeof(int32_t) * kMaxParticles);
constexpr size_t kOffY = kOffX + align256(sizeof(double) * kMaxParticles);
constexpr size_t kOffZ = kOffY + align256(sizeof(double) * kMaxParticles);
constexpr size_t kOffScan = kOffZ + align256(sizeof(double) * kMaxParticles);
constexpr size_t kScratchBytes = kOffScan + align256(sizeof(int32_t) * kScanTmpInts);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mutex;
constexpr int kMaxDevices = 64;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

int na_fail(int code, const std::string& m) {
    set_last_error(m);
    return code;
}

struct NaView {
    int32_t *count, *start, *key, *rank, *perm, *id, *skey, *scan;
    double *x, *y, *z;
};

__global__ void k_na_keys(Consts c, int n, const double* __restrict__ pos, const int32_t* __restrict__ type,
                          NaView v) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t kk = c.nkeys;
    const double x = pos[3 * (size_t)i], y = pos[3 * (size_t)i + 1], z = pos[3 * (size_t)i + 2];
    if (type[i] != T_GHOST && isfinite(x) && isfinite(y) && isfinite(z)) kk = cell_key(c, x, y, z);
    v.key[i] = kk;
    v.rank[i] = atomicAdd(v.count + kk, 1);
}

__global__ void k_na_scatter(int n, NaView v) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v.perm[v.start[v.key[i]] + v.rank[i]] = i;
}

// ascending particle index inside each cell (the reference's linked-list order)
__global__ void k_na_cellsort(int nkeys, NaView v) {
    int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= nkeys) return;
    const int b = v.start[cell], e = v.start[cell + 1];
    for (int t = b + 1; t < e; t++) {
        const int pv = v.perm[t];
        int u = t - 1;
        while (u >= b && v.perm[u] > pv) {
            v.perm[u + 1] = v.perm[u];
            u--;
        }
        v.perm[u + 1] = pv;
    }
}

__global__ void k_na_gather(int n, const double* __restrict__ pos, NaView v) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = v.perm[k];
    v.id[k] = i;
    v.skey[k] = v.key[i];
    v.x[k] = pos[3 * (size_t)i];
    v.y[k] = pos[3 * (size_t)i + 1];
    v.z[k] = pos[3 * (size_t)i + 2];
}

// MPS::setNumberDensity at load (src/mps.cpp:627-641): boundary conditions
// are all Ignored there, so the ratio is sum(w(d, re_p)) / n0 over the
// neighbours (d < re_max) in the reference's sweep order.
__global__ void k_na_density(Consts c, int n, const int32_t* __restrict__ type, NaView v,
                             double* __restrict__ ndr) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = v.id[k];
    const int32_t key = v.skey[k];
    if (key >= c.nkeys) {  // Ghost (never in a neighbour list) or non-finite position
        ndr[i] = type[i] == T_GHOST ? 0.0 : __longlong_as_double(0x7ff8000000000000ll);
        return;
    }
    StateBuf s{};
    s.x = v.x;
    s.y = v.y;
    s.z = v.z;
    const double xi = v.x[k], yi = v.y[k], zi = v.z[k];
    double nd = 0.0;
    for_each_candidate<false>(c, v.start, key, [&](int j) {
        if (j == k) return;
        const double d2 = dist2<false>(s, k, j, xi, yi, zi);
        if (d2 < c.t_max && d2 < c.t_p) nd = mpsg::dadd(nd, mpsg::weight(mpsg::dsqrt(d2), c.re_p));
    });
    ndr[i] = mpsg::ddiv(nd, c.n0_p);
}

}  // namespace

extern "C" int mps_number_density_static(const mps_params* prm, int32_t n, const double* d_pos,
                                         const int32_t* d_type, double* d_ndr, void* stream) {
    if (!prm || !d_pos || !d_type || !d_ndr || n <= 0)
        return na_fail(MPS_ERR_ARG, "mps_number_density_static: null pointer or n <= 0");
    if (n > kMaxParticles)
        return na_fail(MPS_ERR_ARG, "mps_number_density_static: " + std::to_string(n) +
                                        " particles exceed the static scratch limit of " +
                                        std::to_string(kMaxParticles));
    const mps_params& P = *prm;
    if (!(P.particle_distance > 0) || !(P.re_pressure > 0) || !(P.re_viscosity > 0) ||
        !(P.re_surface > 0) || (P.dim != 2 && P.dim != 3))
        return na_fail(MPS_ERR_ARG, "mps_number_density_static: invalid dim, distance or radius");
    Consts c{};
    c.n = n;
    c.dim = P.dim;
    c.planar = 0;  // the general (x, y, z) cell key; in 2-D it visits the same cells in the same order
    for (int d = 0; d < 3; d++) c.dmin[d] = P.domain_min[d];
    c.re_p = P.re_pressure;
    c.re_max = std::max({P.re_pressure, P.re_viscosity, P.re_surface});  // src/settings.cpp:138
    c.len = c.re_max;
    {
        // src/bucket.cpp:14-16; a non-finite or inverted domain is refused
        // here, before the GPU is touched (every axis then has >= 3 cells)
        int32_t dims[3];
        std::string why;
        if (!bucket_grid(P, c.len, dims, &why))
            return na_fail(MPS_ERR_ARG, "mps_number_density_static: " + why);
        c.numX = dims[0];
        c.numY = dims[1];
        c.numZ = dims[2];
    }
    const double nk = (double)c.numX * c.numY * c.numZ;
    if (!(nk <= (double)kMaxCells))
        return na_fail(MPS_ERR_ARG, "mps_number_density_static: the bucket grid has " +
                                        std::to_string((long long)nk) + " cells, above the static scratch limit of " +
                                        std::to_string(kMaxCells));
    c.nkeys = (int32_t)nk;
    c.t_p = sq_threshold(c.re_p);
    c.t_max = sq_threshold(c.re_max);
    ref_values(P.dim, P.particle_distance, c.re_p, &c.n0_p, nullptr);

    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) return na_fail(MPS_ERR_NO_DEVICE, cudaGetErrorString(ce));
    if (dev < 0 || dev >= kMaxDevices) return na_fail(MPS_ERR_NO_DEVICE, "device index out of range");
    unsigned char* base;
    {
        std::lock_guard<std::mutex> lk(g_mutex);
        if (!g_scratch_ptr[dev]) {
            void* p = nullptr;
            ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (ce != cudaSuccess)
                return na_fail(MPS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(ce));
            g_scratch_ptr[dev] = (unsigned char*)p;
        }
        base = g_scratch_ptr[dev];
    }
    NaView v;
    v.count = (int32_t*)(base + kOffCount);
    v.start = (int32_t*)(base + kOffStart);
    v.key = (int32_t*)(base + kOffKey);
    v.rank = (int32_t*)(base + kOffRank);
    v.perm = (int32_t*)(base + kOffPerm);
    v.id = (int32_t*)(base + kOffId);
    v.skey = (int32_t*)(base + kOffSkey);
    v.x = (double*)(base + kOffX);
    v.y = (double*)(base + kOffY);
    v.z = (double*)(base + kOffZ);
    v.scan = (int32_t*)(base + kOffScan);

    cudaStream_t st = (cudaStream_t)stream;
    const int T = 256, G = (n + T - 1) / T;
    ce = cudaMemsetAsync(v.count, 0, sizeof(int32_t) * (c.nkeys + 1), st);
    if (ce != cudaSuccess) return na_fail(MPS_ERR_CUDA, cudaGetErrorString(ce));
    k_na_keys<<<G, T, 0, st>>>(c, n, d_pos, d_type, v);
    launch_exclusive_scan(v.count, v.start, c.nkeys + 1, v.scan, st);
    k_na_scatter<<<G, T, 0, st>>>(n, v);
    k_na_cellsort<<<(c.nkeys + T - 1) / T, T, 0, st>>>(c.nkeys, v);
    k_na_gather<<<G, T, 0, st>>>(n, d_pos, v);
    k_na_density<<<G, T, 0, st>>>(c, n, d_type, v, d_ndr);
    ce = cudaGetLastError();
    if (ce != cudaSuccess) return na_fail(MPS_ERR_CUDA, cudaGetErrorString(ce));
    return MPS_OK;
}
