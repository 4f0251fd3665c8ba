// Bucket neighbour-search rebuild: the GB300 form of Bucket::storeParticles
// (src/bucket.cpp:24-51).
//
// The reference threads particles into per-cell linked lists in ascending id
// order.  Here each build is a counting sort of the particle slots by cell
// key (x-major: key = (ix * numY + iy) * numZ + iz), followed by an id sort
// inside every cell, which reproduces the reference's in-cell order, and a
// gather of every state array into the second buffer.  Ghost particles get
// the sentinel key nkeys and collect after all cells.  Roofline: HBM; per
// particle and build the gather moves ~2 x 80 B.
#include "devutil.cuh"
#include "engine.cuh"

namespace mpsg {

thread_local int32_t g_launches = 0;

namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void k_keys(Consts c, StateBuf s, int32_t* __restrict__ key, int32_t* __restrict__ rank,
                       int32_t* __restrict__ count, DevStats* ds) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c.n) return;
    int32_t kk = c.nkeys;
    if (s.type[k] != T_GHOST) {
        const double x = s.x[k], y = s.y[k], z = c.planar ? 0.0 : s.z[k];
        if (isfinite(x) && isfinite(y) && isfinite(z)) {
            kk = cell_key(c, x, y, z);
        } else {
            // the reference has no defined behaviour here; the particle is
            // taken out of the neighbour search and the step reports an error
            s.type[k] = T_GHOST;
            atomicOr(&ds->status, ST_NONFINITE);
        }
    }
    key[k] = kk;
    rank[k] = atomicAdd(count + kk, 1);
}

__global__ void k_scatter(int n, const int32_t* __restrict__ key, const int32_t* __restrict__ rank,
                          const int32_t* __restrict__ start, int32_t* __restrict__ perm) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    perm[start[key[k]] + rank[k]] = k;
}

// Ascending id inside each cell (the reference's linked-list order).
__global__ void k_cellsort(int nkeys, const int32_t* __restrict__ start, int32_t* __restrict__ perm,
                           const int32_t* __restrict__ id) {
    int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= nkeys) return;
    int b = start[cell], e = start[cell + 1];
    int m = e - b;
    if (m < 2) return;
    constexpr int R = 24;
    if (m <= R) {
        int ps[R], is[R];
        for (int t = 0; t < m; t++) {
            ps[t] = perm[b + t];
            is[t] = id[ps[t]];
        }
        for (int t = 1; t < m; t++) {
            int pv = ps[t], iv = is[t], u = t - 1;
            while (u >= 0 && is[u] > iv) {
                ps[u + 1] = ps[u];
                is[u + 1] = is[u];
                u--;
            }
            ps[u + 1] = pv;
            is[u + 1] = iv;
        }
        for (int t = 0; t < m; t++) perm[b + t] = ps[t];
    } else {  // crowded cell: in place
        for (int t = b + 1; t < e; t++) {
            int pv = perm[t], iv = id[pv], u = t - 1;
            while (u >= b && id[perm[u]] > iv) {
                perm[u + 1] = perm[u];
                u--;
            }
            perm[u + 1] = pv;
        }
    }
}

__global__ void k_gather(int n, const int32_t* __restrict__ perm, const int32_t* __restrict__ key,
                         int32_t* __restrict__ skey, StateBuf in, StateBuf out, int planar) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int o = perm[k];
    skey[k] = key[o];
    const double x = in.x[o], y = in.y[o];
    out.x[k] = x;
    out.y[k] = y;
    const float xh = f32(x), yh = f32(y);
    out.xyf[k] = make_float2(xh, yh);
    // x - xh is exact in FP64 (xh is x rounded to 24 bits)
    out.xylo[k] = make_float2(f32(x - (double)xh), f32(y - (double)yh));
    const double vx = in.vx[o], vy = in.vy[o];
    out.vx[k] = vx;
    out.vy[k] = vy;
    out.vf[k] = make_float2(f32(vx), f32(vy));
    if (!planar) {
        const double z = in.z[o];
        out.z[k] = z;
        out.zf[k] = f32(z);
        out.vz[k] = in.vz[o];
    }
    out.p[k] = in.p[o];
    out.minp[k] = in.minp[o];
    out.ndr[k] = in.ndr[o];
    out.nd_last[k] = in.nd_last[o];
    out.id[k] = in.id[o];
    out.type[k] = in.type[o];
    out.bc[k] = in.bc[o];
    out.dir[k] = in.dir[o];
}

// ---- exclusive scan (three passes: tile sums, scan of sums, tile scan) ----

__device__ __forceinline__ int block_exclusive_scan(int v, int* sh, int* total) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[w] = x;
    __syncthreads();
    if (w == 0) {
        int nw = blockDim.x >> 5;
        int t = lane < nw ? sh[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < nw) sh[lane] = t;
    }
    __syncthreads();
    int pre = (w > 0 ? sh[w - 1] : 0) + x - v;
    *total = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    return pre;
}

__global__ void k_scan_reduce(const int32_t* __restrict__ in, int n, int32_t* __restrict__ sums) {
    __shared__ int sh[32];
    int base = blockIdx.x * kScanTile;
    int s = 0;
#pragma unroll
    for (int t = 0; t < kScanItems; t++) {
        int i = base + t * kScanThreads + threadIdx.x;
        if (i < n) s += in[i];
    }
    int tot;
    block_exclusive_scan(s, sh, &tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_scan_top(int32_t* sums, int nb) {
    __shared__ int sh[32];
    int carry = 0;
    for (int b0 = 0; b0 < nb; b0 += blockDim.x) {
        int i = b0 + threadIdx.x;
        int v = i < nb ? sums[i] : 0;
        int tot;
        int pre = block_exclusive_scan(v, sh, &tot);
        if (i < nb) sums[i] = carry + pre;
        carry += tot;
    }
}

__global__ void k_scan_apply(const int32_t* in, int n, const int32_t* __restrict__ sums,
                             int32_t* out) {
    __shared__ int sh[32];
    int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int t = 0; t < kScanItems; t++) {
        int i = base + t;
        v[t] = i < n ? in[i] : 0;
        s += v[t];
    }
    int tot;
    int pre = block_exclusive_scan(s, sh, &tot) + sums[blockIdx.x];
#pragma unroll
    for (int t = 0; t < kScanItems; t++) {
        int i = base + t;
        if (i < n) out[i] = pre;
        pre += v[t];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[n] = pre;
}

}  // namespace

size_t scan_tmp_ints(int32_t n) { return (size_t)(n + kScanTile - 1) / kScanTile + 32; }

void launch_exclusive_scan(const int32_t* in, int32_t* out, int32_t n, int32_t* tmp,
                           cudaStream_t st) {
    int nb = (n + kScanTile - 1) / kScanTile;
    if (nb < 1) nb = 1;
    k_scan_reduce<<<nb, kScanThreads, 0, st>>>(in, n, tmp);
    ++g_launches;
    k_scan_top<<<1, 1024, 0, st>>>(tmp, nb);
    ++g_launches;
    k_scan_apply<<<nb, kScanThreads, 0, st>>>(in, n, tmp, out);
    ++g_launches;
}

void launch_rebuild(const Consts& c, const StateBuf& in, const StateBuf& out, SortScratch& s,
                    DevStats* ds, cudaStream_t st) {
    const int T = 256;
    int nb = (c.n + T - 1) / T;
    cudaMemsetAsync(s.cell_count, 0, sizeof(int32_t) * (c.nkeys + 1), st);
    k_keys<<<nb, T, 0, st>>>(c, in, s.key, s.rank, s.cell_count, ds);
    ++g_launches;
    launch_exclusive_scan(s.cell_count, s.cell_start, c.nkeys + 1, s.scan_tmp, st);
    k_scatter<<<nb, T, 0, st>>>(c.n, s.key, s.rank, s.cell_start, s.perm);
    ++g_launches;
    k_cellsort<<<(c.nkeys + T - 1) / T, T, 0, st>>>(c.nkeys, s.cell_start, s.perm, in.id);
    ++g_launches;
    k_gather<<<nb, T, 0, st>>>(c.n, s.perm, s.key, s.skey, in, out, c.planar);
    ++g_launches;
}

}  // namespace mpsg
