// Setup of the aggregation multigrid preconditioner used by the mixed
// pressure solver (the V-cycle itself runs inside k_cg_mixed, solver.cu).
//
// Level 1: one unknown per bucket cell (numX x numY, cell index
// cx * numY + cy, the planar cell key).  Its operator is the Galerkin
// product P^T A P of the FP32 particle matrix with piecewise-constant P over
// the Inner particles of each cell; since a particle couples only to the
// 3x3 cells around its own, the result is a 9-point stencil.  Level l+1
// aggregates 2x2 cells of level l, again a 9-point stencil.  Every coarse
// entry is summed by one thread in a fixed order, so the hierarchy is
// deterministic.  The coarsest level gets an explicit inverse (Gauss-Jordan
// without pivoting: the Galerkin operator of an SPD matrix is SPD).
#include "devutil.cuh"
#include "engine.cuh"

namespace mpsg {

namespace {

// Adds v to stencil entry d, the nine entries kept in registers (an
// indexed local array would live in local memory); the other entries add
// +0, which leaves them unchanged, so the sums equal one indexed add.
__device__ __forceinline__ void add_tap(float (&st)[9], int d, float v) {
#pragma unroll
    for (int q = 0; q < 9; q++) st[q] += q == d ? v : 0.f;
}

// Appends cell I to the level's list of cells with unknowns: one atomic per
// warp, the warp's cells in ascending order.
// Returns the entry's position (-1 for a cell that is not listed).
__device__ __forceinline__ int list_active(bool act, int I, int32_t* list, int32_t* count) {
    const unsigned am = __activemask();
    const unsigned m = __ballot_sync(am, act);
    if (!m) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(m));
    base = __shfl_sync(am, base, leader);
    const int pos = base + __popc(m & ((1u << lane) - 1u));
    if (act) list[pos] = I;
    return act ? pos : -1;
}

// Every cell's r, e and t to 0 on the levels the grid-wide phases visit by
// list (levels 1 .. ngrid + 1), and the list lengths to 0.
__global__ void k_mg_clear(Mg mg) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
    if (t < kMgMaxLevels) mg.nact[t] = 0;
    for (int l = 1; l <= mg.ngrid + 1 && l <= mg.nlev; l++) {
        const MgLevel& L = mg.lev[l];
        const int n = L.nx * L.ny;
        for (int I = t; I < n; I += nt) {
            L.r[I] = 0.f;
            L.e[I] = 0.f;
            L.t[I] = 0.f;
        }
    }
}

// Level 1's 9-point stencil of cell I: the sum over the cell's rows of
// their row-to-cell sums B (k_mg_rowcell), which is P1^T A P1 (rows that are
// not unknowns have B = 0).  Nine coalesced loads per row instead of a walk
// over the rows' entries.
__global__ void k_mg_level1(Consts c, MgLevel L, const float* __restrict__ B, size_t np, const int32_t* cs,
                            int32_t* nact, int2* act_rng) {
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= L.nx * L.ny) return;
    float st[9];
#pragma unroll
    for (int d = 0; d < 9; d++) st[d] = 0.f;
    const int b = cs[I], e = cs[I + 1];
    for (int k = b; k < e; k++) {
#pragma unroll
        for (int d = 0; d < 9; d++) st[d] += __ldg(B + (size_t)d * np + k);
    }
    const int n = L.nx * L.ny;
#pragma unroll
    for (int d = 0; d < 9; d++) L.st[(size_t)d * n + I] = st[d];
    L.invd[I] = st[4] > 0.f ? 1.f / st[4] : 0.f;
    const int pos = list_active(st[4] > 0.f, I, L.act, nact + 1);
    if (pos >= 0) act_rng[pos] = make_int2(b, e - b);  // the cell's slots, beside its list entry
}

// Smoothed transfer: B = A P1 per slot (the row's sums over the 3x3 cells
// around its own, diagonal included), in the entry order of k_mg_level1.
// Slots that are not unknowns get 0.
__global__ void k_mg_rowcell(Consts c, Ppe A, MatFree mf, size_t np, float* __restrict__ B) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    float st[9];
#pragma unroll
    for (int d = 0; d < 9; d++) st[d] = 0.f;
    const float dg = A.diag32[i];
    if (dg > 0.f) {
        st[4] = dg;
        // an unknown is Inner, so its cell is an interior cell of the grid
        const int key = mf.skey[i];
        const int cx = key / c.numY, cy = key - cx * c.numY;
        const int cnt = A.offcnt[i];
        if (mf.enabled && !mf.sell_row[i]) {
            int rs[3][4];
            for (int r = 0; r < 3; r++) {
                const int kk = (cx - 1 + r) * c.numY + cy - 1;
                for (int q = 0; q < 4; q++) rs[r][q] = mf.cs[kk + q];
            }
            const size_t q0 = qsell_index(i, 0, c.K) >> 2;
            const float4* vp = reinterpret_cast<const float4*>(A.val32) + q0;
            const uint32_t* ip = reinterpret_cast<const uint32_t*>(mf.idx8) + q0;
            const int ng = (cnt + 3) >> 2;
            for (int g0 = 0; g0 < ng; g0 += 4) {
                float4 v[4];
                uint32_t b4[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int gi = min(g0 + q, ng - 1);
                    v[q] = __ldg(vp + gi * 32);
                    b4[q] = __ldg(ip + gi * 32);
                }
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const float vv[4] = {v[q].x, v[q].y, v[q].z, v[q].w};
#pragma unroll
                    for (int t = 0; t < 4; t++) {
                        if ((g0 + q) * 4 + t >= cnt) break;
                        const int bt = (b4[q] >> (8 * t)) & 255;
                        const int r = bt >> 6;
                        const int j = rs[r][0] + (bt & 63);
                        const int dy = (j >= rs[r][1]) + (j >= rs[r][2]) - 1;
                        add_tap(st, r * 3 + (dy + 1), vv[t]);
                    }
                }
            }
        } else {
            const size_t base = (size_t)(i >> 5) * c.K * 32 + (i & 31);
            for (int m = 0; m < cnt; m++) {
                const float v = A.val32[qsell_index(i, m, c.K)];
                const int j = A.col[base + (size_t)m * 32];
                const int kj = mf.skey[j];
                const int jx = kj / c.numY, jy = kj - jx * c.numY;
                add_tap(st, (jx - cx + 1) * 3 + (jy - cy + 1), v);
            }
        }
    }
#pragma unroll
    for (int d = 0; d < 9; d++) B[(size_t)d * np + i] = st[d];
}

// Coarse level C from fine level F: the Galerkin 9-point stencil and C's
// restriction weights (MgLevel::rw).  The residual that the V-cycle hands
// from F to C is, for each child c of a coarse cell, r_c - sum_d st_d(c)
// omega invd_j r_j (one Jacobi step from zero on F, then its residual);
// summed over the 2x2 children it is a fixed 4x4 stencil on r_F, whose
// weights depend only on the operator and omega.
__global__ void k_mg_coarsen(MgLevel F, MgLevel C, float omega, int32_t* nact_c) {
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    const int nc = C.nx * C.ny;
    if (I >= nc) return;
    const int X = I / C.ny, Y = I - X * C.ny;
    const int nf = F.nx * F.ny;
    float st[9], w[16];
#pragma unroll
    for (int d = 0; d < 9; d++) st[d] = 0.f;
#pragma unroll
    for (int k = 0; k < 16; k++) w[k] = 0.f;
    for (int a = 0; a < 2; a++)
        for (int bb = 0; bb < 2; bb++) {
            const int x = 2 * X + a, y = 2 * Y + bb;
            if (x >= F.nx || y >= F.ny) continue;
            const int cf = x * F.ny + y;
            w[(a + 1) * 4 + (bb + 1)] += 1.f;
            for (int d = 0; d < 9; d++) {
                const int nx = x + d / 3 - 1, ny = y + d % 3 - 1;
                if (nx < 0 || ny < 0 || nx >= F.nx || ny >= F.ny) continue;
                const float s = F.st[(size_t)d * nf + cf];
                const int DX = nx / 2 - X, DY = ny / 2 - Y;
                st[(DX + 1) * 3 + (DY + 1)] += s;
                // tap (nx, ny) sits at (nx - 2X + 1, ny - 2Y + 1) of the 4x4 patch
                w[(nx - 2 * X + 1) * 4 + (ny - 2 * Y + 1)] -= omega * F.invd[nx * F.ny + ny] * s;
            }
        }
#pragma unroll
    for (int d = 0; d < 9; d++) C.st[(size_t)d * nc + I] = st[d];
    C.invd[I] = st[4] > 0.f ? 1.f / st[4] : 0.f;
    list_active(st[4] > 0.f, I, C.act, nact_c);
#pragma unroll
    for (int k = 0; k < 16; k++) C.rw[(size_t)k * nc + I] = w[k];
}

// Dense inverse of the coarsest operator; cells without unknowns get an
// identity row so that the matrix stays invertible (their residual is 0).
__global__ void k_mg_dense(MgLevel L, float* out) {
    __shared__ float M[kMgMaxCoarsest][kMgMaxCoarsest];
    const int n = L.nx * L.ny;
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
        const int i = t / n, j = t % n;
        float v = 0.f;
        const bool act = L.invd[i] > 0.f;
        if (!act) {
            v = (i == j) ? 1.f : 0.f;
        } else if (L.invd[j] > 0.f) {
            const int xi = i / L.ny, yi = i % L.ny, xj = j / L.ny, yj = j % L.ny;
            const int dx = xj - xi, dy = yj - yi;
            if (dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1) v = L.st[(size_t)((dx + 1) * 3 + (dy + 1)) * n + i];
        }
        M[i][j] = v;
    }
    __shared__ float fcol[kMgMaxCoarsest];
    __syncthreads();
    for (int k = 0; k < n; k++) {
        const float piv = 1.f / M[k][k];
        __syncthreads();
        for (int j = threadIdx.x; j < n; j += blockDim.x) M[k][j] = (j == k ? 1.f : M[k][j]) * piv;
        for (int i = threadIdx.x; i < n; i += blockDim.x) fcol[i] = M[i][k];
        __syncthreads();
        for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
            const int i = t / n, j = t % n;
            if (i == k) continue;
            const float f = fcol[i];
            if (j == k)
                M[i][j] = -f * M[k][k];
            else
                M[i][j] -= f * M[k][j];
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) out[t] = M[t / n][t % n];
}

}  // namespace

void launch_mg_setup(const Consts& c, const Ppe& A, const MatFree& mf, const Mg& mg,
                     cudaStream_t st) {
    if (!mg.enabled) return;
    const int T = 256;
    // the rows' 3x3-cell sums: the operator of modes 1 and 3, and level 1's stencil
    k_mg_rowcell<<<(c.n + T - 1) / T, T, 0, st>>>(c, A, mf, (size_t)mg.n_pad, mg.rowcell);
    ++g_launches;
    const MgLevel& L1 = mg.lev[1];
    k_mg_clear<<<(L1.nx * L1.ny + T - 1) / T, T, 0, st>>>(mg);
    k_mg_level1<<<(L1.nx * L1.ny + T - 1) / T, T, 0, st>>>(c, L1, mg.rowcell, (size_t)mg.n_pad, mf.cs, mg.nact,
                                                             mg.act1_rng);
    g_launches += 2;
    for (int l = 1; l < mg.nlev; l++) {
        const MgLevel& C = mg.lev[l + 1];
        k_mg_coarsen<<<(C.nx * C.ny + T - 1) / T, T, 0, st>>>(mg.lev[l], C, mg.omega, mg.nact + l + 1);
        ++g_launches;
    }
    k_mg_dense<<<1, 1024, 0, st>>>(mg.lev[mg.nlev], mg.dense);
    ++g_launches;
}

}  // namespace mpsg
