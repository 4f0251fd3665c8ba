// Particle-interaction kernels of the MPS step (src/mps.cpp:165-667).
//
// Every kernel works on the cell-sorted slots of the current StateBuf; the
// neighbour sweep visits candidates in the reference's order so that the
// FP64 sums (viscosity, number densities, matrix diagonal, gradient) round
// exactly like the reference's.  Roofline of this family: FP64 issue on
// GB300 (~0.5 T DFMA/s, ~52 G div or sqrt/s per GPU) for the exact sweeps,
// HBM for the list-driven ones.
#include "devutil.cuh"
#include "engine.cuh"

namespace mpsg {

namespace {

constexpr int kThreads = 256;
constexpr int kCollBlocks = 304;  // blocks of the parallel collision pass (two per SM)

inline int blocks_for(int n, int t = kThreads) { return (n + t - 1) / t; }

__device__ __forceinline__ void raise_status(DevStats* ds, int32_t bit) { atomicOr(&ds->status, bit); }

__device__ __forceinline__ bool outside_domain(const Consts& c, double x, double y, double z) {
    // MPS::checkBoundaryViolation: src/mps.cpp:643-667
    return x < c.dmin[0] || c.dmax[0] < x || y < c.dmin[1] || c.dmax[1] < y || z < c.dmin[2] ||
           c.dmax[2] < z;
}

// Visits, in sweep order, the candidates of particle k that survive the FP32
// pre-filter at `bound`: pass 1 collects them in a local list, pass 2 calls
// f(j), where f runs the exact FP64 test and the work.  Splitting the sweep
// keeps the FP64 work on compact lists, with nearly all lanes of a warp busy.
// More survivors than the list holds: f(j) for every candidate (f's exact
// test then selects the same neighbours in the same order).
constexpr int kNear = 64;
template <bool PLANAR, class F>
__device__ __forceinline__ void for_each_near(const Consts& c, const StateBuf& s,
                                              const int32_t* __restrict__ cs, int32_t key, int k,
                                              float bound, F&& f) {
    const float2 fk = s.xyf[k];
    const float fx = fk.x, fy = fk.y, fz = PLANAR ? 0.f : s.zf[k];
    int cand[kNear];
    int ns = 0;
    for_each_candidate<PLANAR>(c, cs, key, [&](int j) {
        if (j == k || far32<PLANAR>(s, j, fx, fy, fz, bound)) return;
        if (ns < kNear) cand[ns] = j;
        ns++;
    });
    if (ns <= kNear) {
        for (int q = 0; q < ns; q++) f(cand[q]);
    } else {
        for_each_candidate<PLANAR>(c, cs, key, [&](int j) {
            if (j != k) f(j);
        });
    }
}

// Number density at re_p over a particle's current neighbours (d < re_max),
// in sweep order: the value a later setNumberDensity reads from the stale
// list of a particle that has just become a ghost (src/mps.cpp:590-593).
template <bool PLANAR>
__device__ double sweep_number_density_p(const Consts& c, const StateBuf& s, const int32_t* cs,
                                         int32_t key, int k) {
    double xi = s.x[k], yi = s.y[k], zi = PLANAR ? 0.0 : s.z[k];
    const float2 fk = s.xyf[k];
    const float fx = fk.x, fy = fk.y, fz = PLANAR ? 0.f : s.zf[k];
    double nd = 0.0;
    for_each_candidate<PLANAR>(c, cs, key, [&](int j) {
        if (j == k || far32<PLANAR>(s, j, fx, fy, fz, c.ft_max)) return;
        double d2 = dist2<PLANAR>(s, k, j, xi, yi, zi);
        if (lt_cut(d2, c.t_max) && lt_cut(d2, c.t_p)) nd = dadd(nd, weight(dsqrt(d2), c.re_p));
    });
    return nd;
}

// ---------------------------------------------------------------------------
// calcGravity + calcViscosity + moveParticles (+ checkBoundaryViolation),
// src/mps.cpp:165-215 and 643-667, fused with the first neighbour sweep.
// Reads `in`, writes the moved state to `out` (same slot order).
template <bool PLANAR, bool MIXED>
__global__ void __launch_bounds__(kThreads) k_explicit(Consts c, StateBuf in, StateBuf out,
                                                       const int32_t* __restrict__ skey,
                                                       const int32_t* __restrict__ cs,
                                                       DevStats* ds) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c.n) return;
    int8_t t = in.type[k];
    double x = in.x[k], y = in.y[k], vx = in.vx[k], vy = in.vy[k];
    double z = PLANAR ? c.z0 : in.z[k], vz = PLANAR ? 0.0 : in.vz[k];
    double nd_last = in.nd_last[k];
    if (t == T_FLUID) {
        const int32_t key = skey[k];
        double ax, ay, az;
        if (!MIXED) {
            double tx = 0.0, ty = 0.0, tz = 0.0;
            for_each_near<PLANAR>(c, in, cs, key, k, c.ft_v, [&](int j) {
                double d2 = dist2<PLANAR>(in, k, j, x, y, z);
                if (lt_cut(d2, c.t_max) && lt_cut(d2, c.t_v)) {
                    double w = weight(dsqrt(d2), c.re_v);
                    tx = dadd(tx, dmul(dsub(in.vx[j], vx), w));
                    ty = dadd(ty, dmul(dsub(in.vy[j], vy), w));
                    if (!PLANAR) tz = dadd(tz, dmul(dsub(in.vz[j], vz), w));
                }
            });
            ax = dadd(c.g[0], dmul(tx, c.visc_a));
            ay = dadd(c.g[1], dmul(ty, c.visc_a));
            az = PLANAR ? 0.0 : dadd(c.g[2], dmul(tz, c.visc_a));
        } else if (PLANAR) {
            // FP32 weights and FP32 accumulation; the neighbour set is the
            // exact FP64 one: the FP32 squared distance of the coordinate
            // pairs decides outside the band [fv_in, fv_out] around the
            // threshold (its error is far inside the band), the exact FP64
            // test inside it
            float tx = 0.f, ty = 0.f;
            const float2 hk = in.xyf[k], lk = in.xylo[k], vk = in.vf[k];
            for_each_near<PLANAR>(c, in, cs, key, k, c.ft_v, [&](int j) {
                const float2 hj = in.xyf[j], lj = in.xylo[j];
                const float dx = (hj.x - hk.x) + (lj.x - lk.x);
                const float dy = (hj.y - hk.y) + (lj.y - lk.y);
                const float d2f = dx * dx + dy * dy;
                bool inside = d2f < c.fv_in;
                if (!inside && !(d2f > c.fv_out)) {
                    const double d2 = dist2<PLANAR>(in, k, j, x, y, z);
                    inside = lt_cut(d2, c.t_max) && lt_cut(d2, c.t_v);
                }
                if (inside) {
                    const float2 vj = in.vf[j];
                    const float w = c.fre_v * rsqrtf(d2f) - 1.f;
                    tx = fmaf(vj.x - vk.x, w, tx);
                    ty = fmaf(vj.y - vk.y, w, ty);
                }
            });
            ax = c.g[0] + (double)(tx * c.fvisc_a);
            ay = c.g[1] + (double)(ty * c.fvisc_a);
            az = 0.0;
        } else {
            // FP32 weights and FP32 accumulation; the neighbour set is the
            // exact FP64 one.
            float tx = 0.f, ty = 0.f, tz = 0.f;
            const float fvx = f32(vx), fvy = f32(vy), fvz = f32(vz);
            for_each_near<PLANAR>(c, in, cs, key, k, c.ft_v, [&](int j) {
                double d2 = dist2<PLANAR>(in, k, j, x, y, z);
                if (lt_cut(d2, c.t_max) && lt_cut(d2, c.t_v)) {
                    float w = c.fre_v * rsqrtf(f32(d2)) - 1.f;
                    tx = fmaf(f32(in.vx[j]) - fvx, w, tx);
                    ty = fmaf(f32(in.vy[j]) - fvy, w, ty);
                    if (!PLANAR) tz = fmaf(f32(in.vz[j]) - fvz, w, tz);
                }
            });
            ax = c.g[0] + (double)(tx * c.fvisc_a);
            ay = c.g[1] + (double)(ty * c.fvisc_a);
            az = PLANAR ? 0.0 : c.g[2] + (double)(tz * c.fvisc_a);
        }
        vx = dadd(vx, dmul(ax, c.dt));
        vy = dadd(vy, dmul(ay, c.dt));
        double nx = dadd(x, dmul(vx, c.dt));
        double ny = dadd(y, dmul(vy, c.dt));
        double nz = z;
        if (!PLANAR) {
            vz = dadd(vz, dmul(az, c.dt));
            nz = dadd(z, dmul(vz, c.dt));
        }
        if (outside_domain(c, nx, ny, nz)) {
            t = T_GHOST;
            atomicAdd(&ds->n_new_ghosts, 1);
            nd_last = sweep_number_density_p<PLANAR>(c, in, cs, key, k);
        }
        x = nx;
        y = ny;
        z = nz;
    }
    out.x[k] = x;
    out.y[k] = y;
    out.vx[k] = vx;
    out.vy[k] = vy;
    if (!PLANAR) {
        out.z[k] = z;
        out.vz[k] = vz;
    }
    out.type[k] = t;
    out.nd_last[k] = nd_last;
    out.p[k] = in.p[k];
    out.minp[k] = in.minp[k];
    out.ndr[k] = in.ndr[k];
    out.id[k] = in.id[k];
    out.bc[k] = in.bc[k];
    out.dir[k] = in.dir[k];
}

// ---------------------------------------------------------------------------
// MPS::collision (src/mps.cpp:217-250).  The candidate pairs — fluid i,
// neighbour j with the stale distance < cd, skipping fluid j with id >= id_i
// — are found in parallel and laid out in the reference's order (ascending
// id_i, sweep order).  Their effect is order dependent (Gauss-Seidel, in
// place): pair t reads and writes the state of i and, for a fluid j, of j
// (a wall j is read but never changed: its inverse density is 0).  Pair t
// therefore depends exactly on the earlier pairs that touch i_t or a fluid
// j_t, and applying every pair after those (in any order otherwise) gives
// the serial loop's result bit for bit.  Each pair counts the earlier pairs
// touching each of its particles: for i_t its position in i_t's own run of
// pairs (no earlier pair has i_t as j: that needs id_i' > id_i_t); for j_t
// the pairs of j_t's own run (all earlier) plus the earlier pairs with the
// same j (from a short per-particle list).  A pair waits until the
// particles' counters of applied pairs reach those numbers, applies itself
// and increments them; chunks of pairs are taken in order from a ticket
// counter, so every pair waited on belongs to a running or finished block.
// More than kCollJList pairs with one j fall back to the serial pass.
template <bool PLANAR>
__device__ __forceinline__ int for_each_collision(const Consts& c, const StateBuf& s,
                                                  const int32_t* cs, int32_t key, int k,
                                                  CollPair* out) {
    double xi = s.x[k], yi = s.y[k], zi = PLANAR ? 0.0 : s.z[k];
    const float2 fk = s.xyf[k];
    const float fx = fk.x, fy = fk.y, fz = PLANAR ? 0.f : s.zf[k];
    int32_t idi = s.id[k];
    int m = 0;
    for_each_candidate<PLANAR>(c, cs, key, [&](int j) {
        if (j == k || far32<PLANAR>(s, j, fx, fy, fz, c.ft_cd)) return;
        double d2 = dist2<PLANAR>(s, k, j, xi, yi, zi);
        if (!(lt_cut(d2, c.t_max) && lt_cut(d2, c.t_cd))) return;
        if (s.type[j] == T_FLUID && s.id[j] >= idi) return;
        if (out) out[m] = CollPair{k, j, idi, s.id[j], dsqrt(d2)};
        m++;
    });
    return m;
}

template <bool PLANAR>
__global__ void __launch_bounds__(kThreads) k_coll_count(Consts c, StateBuf s,
                                                         const int32_t* __restrict__ skey,
                                                         const int32_t* __restrict__ cs,
                                                         int32_t* __restrict__ cnt_by_id) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c.n || s.type[k] != T_FLUID) return;
    int m = for_each_collision<PLANAR>(c, s, cs, skey[k], k, nullptr);
    if (m) cnt_by_id[s.id[k]] = m;
}

template <bool PLANAR>
__global__ void __launch_bounds__(kThreads) k_coll_write(Consts c, StateBuf s,
                                                         const int32_t* __restrict__ skey,
                                                         const int32_t* __restrict__ cs,
                                                         const int32_t* __restrict__ cnt_by_id,
                                                         const int32_t* __restrict__ base_by_id,
                                                         CollPair* pairs, int32_t cap,
                                                         DevStats* ds) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c.n || s.type[k] != T_FLUID) return;
    int32_t id = s.id[k];
    if (cnt_by_id[id] == 0) return;
    int32_t b = base_by_id[id];
    if (b + cnt_by_id[id] > cap) {
        raise_status(ds, ST_CAPACITY);
        return;
    }
    for_each_collision<PLANAR>(c, s, cs, skey[k], k, pairs + b);
}

// One pair of the collision loop (the body of src/mps.cpp:222-247), with
// loads and stores through L2 (other threads apply the neighbouring pairs).
// A wall or dummy j has inverse density 0: its update adds +-0, which leaves
// it unchanged unless it holds -0 (turned into +0); the parallel pass
// (WRITE_WALL false) skips that store, so that pairs sharing a wall do not
// race; walls hold no -0 (their velocities start at +0 and only such
// updates touch them), so both passes give the same state.
template <bool PLANAR, bool WRITE_WALL>
__device__ __forceinline__ void coll_apply_pair(const Consts& c, const StateBuf& s, const CollPair& q,
                                                double inv_rho) {
    const int i = q.si, j = q.sj;
    const double inv_i = inv_rho;  // i is fluid; Particle::inverseDensity, src/particle.cpp:19-29
    const bool jfluid = s.type[j] == T_FLUID;
    const bool wj = WRITE_WALL || jfluid;
    const double inv_j = jfluid ? inv_rho : 0.0;
    const double reduced = ddiv(1.0, dadd(inv_i, inv_j));
    const double xi = __ldcg(s.x + i), yi = __ldcg(s.y + i), xj = __ldcg(s.x + j), yj = __ldcg(s.y + j);
    const double dx = dsub(xj, xi), dy = dsub(yj, yi);
    double zi = 0.0, zj = 0.0;
    if (!PLANAR) {
        zi = __ldcg(s.z + i);
        zj = __ldcg(s.z + j);
    }
    const double dz = PLANAR ? 0.0 : dsub(zj, zi);
    const double z2 = dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
    double nx = dx, ny = dy, nz = dz;
    if (z2 > 0.0) {
        const double r = dsqrt(z2);
        nx = ddiv(dx, r);
        ny = ddiv(dy, r);
        nz = ddiv(dz, r);
    }
    const double vxi = __ldcg(s.vx + i), vyi = __ldcg(s.vy + i), vxj = __ldcg(s.vx + j), vyj = __ldcg(s.vy + j);
    double vzi = 0.0, vzj = 0.0;
    if (!PLANAR) {
        vzi = __ldcg(s.vz + i);
        vzj = __ldcg(s.vz + j);
    }
    const double ux = dsub(vxj, vxi), uy = dsub(vyj, vyi);
    const double uz = PLANAR ? 0.0 : dsub(vzj, vzi);
    const double rel = dadd(dadd(dmul(ux, nx), dmul(uy, ny)), dmul(uz, nz));
    if (rel < 0.0) {
        const double impulse = dmul(dmul(-dadd(1.0, c.e), rel), reduced);
        const double ci = dmul(impulse, inv_i), cj = dmul(impulse, inv_j);
        __stcg(s.vx + i, dsub(vxi, dmul(ci, nx)));
        __stcg(s.vy + i, dsub(vyi, dmul(ci, ny)));
        if (wj) {
            __stcg(s.vx + j, dadd(vxj, dmul(cj, nx)));
            __stcg(s.vy + j, dadd(vyj, dmul(cj, ny)));
        }
        const double pimp = dmul(dsub(c.cd, q.dist), reduced);
        const double pi_ = dmul(pimp, inv_i), pj_ = dmul(pimp, inv_j);
        __stcg(s.x + i, dsub(xi, dmul(pi_, nx)));
        __stcg(s.y + i, dsub(yi, dmul(pi_, ny)));
        if (wj) {
            __stcg(s.x + j, dadd(xj, dmul(pj_, nx)));
            __stcg(s.y + j, dadd(yj, dmul(pj_, ny)));
        }
        if (!PLANAR) {
            __stcg(s.vz + i, dsub(vzi, dmul(ci, nz)));
            __stcg(s.z + i, dsub(zi, dmul(pi_, nz)));
            if (wj) {
                __stcg(s.vz + j, dadd(vzj, dmul(cj, nz)));
                __stcg(s.z + j, dadd(zj, dmul(pj_, nz)));
            }
        }
    }
}

// The serial pass: every pair in order by one thread (verification mode, or
// when a particle is the partner of more than kCollJList pairs).  Also
// reports the candidate count.
template <bool PLANAR>
__global__ void k_coll_apply(Consts c, StateBuf s, const CollPair* __restrict__ pairs,
                             const int32_t* __restrict__ total_p, int32_t cap, CollWork cw, DevStats* ds) {
    int32_t total = *total_p;
    ds->n_cand = total;
    if (total > cap) total = cap;
    if (!cw.serial && !cw.ctl[1]) return;  // the parallel pass applied them
    const double inv_rho = ddiv(1.0, c.rho);
    for (int32_t t = 0; t < total; t++) coll_apply_pair<PLANAR, true>(c, s, pairs[t], inv_rho);
}

// Per pair with a fluid partner j: its index in j's short list.
__global__ void k_coll_jlists(StateBuf s, const CollPair* __restrict__ pairs, const int32_t* __restrict__ total_p,
                              int32_t cap, CollWork cw) {
    const int32_t total = min(*total_p, cap);
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        const CollPair q = pairs[t];
        if (s.type[q.sj] != T_FLUID) continue;
        const int p = atomicAdd(cw.jn + q.ij, 1);
        if (p < kCollJList)
            cw.jl[(size_t)q.ij * kCollJList + p] = t;
        else
            atomicOr(cw.ctl + 1, 1);
    }
}

__device__ __forceinline__ int ld_acquire_i32(const int32_t* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Polls before a pair gives up waiting (~0.3 us each: ~2.5 s in all); a pair
// that gives up raises ST_TIMEOUT and the abort flag, on which every waiting
// pair gives up at once.
constexpr int kCollSpinLimit = 1 << 23;

template <bool PLANAR>
__global__ void __launch_bounds__(kThreads) k_coll_wave(Consts c, StateBuf s, const CollPair* __restrict__ pairs,
                                                        const int32_t* __restrict__ total_p, int32_t cap,
                                                        const int32_t* __restrict__ cnt_by_id,
                                                        const int32_t* __restrict__ base_by_id, CollWork cw,
                                                        DevStats* ds) {
    const int32_t total = min(*total_p, cap);
    if (total == 0 || cw.serial || *(volatile int32_t*)(cw.ctl + 1)) return;
    const double inv_rho = ddiv(1.0, c.rho);
    __shared__ int s_chunk;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_chunk = atomicAdd(cw.ctl, 1);
        __syncthreads();
        const int t0 = s_chunk * (int)blockDim.x;
        if (t0 >= total) return;
        const int t = t0 + (int)threadIdx.x;
        if (t >= total) continue;
        const CollPair q = pairs[t];
        const bool jf = s.type[q.sj] == T_FLUID;
        const int ri = t - base_by_id[q.ii];
        int rj = 0;
        if (jf) {
            rj = cnt_by_id[q.ij];
            const int m = min(cw.jn[q.ij], kCollJList);
            for (int u = 0; u < m; u++) rj += cw.jl[(size_t)q.ij * kCollJList + u] < t;
        }
        bool go = true;
        for (int it = 0; ld_acquire_i32(cw.ver + q.ii) != ri || (jf && ld_acquire_i32(cw.ver + q.ij) != rj);
             it++) {
            if (*(volatile int32_t*)(cw.ctl + 2)) {
                go = false;
                break;
            }
            if (it > kCollSpinLimit) {
                atomicOr(&ds->status, ST_TIMEOUT);
                atomicExch(cw.ctl + 2, 1);
                go = false;
                break;
            }
            __nanosleep(64);
        }
        if (!go) continue;
        coll_apply_pair<PLANAR, false>(c, s, q, inv_rho);
        __threadfence();
        atomicAdd(cw.ver + q.ii, 1);
        if (jf) atomicAdd(cw.ver + q.ij, 1);
    }
}

// ---------------------------------------------------------------------------
// MPS::setNeighbors (src/mps.cpp:585-619): the neighbour list of the build
// that the pressure part uses, stored column-major (slot, FP64 distance,
// FP64 weight at re_p), plus the number density at re_p (kept per particle
// as the value a stale-list read returns once it becomes a ghost).  With BC
// (the pressure part's build) the same pass also runs setBoundaryCondition
// and the classic setSourceTerm (src/mps.cpp:262-320): the surface number
// density summed over the list entries within re_s, in list order (the
// order in which the reference's getNumberDensity reads the stored list).
template <bool PLANAR, bool BC>
__global__ void __launch_bounds__(kThreads) k_build_list(Consts c, StateBuf s,
                                                         const int32_t* __restrict__ skey,
                                                         const int32_t* __restrict__ cs, NbList nb,
                                                         Ppe A, DevStats* ds) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = k < c.n && s.type[k] != T_GHOST;
    const int np = nb.n_pad;
    int m = 0;
    double nd = 0.0, nsurf = 0.0;  // number densities at re_p and (BC) re_s
    if (valid) {
        const double xi = s.x[k], yi = s.y[k], zi = PLANAR ? 0.0 : s.z[k];
        const float2 fk = s.xyf[k];
        const float fx = fk.x, fy = fk.y, fz = PLANAR ? 0.f : s.zf[k];
        // Pass 1: the candidates that survive the FP32 pre-filter, in sweep
        // order.  Pass 2 then runs the exact FP64 test, square root and
        // division on these compact per-particle lists, with nearly all lanes
        // of a warp busy (a candidate survives for only part of a warp).
        int ns = 0;
        for_each_candidate<PLANAR>(c, cs, skey[k], [&](int j) {
            if (j == k || far32<PLANAR>(s, j, fx, fy, fz, c.ft_max)) return;
            if (ns < c.K) nb.slot[(size_t)ns * np + k] = j;
            ns++;
        });
        if (ns <= c.K) {
            // exact test, compacting in place (order kept): src/mps.cpp:585-619
            for (int q = 0; q < ns; q++) {
                const int j = nb.slot[(size_t)q * np + k];
                const double d2 = dist2<PLANAR>(s, k, j, xi, yi, zi);
                if (!lt_cut(d2, c.t_max)) continue;
                const double dist = dsqrt(d2);
                const double w = weight(dist, c.re_p);
                if (lt_cut(dist, c.re_p)) nd = dadd(nd, w);  // src/mps.cpp:573-583
                if (BC && lt_cut(dist, c.re_s)) nsurf = dadd(nsurf, weight(dist, c.re_s));
                const size_t e = (size_t)m * np + k;
                nb.slot[e] = j;
                nb.dist[e] = dist;
                nb.wp[e] = w;
                m++;
            }
        } else {
            // more survivors than the list holds: the exact one-pass sweep
            for_each_candidate<PLANAR>(c, cs, skey[k], [&](int j) {
                if (j == k) return;
                const double d2 = dist2<PLANAR>(s, k, j, xi, yi, zi);
                if (!lt_cut(d2, c.t_max)) return;
                const double dist = dsqrt(d2);
                const double w = weight(dist, c.re_p);
                if (lt_cut(dist, c.re_p)) nd = dadd(nd, w);
                if (m < c.K) {
                    if (BC && lt_cut(dist, c.re_s)) nsurf = dadd(nsurf, weight(dist, c.re_s));
                    const size_t e = (size_t)m * np + k;
                    nb.slot[e] = j;
                    nb.dist[e] = dist;
                    nb.wp[e] = w;
                }
                m++;
            });
        }
        s.nd_last[k] = nd;
    }
    if (k < c.n) nb.cnt[k] = m < c.K ? m : c.K;
    if (m > c.K) raise_status(ds, ST_CAPACITY);
    if (BC) {
        int8_t bc = BC_IGNORED;
        if (k < c.n) {
            const int8_t t = s.type[k];
            if (t != T_GHOST && t != T_DUMMY) bc = nsurf < c.beta_n0s ? BC_SURFACE : BC_INNER;
            s.bc[k] = bc;
            double b = 0.0;
            if (bc == BC_INNER && !c.ho_on) b = ddiv(dmul(c.src_g1, dsub(nd, c.n0_p)), c.n0_p);
            A.src[k] = b;
        }
        const unsigned in_mask = __ballot_sync(0xffffffffu, k < c.n && bc == BC_INNER);
        const unsigned sf_mask = __ballot_sync(0xffffffffu, k < c.n && bc == BC_SURFACE);
        if ((threadIdx.x & 31) == 0) {
            if (in_mask) atomicAdd(&ds->n_inner, __popc(in_mask));
            if (sf_mask) atomicAdd(&ds->n_surface, __popc(sf_mask));
        }
    }
    // one atomic per warp for the largest neighbour count
    const int wmax = __reduce_max_sync(0xffffffffu, m);
    if ((threadIdx.x & 31) == 0 && wmax > 0) atomicMax(&ds->max_neighbors, wmax);
}

// Higher-order source term (src/mps.cpp:288-306), needs every neighbour's BC.
template <bool PLANAR>
__global__ void __launch_bounds__(kThreads) k_source_ho(Consts c, StateBuf s, NbList nb, Ppe A) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c.n || s.bc[k] != BC_INNER) return;
    double b = dmul(c.ho_g1, dsub(s.ndr[k], 1.0));
    const double xi = s.x[k], yi = s.y[k], zi = PLANAR ? 0.0 : s.z[k];
    const double ui = s.vx[k], vi = s.vy[k], wi = PLANAR ? 0.0 : s.vz[k];
    const double cre = dmul(c.ho_c, c.re_p);
    const int np = nb.n_pad, m = nb.cnt[k];
    for (int q = 0; q < m; q++) {
        int j = nb.slot[(size_t)q * np + k];
        if (s.bc[j] == BC_IGNORED) continue;
        double dist = nb.dist[(size_t)q * np + k];
        if (!lt_cut(dist, c.re_p)) continue;
        double rx = dsub(s.x[j], xi), ry = dsub(s.y[j], yi);
        double ux = dsub(s.vx[j], ui), uy = dsub(s.vy[j], vi);
        double dot = dadd(dmul(rx, ux), dmul(ry, uy));
        if (!PLANAR) dot = dadd(dot, dmul(dsub(s.z[j], zi), dsub(s.vz[j], wi)));
        b = dsub(b, ddiv(dmul(cre, dot), dmul(dmul(dist, dist), dist)));
    }
    A.src[k] = b;
}

// MPS::setMatrix (src/mps.cpp:322-360): one SELL-32 row per Inner slot.
__global__ void __launch_bounds__(kThreads) k_assemble(Consts c, StateBuf s, NbList nb, Ppe A,
                                                       DevStats* ds) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    int off = 0;
    if (k < c.n) {
        double diag = 0.0;
        double rsum = 0.0;  // diag + the off-diagonals: the terms of neighbours without an unknown
        if (s.bc[k] == BC_INNER) {
            const int np = nb.n_pad, m = nb.cnt[k];
            const size_t sbase = (size_t)(k >> 5) * c.K * 32 + (k & 31);
            for (int q = 0; q < m; q++) {
                int j = nb.slot[(size_t)q * np + k];
                int8_t bj = s.bc[j];
                if (bj == BC_IGNORED) continue;
                double dist = nb.dist[(size_t)q * np + k];
                if (!lt_cut(dist, c.re_p)) continue;
                double a = ddiv(dmul(c.mat_c, nb.wp[(size_t)q * np + k]), c.rho);
                diag = dadd(diag, a);
                if (bj == BC_INNER) {
                    A.col[sbase + (size_t)off * 32] = j;
                    A.val[sbase + (size_t)off * 32] = -a;
                    off++;
                } else {
                    rsum = dadd(rsum, a);
                }
            }
            if (c.qc_on) {
                diag = dadd(diag, c.qc_term);
                rsum = dadd(rsum, c.qc_term);
            }
        }
        A.diag[k] = diag;
        A.rsum[k] = rsum;
        A.offcnt[k] = off;
    }
    int w = __reduce_max_sync(0xffffffffu, off);
    unsigned tot = __reduce_add_sync(0xffffffffu, (unsigned)off);
    // pad the row to the slice width with (own slot, 0) so that SpMV loops
    // need no per-entry predicate
    if (k < c.n) {
        const size_t sbase = (size_t)(k >> 5) * c.K * 32 + (k & 31);
        for (int m = off; m < w; m++) {
            A.col[sbase + (size_t)m * 32] = k;
            A.val[sbase + (size_t)m * 32] = 0.0;
        }
    }
    if ((threadIdx.x & 31) == 0 && (k >> 5) < (c.n + 31) / 32) {
        A.slice_w[k >> 5] = w;
        if (tot) atomicAdd(&ds->nnz_off, (unsigned long long)tot);
    }
}

// ---------------------------------------------------------------------------
// MPS::ensureDirichletBoundaryConnection (src/mps.cpp:362-415).  The BFS
// from every Surface particle over edges with dist < re_p marks exactly the
// connected components that contain a Surface particle, so it is computed as
// a lock-free union-find over those edges.
constexpr int kUfLimit = 1 << 22;

__device__ int uf_find(int* par, int x, DevStats* ds) {
    volatile int* vp = par;
    for (int it = 0; it < kUfLimit; it++) {
        int p = vp[x];
        if (p == x) return x;
        int gp = vp[p];
        if (gp != p) vp[x] = gp;  // path halving; any ancestor is a valid parent
        x = p;
    }
    raise_status(ds, ST_TIMEOUT);
    return x;
}

__device__ void uf_union(int* par, int a, int b, DevStats* ds) {
    for (int it = 0; it < kUfLimit; it++) {
        a = uf_find(par, a, ds);
        b = uf_find(par, b, ds);
        if (a == b) return;
        if (a < b) {
            int t = a;
            a = b;
            b = t;
        }
        if (atomicCAS(par + a, a, b) == a) return;
    }
    raise_status(ds, ST_TIMEOUT);
}

__global__ void k_cc_init(int n, int* par) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) par[k] = k;
}

// Sampled linking (the Afforest scheme of Sutton et al., 2018): almost every
// particle of a scene belongs to one large component, and its edges need not
// all be processed.  Pass 1 joins each particle to the components of its first
// kCcLinks neighbours within re_p; after full compression, the most frequent
// root of a fixed sample of particles names the large component; pass 2 runs
// every edge of each particle outside it.  Every edge with an endpoint outside
// the large component is then processed from that endpoint (the pressure
// phase's lists are symmetric and hold no ghost: ghosts are in no cell), so
// the components, and every flag derived from them, are those of processing
// all edges.
constexpr int kCcLinks = 2;
constexpr int kCcSamples = 1024;

__global__ void __launch_bounds__(kThreads) k_cc_link(Consts c, StateBuf s, NbList nb, int* par,
                                                      DevStats* ds) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c.n || s.type[k] == T_GHOST) return;
    const int np = nb.n_pad, m = nb.cnt[k];
    int links = 0;
    for (int q = 0; q < m && links < kCcLinks; q++) {
        const size_t o = (size_t)q * np + k;
        if (lt_cut(nb.dist[o], c.re_p)) {
            uf_union(par, k, nb.slot[o], ds);
            links++;
        }
    }
}

// No unions run here, so every find returns the final root.
__global__ void k_cc_compress(int n, int* par, DevStats* ds) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) par[k] = uf_find(par, k, ds);
}

// One block: the most frequent root among kCcSamples evenly spaced
// particles (ties: the smaller root).
__global__ void k_cc_giant(int n, const int* __restrict__ par, int* giant) {
    __shared__ int roots[kCcSamples];
    __shared__ unsigned long long best;
    const int tid = threadIdx.x;
    if (tid == 0) best = 0ull;
    for (int i = tid; i < kCcSamples; i += blockDim.x)
        roots[i] = par[(int)(((long long)i * n) / kCcSamples)];
    __syncthreads();
    for (int i = tid; i < kCcSamples; i += blockDim.x) {
        int cnt = 0;
        for (int j = 0; j < kCcSamples; j++) cnt += roots[j] == roots[i];
        // larger count first, then smaller root
        const unsigned long long key =
            ((unsigned long long)cnt << 32) | (unsigned int)(0x7fffffff - roots[i]);
        atomicMax(&best, key);
    }
    __syncthreads();
    if (tid == 0) *giant = 0x7fffffff - (int)(unsigned int)(best & 0xffffffffull);
}

__global__ void __launch_bounds__(kThreads) k_cc_hook(Consts c, StateBuf s, NbList nb, int* par,
                                                      const int* giant, DevStats* ds) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c.n || s.type[k] == T_GHOST) return;
    // after compression par[k] is k's root, unless a find moved it higher since
    if (((volatile int*)par)[k] == *giant) return;
    const int np = nb.n_pad, m = nb.cnt[k];
    for (int q = 0; q < m; q++) {
        const size_t o = (size_t)q * np + k;
        if (lt_cut(nb.dist[o], c.re_p)) uf_union(par, k, nb.slot[o], ds);
    }
}

__global__ void k_cc_mark(Consts c, StateBuf s, int* par, int8_t* has_surface, DevStats* ds) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c.n) return;
    int r = uf_find(par, k, ds);
    if (s.bc[k] == BC_SURFACE) has_surface[r] = 1;
}

__global__ void k_cc_apply(Consts c, StateBuf s, const int* __restrict__ par,
                           const int8_t* __restrict__ has_surface, Ppe A, DevStats* ds) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c.n) return;
    int r = k;
    for (int it = 0; it < kUfLimit && par[r] != r; it++) r = par[r];  // roots are final here
    int8_t conn = (s.type[k] != T_GHOST && has_surface[r]) ? 1 : 0;
    s.dir[k] = conn;
    if (!conn && s.bc[k] == BC_INNER) {
        A.rsum[k] = dadd(A.rsum[k], A.diag[k]);  // the row sum grows by the old diagonal
        A.diag[k] = dmul(A.diag[k], 2.0);
        atomicAdd(&ds->n_unconnected, 1);
    }
}

// ---------------------------------------------------------------------------
// solvePoissonEquation's scatter + removeNegativePressure (src/mps.cpp:466-479)
__global__ void k_pressure_out(int n, const double* __restrict__ x, double* __restrict__ p,
                               float2* __restrict__ pf, const int32_t* __restrict__ id,
                               double* __restrict__ x_prev, DevStats* ds) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double v = x[k];
    if (!isfinite(v)) atomicOr(&ds->status, ST_NONFINITE);
    const double pv = v < 0.0 ? 0.0 : v;
    p[k] = pv;
    const float ph = f32(pv);
    pf[k] = make_float2(ph, f32(pv - (double)ph));  // pv - ph is exact
    if (x_prev) x_prev[id[k]] = v;
}

// MPS::setMinimumPressure (src/mps.cpp:481-503) for every particle that is
// not Ignored, then MPS::calcPressureGradient (src/mps.cpp:505-533) for the
// fluid ones, which use their own minimum: one kernel, two passes over the
// particle's list (the second mostly from cache).
template <bool PLANAR, bool MIXED>
__global__ void __launch_bounds__(kThreads) k_gradient(Consts c, StateBuf s, NbList nb, double* ax,
                                                       double* ay, double* az) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c.n || s.bc[k] == BC_IGNORED) return;
    const int np = nb.n_pad, m = nb.cnt[k];
    double pmin = s.p[k];
    for (int q = 0; q < m; q++) {
        int j = nb.slot[(size_t)q * np + k];
        if (s.type[j] == T_DUMMY) continue;
        if (lt_cut(nb.dist[(size_t)q * np + k], c.re_p)) {
            double pj = s.p[j];
            if (pmin > pj) pmin = pj;
        }
    }
    s.minp[k] = pmin;
    // a fluid particle is never Ignored (only dummies and ghosts are)
    if (s.type[k] != T_FLUID) return;
    const double xi = s.x[k], yi = s.y[k], zi = PLANAR ? 0.0 : s.z[k];
    if (!MIXED) {
        double gx = 0.0, gy = 0.0, gz = 0.0;
        for (int q = 0; q < m; q++) {
            int j = nb.slot[(size_t)q * np + k];
            if (s.type[j] == T_DUMMY) continue;
            double dist = nb.dist[(size_t)q * np + k];
            if (!lt_cut(dist, c.re_p)) continue;
            double dp = dsub(s.p[j], pmin);
            double w = nb.wp[(size_t)q * np + k];
            double d2 = dmul(dist, dist);
            gx = dadd(gx, ddiv(dmul(dmul(dsub(s.x[j], xi), dp), w), d2));
            gy = dadd(gy, ddiv(dmul(dmul(dsub(s.y[j], yi), dp), w), d2));
            if (!PLANAR) gz = dadd(gz, ddiv(dmul(dmul(dsub(s.z[j], zi), dp), w), d2));
        }
        gx = dmul(gx, c.grad_scale);
        gy = dmul(gy, c.grad_scale);
        ax[k] = ddiv(dmul(-1.0, gx), c.rho);
        ay[k] = ddiv(dmul(-1.0, gy), c.rho);
        if (!PLANAR) az[k] = ddiv(dmul(-1.0, dmul(gz, c.grad_scale)), c.rho);
    } else if (PLANAR) {
        // FP32 throughout: the coordinate and pressure differences from the
        // FP32 pairs (hi, lo), each within FP32 rounding of the exact
        // difference (the FP64 subtractions they replace were most of this
        // kernel's FP64 pipe time)
        float gx = 0.f, gy = 0.f;
        const float2 hk = s.xyf[k], lk = s.xylo[k];
        const float pmh = f32(pmin), pml = f32(pmin - (double)pmh);
        for (int q = 0; q < m; q++) {
            int j = nb.slot[(size_t)q * np + k];
            if (s.type[j] == T_DUMMY) continue;
            double dist = nb.dist[(size_t)q * np + k];
            if (!lt_cut(dist, c.re_p)) continue;
            const float2 hj = s.xyf[j], lj = s.xylo[j], pj = s.pf[j];
            const float fd = f32(dist);
            const float dp = (pj.x - pmh) + (pj.y - pml);
            const float coef = dp * (c.fre_p / fd - 1.f) / (fd * fd);
            gx = fmaf((hj.x - hk.x) + (lj.x - lk.x), coef, gx);
            gy = fmaf((hj.y - hk.y) + (lj.y - lk.y), coef, gy);
        }
        const float sc = -c.fgrad_scale / f32(c.rho);
        ax[k] = (double)(gx * sc);
        ay[k] = (double)(gy * sc);
    } else {
        float gx = 0.f, gy = 0.f, gz = 0.f;
        for (int q = 0; q < m; q++) {
            int j = nb.slot[(size_t)q * np + k];
            if (s.type[j] == T_DUMMY) continue;
            double dist = nb.dist[(size_t)q * np + k];
            if (!lt_cut(dist, c.re_p)) continue;
            float fd = f32(dist);
            float coef = f32(s.p[j] - pmin) * (c.fre_p / fd - 1.f) / (fd * fd);
            gx = fmaf(f32(s.x[j] - xi), coef, gx);
            gy = fmaf(f32(s.y[j] - yi), coef, gy);
            gz = fmaf(f32(s.z[j] - zi), coef, gz);
        }
        const float sc = -c.fgrad_scale / f32(c.rho);
        ax[k] = (double)(gx * sc);
        ay[k] = (double)(gy * sc);
        if (!PLANAR) az[k] = (double)(gz * sc);
    }
}

// moveParticlesWithPressureGradient + checkBoundaryViolation + the Courant
// number (src/mps.cpp:535-571).
template <bool PLANAR>
__global__ void __launch_bounds__(kThreads) k_move2(Consts c, StateBuf s, const double* __restrict__ ax,
                                                    const double* __restrict__ ay,
                                                    const double* __restrict__ az, DevStats* ds) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    double cour = 0.0;  // Courant numbers are >= 0: 0 is neutral for the max
    if (k < c.n && s.type[k] == T_FLUID) {
        double a0 = ax[k], a1 = ay[k];
        double vx = dadd(s.vx[k], dmul(a0, c.dt));
        double vy = dadd(s.vy[k], dmul(a1, c.dt));
        double x = dadd(s.x[k], dmul(dmul(a0, c.dt), c.dt));
        double y = dadd(s.y[k], dmul(dmul(a1, c.dt), c.dt));
        double vz = 0.0, z = c.z0;
        if (!PLANAR) {
            double a2 = az[k];
            vz = dadd(s.vz[k], dmul(a2, c.dt));
            z = dadd(s.z[k], dmul(dmul(a2, c.dt), c.dt));
            s.vz[k] = vz;
            s.z[k] = z;
        }
        s.vx[k] = vx;
        s.vy[k] = vy;
        s.x[k] = x;
        s.y[k] = y;
        if (outside_domain(c, x, y, z)) {
            s.type[k] = T_GHOST;
            atomicAdd(&ds->n_new_ghosts, 1);
        } else {
            double sp = dadd(dadd(dmul(vx, vx), dmul(vy, vy)), dmul(vz, vz));
            cour = ddiv(dmul(dsqrt(sp), c.dt), c.l0);
        }
    }
    // one atomic per warp instead of one per particle
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cour = fmax(cour, __shfl_xor_sync(0xffffffffu, cour, o));
    if ((threadIdx.x & 31) == 0 && cour > 0.0) atomic_max_nonneg_double(&ds->courant_bits, cour);
}

// MPS::setNumberDensity's ratio (src/mps.cpp:627-641)
__global__ void k_number_density(Consts c, StateBuf s) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c.n) return;
    s.ndr[k] = s.bc[k] == BC_SURFACE ? 0.0 : ddiv(s.nd_last[k], c.n0_p);
}

}  // namespace

// ------------------------------------------------------------------ launchers

void launch_explicit(const Consts& c, const StateBuf& in, const StateBuf& out,
                     const SortScratch& sc, int mixed, DevStats* ds, cudaStream_t st) {
    int nb = blocks_for(c.n);
    if (c.planar) {
        if (mixed) {
            k_explicit<true, true><<<nb, kThreads, 0, st>>>(c, in, out, sc.skey, sc.cell_start, ds);
            ++g_launches;
        } else {
            k_explicit<true, false><<<nb, kThreads, 0, st>>>(c, in, out, sc.skey, sc.cell_start, ds);
            ++g_launches;
        }
    } else {
        if (mixed) {
            k_explicit<false, true><<<nb, kThreads, 0, st>>>(c, in, out, sc.skey, sc.cell_start, ds);
            ++g_launches;
        } else {
            k_explicit<false, false><<<nb, kThreads, 0, st>>>(c, in, out, sc.skey, sc.cell_start, ds);
            ++g_launches;
        }
    }
}

void launch_collision(const Consts& c, const StateBuf& s, const SortScratch& sc,
                      int32_t* cand_cnt, int32_t* cand_base, const CollWork& cw, CollPair* pairs,
                      int32_t pair_cap, int32_t* scan_tmp, DevStats* ds, cudaStream_t st) {
    int nb = blocks_for(c.n);
    cudaMemsetAsync(cand_cnt, 0, sizeof(int32_t) * (c.n + 1), st);
    if (c.planar) {
        k_coll_count<true><<<nb, kThreads, 0, st>>>(c, s, sc.skey, sc.cell_start, cand_cnt);
        ++g_launches;
    } else {
        k_coll_count<false><<<nb, kThreads, 0, st>>>(c, s, sc.skey, sc.cell_start, cand_cnt);
        ++g_launches;
    }
    launch_exclusive_scan(cand_cnt, cand_base, c.n, scan_tmp, st);
    const int32_t* total = cand_base + c.n;
    if (c.planar) {
        k_coll_write<true><<<nb, kThreads, 0, st>>>(c, s, sc.skey, sc.cell_start, cand_cnt,
                                                    cand_base, pairs, pair_cap, ds);
    } else {
        k_coll_write<false><<<nb, kThreads, 0, st>>>(c, s, sc.skey, sc.cell_start, cand_cnt,
                                                     cand_base, pairs, pair_cap, ds);
    }
    ++g_launches;
    if (!cw.serial) {
        cudaMemsetAsync(cw.jn, 0, sizeof(int32_t) * c.n, st);
        cudaMemsetAsync(cw.ver, 0, sizeof(int32_t) * c.n, st);
        cudaMemsetAsync(cw.ctl, 0, sizeof(int32_t) * 4, st);
        k_coll_jlists<<<kCollBlocks, kThreads, 0, st>>>(s, pairs, total, pair_cap, cw);
        if (c.planar)
            k_coll_wave<true><<<kCollBlocks, kThreads, 0, st>>>(c, s, pairs, total, pair_cap, cand_cnt,
                                                                cand_base, cw, ds);
        else
            k_coll_wave<false><<<kCollBlocks, kThreads, 0, st>>>(c, s, pairs, total, pair_cap, cand_cnt,
                                                                 cand_base, cw, ds);
        g_launches += 2;
    }
    if (c.planar)
        k_coll_apply<true><<<1, 1, 0, st>>>(c, s, pairs, total, pair_cap, cw, ds);
    else
        k_coll_apply<false><<<1, 1, 0, st>>>(c, s, pairs, total, pair_cap, cw, ds);
    ++g_launches;
}

void launch_build_list(const Consts& c, const StateBuf& s, const SortScratch& sc,
                       const NbList& nb, DevStats* ds, cudaStream_t st) {
    int g = blocks_for(c.n);
    const Ppe none{};
    if (c.planar) {
        k_build_list<true, false><<<g, kThreads, 0, st>>>(c, s, sc.skey, sc.cell_start, nb, none, ds);
        ++g_launches;
    } else {
        k_build_list<false, false><<<g, kThreads, 0, st>>>(c, s, sc.skey, sc.cell_start, nb, none, ds);
        ++g_launches;
    }
}

void launch_build_list_bc_source(const Consts& c, const StateBuf& s, const SortScratch& sc,
                                 const NbList& nb, const Ppe& A, DevStats* ds, cudaStream_t st) {
    int g = blocks_for(c.n);
    if (c.planar) {
        k_build_list<true, true><<<g, kThreads, 0, st>>>(c, s, sc.skey, sc.cell_start, nb, A, ds);
        ++g_launches;
    } else {
        k_build_list<false, true><<<g, kThreads, 0, st>>>(c, s, sc.skey, sc.cell_start, nb, A, ds);
        ++g_launches;
    }
    if (c.ho_on) {
        if (c.planar) {
            k_source_ho<true><<<g, kThreads, 0, st>>>(c, s, nb, A);
            ++g_launches;
        } else {
            k_source_ho<false><<<g, kThreads, 0, st>>>(c, s, nb, A);
            ++g_launches;
        }
    }
}

void launch_assemble(const Consts& c, const StateBuf& s, const NbList& nb, const Ppe& A,
                     DevStats* ds, cudaStream_t st) {
    k_assemble<<<blocks_for(c.n), kThreads, 0, st>>>(c, s, nb, A, ds);
    ++g_launches;
}

void launch_dirichlet(const Consts& c, const StateBuf& s, const NbList& nb, const Ppe& A,
                      int32_t* parent, int8_t* has_surface, DevStats* ds, cudaStream_t st) {
    int g = blocks_for(c.n);
    cudaMemsetAsync(has_surface, 0, c.n, st);
    int* giant = parent + c.n;  // the parent array has one spare element
    k_cc_init<<<g, kThreads, 0, st>>>(c.n, parent);
    ++g_launches;
    k_cc_link<<<g, kThreads, 0, st>>>(c, s, nb, parent, ds);
    ++g_launches;
    k_cc_compress<<<g, kThreads, 0, st>>>(c.n, parent, ds);
    ++g_launches;
    k_cc_giant<<<1, 1024, 0, st>>>(c.n, parent, giant);
    ++g_launches;
    k_cc_hook<<<g, kThreads, 0, st>>>(c, s, nb, parent, giant, ds);
    ++g_launches;
    k_cc_mark<<<g, kThreads, 0, st>>>(c, s, parent, has_surface, ds);
    ++g_launches;
    k_cc_apply<<<g, kThreads, 0, st>>>(c, s, parent, has_surface, A, ds);
    ++g_launches;
}

void launch_pressure_post(const Consts& c, const StateBuf& s, const NbList& nb, const double* x,
                          double* x_prev, double* ax, double* ay, double* az, int mixed,
                          DevStats* ds, cudaStream_t st) {
    int g = blocks_for(c.n);
    k_pressure_out<<<g, kThreads, 0, st>>>(c.n, x, s.p, s.pf, s.id, x_prev, ds);
    ++g_launches;
    if (c.planar) {
        if (mixed) {
            k_gradient<true, true><<<g, kThreads, 0, st>>>(c, s, nb, ax, ay, az);
            ++g_launches;
        } else {
            k_gradient<true, false><<<g, kThreads, 0, st>>>(c, s, nb, ax, ay, az);
            ++g_launches;
        }
        k_move2<true><<<g, kThreads, 0, st>>>(c, s, ax, ay, az, ds);
        ++g_launches;
    } else {
        if (mixed) {
            k_gradient<false, true><<<g, kThreads, 0, st>>>(c, s, nb, ax, ay, az);
            ++g_launches;
        } else {
            k_gradient<false, false><<<g, kThreads, 0, st>>>(c, s, nb, ax, ay, az);
            ++g_launches;
        }
        k_move2<false><<<g, kThreads, 0, st>>>(c, s, ax, ay, az, ds);
        ++g_launches;
    }
}

void launch_number_density(const Consts& c, const StateBuf& s, const NbList& /*nb*/,
                           cudaStream_t st) {
    k_number_density<<<blocks_for(c.n), kThreads, 0, st>>>(c, s);
    ++g_launches;
}

void launch_initial_number_density(const Consts& c, const StateBuf& s, const SortScratch& sc,
                                   const NbList& nb, DevStats* ds, cudaStream_t st) {
    launch_build_list(c, s, sc, nb, ds, st);
    launch_number_density(c, s, nb, st);
}

}  // namespace mpsg
