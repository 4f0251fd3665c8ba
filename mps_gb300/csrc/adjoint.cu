// Differentiable trajectories: many MPS steps from one initial condition,
// with a hand-written adjoint (reverse mode) of the whole step.  No
// counterpart in the reference, whose step is not differentiated.
//
// What is differentiated.  A trajectory maps the initial velocities (and
// positions) and the gravity vector to (a) the pressure at chosen sensor
// particles after every step and (b) the final positions and velocities.
// The discrete structure of each step is frozen at its forward values:
// neighbour sets, particle types (ghosts), boundary conditions (surface
// flags), Dirichlet connections, the collision candidate list and which
// candidates fired, the removeNegativePressure mask and the particle that
// attains setMinimumPressure's minimum.  Everything else — weights, the
// viscosity sum, the collision impulses, the number-density source term,
// every PPE matrix entry, the Poisson solve, the pressure gradient and the
// moves — is differentiated exactly.
//
// Memory: checkpoints (positions, velocities, types) every `every` steps;
// the backward pass re-runs each segment forward with a tape attached to
// the engine (tape_phase, called from the step at its phase boundaries) and
// then walks the segment's steps in reverse.  All adjoint arrays are in
// particle-id order; per-particle sums gather over the (symmetric)
// neighbour lists instead of scattering, so they need no atomics.
//
// Reverse step (forward order: explicit, collision, pressure, move):
//   move        a_bar = dt v_bar + dt^2 x_bar            (fluid)
//   gradient    a_i = Kg sum_j r_ij (p+_j - phat_i) w(d)/d^2, Kg = -(D/n0)/rho
//   min press.  phat_bar goes to the particle that attained the minimum
//   clamp       p_bar = p+_bar where the solution was > 0
//   PPE         lambda = A^-1 p_bar (A is symmetric); b_bar = lambda,
//               A_bar = -lambda p^T on the stored entries -> weight adjoints
//   source      b_i = gamma/dt^2 (n_i - n0)/n0 -> n_bar -> weight adjoints
//   collision   the serial pass replayed forward, then reversed pair by pair
//   explicit    v1 = v0 + dt (g + V sum_j (v0_j - v0_i) w(d)), x1 = x0 + dt v1
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "devutil.cuh"
#include "engine_impl.cuh"

using namespace mpsg;

namespace mpsg {
namespace {

constexpr int kT = 256;
inline int nblk(int n) { return (n + kT - 1) / kT; }

struct Arr3 {
    double* p[3];
};
struct Arr6 {
    double* p[6];
};

Arr6 arr6(double* const* a) { return Arr6{{a[0], a[1], a[2], a[3], a[4], a[5]}}; }

// ------------------------------------------------------------ tape kernels
// slot-order state -> id-order arrays (planar engines keep z = z0, v_z = 0)
__global__ void k_tape_state(int n, const int32_t* __restrict__ id, StateBuf s, int planar,
                             double z0, Arr6 o, int8_t* __restrict__ type_out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = id[k];
    o.p[0][i] = s.x[k];
    o.p[1][i] = s.y[k];
    o.p[2][i] = planar ? z0 : s.z[k];
    o.p[3][i] = s.vx[k];
    o.p[4][i] = s.vy[k];
    o.p[5][i] = planar ? 0.0 : s.vz[k];
    if (type_out) type_out[i] = s.type[k];
}

// id-order arrays -> slot-order state (positions, velocities, types)
__global__ void k_restore_state(int n, const int32_t* __restrict__ id, StateBuf s, int planar,
                                Arr6 src, const int8_t* __restrict__ type_src) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = id[k];
    s.x[k] = src.p[0][i];
    s.y[k] = src.p[1][i];
    s.vx[k] = src.p[3][i];
    s.vy[k] = src.p[4][i];
    if (!planar) {
        s.z[k] = src.p[2][i];
        s.vz[k] = src.p[5][i];
    }
    s.type[k] = type_src[i];
}

__global__ void k_tape_list(int n, int np, const int32_t* __restrict__ id,
                            const int32_t* __restrict__ cnt, const int32_t* __restrict__ slot,
                            int32_t* __restrict__ ocnt, int32_t* __restrict__ oid) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = id[k], m = cnt[k];
    ocnt[i] = m;
    for (int q = 0; q < m; q++) oid[(size_t)q * n + i] = id[slot[(size_t)q * np + k]];
}

__global__ void k_tape_pairs(const CollPair* __restrict__ pairs, const int32_t* __restrict__ total_p,
                             int32_t src_cap, CollPair* __restrict__ out, int32_t* __restrict__ nout,
                             int32_t cap, DevStats* ds) {
    int32_t total = *total_p;
    if (total > src_cap) total = src_cap;
    if (total > cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(&ds->status, ST_CAPACITY);
        total = cap;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *nout = total;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x)
        out[t] = pairs[t];
}

__global__ void k_tape_solve(int n, const int32_t* __restrict__ id, const double* __restrict__ x,
                             const int8_t* __restrict__ bc, const int8_t* __restrict__ dir,
                             double* __restrict__ praw, int8_t* __restrict__ obc,
                             int8_t* __restrict__ odir) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int i = id[k];
    praw[i] = x[k];
    obc[i] = bc[k];
    odir[i] = dir[k];
}

__global__ void k_to_id(int n, const int32_t* __restrict__ id, const double* __restrict__ src,
                        double* __restrict__ dst) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) dst[id[k]] = src[k];
}

__global__ void k_pick(int m, const int32_t* __restrict__ sid, const double* __restrict__ v,
                       double* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < m) out[k] = v[sid[k]];
}

// ------------------------------------------------------------ adjoint kernels
__device__ __forceinline__ double d2_of(const double* const* x, int i, int j) {
    // exact FP64 squared distance in the forward's order, (dx^2 + dy^2) + dz^2
    const double dx = dsub(x[0][j], x[0][i]), dy = dsub(x[1][j], x[1][i]),
                 dz = dsub(x[2][j], x[2][i]);
    return dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
}

// move: a_bar = dt v_bar + dt^2 x_bar for particles the move displaced
__global__ void k_adj_move(int n, double dt, int planar, const int8_t* __restrict__ type1,
                           Arr3 xb, Arr3 vb, Arr3 ab) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool f = type1[i] == T_FLUID;
    for (int d = 0; d < 3; d++)
        ab.p[d][i] = (f && !(planar && d == 2)) ? dt * vb.p[d][i] + dt * dt * xb.p[d][i] : 0.0;
}

__global__ void k_adj_pplus(int n, const double* __restrict__ praw, double* __restrict__ pplus) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) pplus[i] = praw[i] < 0.0 ? 0.0 : praw[i];
}

// setMinimumPressure replayed: value and the particle attaining it
__global__ void k_adj_minp(int n, Consts c, TapeStep t, const double* __restrict__ pplus,
                           double* __restrict__ phat, int32_t* __restrict__ amin) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (t.bc[i] == BC_IGNORED) {
        phat[i] = 0.0;
        amin[i] = -1;
        return;
    }
    double mn = pplus[i];
    int arg = i;
    const int m = t.l2cnt[i];
    for (int q = 0; q < m; q++) {
        const int j = t.l2id[(size_t)q * n + i];
        if (t.type1[j] == T_DUMMY) continue;
        if (d2_of(t.st2, i, j) < c.t_p && mn > pplus[j]) {
            mn = pplus[j];
            arg = j;
        }
    }
    phat[i] = mn;
    amin[i] = arg;
}

// phat_bar_i = -Kg sum_j (a_bar_i . r_ij) w(d)/d^2
__global__ void k_adj_grad_local(int n, Consts c, TapeStep t, Arr3 ab, double* __restrict__ phatbar) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (t.type1[i] != T_FLUID) {
        phatbar[i] = 0.0;
        return;
    }
    const double Kg = -c.grad_scale / c.rho;
    const double a0 = ab.p[0][i], a1 = ab.p[1][i], a2 = ab.p[2][i];
    double s = 0.0;
    const int m = t.l2cnt[i];
    for (int q = 0; q < m; q++) {
        const int j = t.l2id[(size_t)q * n + i];
        if (t.type1[j] == T_DUMMY) continue;
        const double d2 = d2_of(t.st2, i, j);
        if (!(d2 < c.t_p)) continue;
        const double d = sqrt(d2);
        const double phi = (c.re_p / d - 1.0) / d2;
        const double r0 = t.st2[0][j] - t.st2[0][i], r1 = t.st2[1][j] - t.st2[1][i],
                     r2 = t.st2[2][j] - t.st2[2][i];
        s += (a0 * r0 + a1 * r1 + a2 * r2) * phi;
    }
    phatbar[i] = -Kg * s;
}

// x_bar += gradient-term adjoints (both sides of every pair); p+_bar from
// the gradient sums of the neighbours and from the minima this particle set.
__global__ void k_adj_grad_gather(int n, Consts c, TapeStep t, const double* __restrict__ pplus,
                                  const double* __restrict__ phat, Arr3 ab,
                                  const double* __restrict__ phatbar, const int32_t* __restrict__ amin,
                                  Arr3 xb, double* __restrict__ pbar) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double accp = amin[i] == i ? phatbar[i] : 0.0;
    if (t.type1[i] == T_GHOST) {
        pbar[i] = accp;
        return;
    }
    const double Kg = -c.grad_scale / c.rho;
    const bool fi = t.type1[i] == T_FLUID, di = t.type1[i] == T_DUMMY;
    const double ai0 = ab.p[0][i], ai1 = ab.p[1][i], ai2 = ab.p[2][i];
    double g0 = 0.0, g1 = 0.0, g2 = 0.0;
    const int m = t.l2cnt[i];
    for (int q = 0; q < m; q++) {
        const int j = t.l2id[(size_t)q * n + i];
        const double d2 = d2_of(t.st2, i, j);
        if (!(d2 < c.t_p)) continue;
        if (amin[j] == i) accp += phatbar[j];
        const bool fj = t.type1[j] == T_FLUID, dj = t.type1[j] == T_DUMMY;
        const double d = sqrt(d2);
        const double phi = (c.re_p / d - 1.0) / d2;
        const double dphi_over_d = (-3.0 * c.re_p / (d2 * d2) + 2.0 / (d2 * d)) / d;
        const double r0 = t.st2[0][j] - t.st2[0][i], r1 = t.st2[1][j] - t.st2[1][i],
                     r2 = t.st2[2][j] - t.st2[2][i];
        if (fi && !dj) {  // a_i's term for j: x_i enters through r_ij = x_j - x_i
            const double qv = pplus[j] - phat[i];
            const double rv = r0 * ai0 + r1 * ai1 + r2 * ai2;
            const double s = Kg * qv;
            g0 -= s * (phi * ai0 + dphi_over_d * rv * r0);
            g1 -= s * (phi * ai1 + dphi_over_d * rv * r1);
            g2 -= s * (phi * ai2 + dphi_over_d * rv * r2);
        }
        if (fj && !di) {  // a_j's term for i: r_ji = -r_ij, and p+_i enters through q_ji
            const double aj0 = ab.p[0][j], aj1 = ab.p[1][j], aj2 = ab.p[2][j];
            const double qv = pplus[i] - phat[j];
            const double rv = r0 * aj0 + r1 * aj1 + r2 * aj2;
            const double s = Kg * qv;
            g0 += s * (phi * aj0 + dphi_over_d * rv * r0);
            g1 += s * (phi * aj1 + dphi_over_d * rv * r1);
            g2 += s * (phi * aj2 + dphi_over_d * rv * r2);
            accp -= Kg * rv * phi;
        }
    }
    xb.p[0][i] += g0;
    xb.p[1][i] += g1;
    xb.p[2][i] += g2;
    pbar[i] = accp;
}

__global__ void k_adj_sensor(int m, const int32_t* __restrict__ sid, const double* __restrict__ ds_,
                             double* __restrict__ pbar) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < m) atomicAdd(pbar + sid[k], ds_[k]);
}

// The PPE of this step in id order (rows = particle ids, SELL-32 like the
// engine's), right-hand side = the clamp-masked pressure adjoint.
__global__ void k_adj_assemble(int n, Consts c, TapeStep t, const double* __restrict__ pbar,
                               Ppe A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int off = 0;
    if (i < n) {
        double diag = 0.0;
        const bool inner = t.bc[i] == BC_INNER;
        if (inner) {
            const size_t sbase = (size_t)(i >> 5) * c.K * 32 + (i & 31);
            const int m = t.l2cnt[i];
            for (int q = 0; q < m; q++) {
                const int j = t.l2id[(size_t)q * n + i];
                const int8_t bj = t.bc[j];
                if (bj == BC_IGNORED) continue;
                const double d2 = d2_of(t.st2, i, j);
                if (!(d2 < c.t_p)) continue;
                const double a = ddiv(dmul(c.mat_c, weight(dsqrt(d2), c.re_p)), c.rho);
                diag = dadd(diag, a);
                if (bj == BC_INNER && off < c.K) {
                    A.col[sbase + (size_t)off * 32] = j;
                    A.val[sbase + (size_t)off * 32] = -a;
                    off++;
                }
            }
            if (c.qc_on) diag = dadd(diag, c.qc_term);
            if (!t.dir[i]) diag = dmul(diag, 2.0);
        }
        A.diag[i] = diag;
        A.offcnt[i] = off;
        A.src[i] = (inner && t.praw[i] > 0.0) ? pbar[i] : 0.0;
    }
    const int w = __reduce_max_sync(0xffffffffu, off);
    if (i < n) {
        const size_t sbase = (size_t)(i >> 5) * c.K * 32 + (i & 31);
        for (int m = off; m < w; m++) {
            A.col[sbase + (size_t)m * 32] = i;
            A.val[sbase + (size_t)m * 32] = 0.0;
        }
    }
    if ((threadIdx.x & 31) == 0 && (i >> 5) < (n + 31) / 32) A.slice_w[i >> 5] = w;
}

// x_bar from lambda: source term and matrix entries, both sides of a pair.
__global__ void k_adj_ppe_gather(int n, Consts c, TapeStep t, const double* __restrict__ lam,
                                 Arr3 xb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || t.type1[i] == T_GHOST) return;
    const double cm = c.mat_c / c.rho, ks = c.src_g1 / c.n0_p;
    const int8_t bi = t.bc[i];
    const bool ii = bi == BC_INNER;
    const double li = ii ? lam[i] : 0.0, pi = t.praw[i];
    const double si = (ii && !t.dir[i]) ? 2.0 : 1.0;
    double g0 = 0.0, g1 = 0.0, g2 = 0.0;
    const int m = t.l2cnt[i];
    for (int q = 0; q < m; q++) {
        const int j = t.l2id[(size_t)q * n + i];
        const double d2 = d2_of(t.st2, i, j);
        if (!(d2 < c.t_p)) continue;
        const int8_t bj = t.bc[j];
        const bool jj = bj == BC_INNER;
        double W = 0.0;
        if (ii) {
            W += li * ks;
            if (bj != BC_IGNORED) W -= li * pi * si * cm;
            if (jj) W += li * t.praw[j] * cm;
        }
        if (jj) {
            const double lj = lam[j], pj = t.praw[j];
            const double sj = t.dir[j] ? 1.0 : 2.0;
            W += lj * ks;
            if (bi != BC_IGNORED) W -= lj * pj * sj * cm;
            if (ii) W += lj * pi * cm;
        }
        if (W == 0.0) continue;
        const double d = sqrt(d2);
        const double coef = W * (-c.re_p / d2) / d;  // W w'(d) / d
        g0 -= coef * (t.st2[0][j] - t.st2[0][i]);
        g1 -= coef * (t.st2[1][j] - t.st2[1][i]);
        g2 -= coef * (t.st2[2][j] - t.st2[2][i]);
    }
    xb.p[0][i] += g0;
    xb.p[1][i] += g1;
    xb.p[2][i] += g2;
}

__global__ void k_copy6(int n, Arr6 src, Arr6 dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int d = 0; d < 6; d++) dst.p[d][i] = src.p[d][i];
}

__global__ void k_zero3(int n, Arr3 a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        for (int d = 0; d < 3; d++) a.p[d][i] = 0.0;
}

__global__ void k_add3(int n, Arr3 src, Arr3 dst) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        for (int d = 0; d < 3; d++) dst.p[d][i] += src.p[d][i];
}

// MPS::collision replayed on a copy of the pre-collision state (cur), then
// reversed pair by pair.  One thread: the pass is serial in the forward too.
// rec holds per pair the pre-pair state of i and j (x_i, x_j, v_i, v_j) and
// whether the impulse fired.
__global__ void k_adj_collision(int n, Consts c, TapeStep t, Arr6 cur, double* __restrict__ rec,
                                Arr3 xb, Arr3 vb, Arr3 xextra) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const int np_ = *t.npairs;
    const double inv_rho = ddiv(1.0, c.rho);
    for (int q = 0; q < np_; q++) {
        const CollPair pr = t.pairs[q];
        const int i = pr.ii, j = pr.ij;
        double* R = rec + (size_t)q * 13;
        for (int d = 0; d < 3; d++) {
            R[d] = cur.p[d][i];
            R[3 + d] = cur.p[d][j];
            R[6 + d] = cur.p[3 + d][i];
            R[9 + d] = cur.p[3 + d][j];
        }
        const double inv_i = inv_rho, inv_j = t.type1[j] == T_FLUID ? inv_rho : 0.0;
        const double reduced = ddiv(1.0, dadd(inv_i, inv_j));
        const double dx = dsub(cur.p[0][j], cur.p[0][i]), dy = dsub(cur.p[1][j], cur.p[1][i]),
                     dz = dsub(cur.p[2][j], cur.p[2][i]);
        const double z2 = dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
        double nx = dx, ny = dy, nz = dz;
        if (z2 > 0.0) {
            const double r = dsqrt(z2);
            nx = ddiv(dx, r);
            ny = ddiv(dy, r);
            nz = ddiv(dz, r);
        }
        const double ux = dsub(cur.p[3][j], cur.p[3][i]), uy = dsub(cur.p[4][j], cur.p[4][i]),
                     uz = dsub(cur.p[5][j], cur.p[5][i]);
        const double rel = dadd(dadd(dmul(ux, nx), dmul(uy, ny)), dmul(uz, nz));
        R[12] = rel < 0.0 ? 1.0 : 0.0;
        if (rel < 0.0) {
            const double impulse = dmul(dmul(-dadd(1.0, c.e), rel), reduced);
            const double ci = dmul(impulse, inv_i), cj = dmul(impulse, inv_j);
            const double pimp = dmul(dsub(c.cd, pr.dist), reduced);
            const double pi_ = dmul(pimp, inv_i), pj_ = dmul(pimp, inv_j);
            const double nn[3] = {nx, ny, nz};
            for (int d = 0; d < 3; d++) {
                cur.p[3 + d][i] = dsub(cur.p[3 + d][i], dmul(ci, nn[d]));
                cur.p[3 + d][j] = dadd(cur.p[3 + d][j], dmul(cj, nn[d]));
                cur.p[d][i] = dsub(cur.p[d][i], dmul(pi_, nn[d]));
                cur.p[d][j] = dadd(cur.p[d][j], dmul(pj_, nn[d]));
            }
        }
    }
    for (int q = np_ - 1; q >= 0; q--) {
        const double* R = rec + (size_t)q * 13;
        if (R[12] == 0.0) continue;
        const CollPair pr = t.pairs[q];
        const int i = pr.ii, j = pr.ij;
        const double inv_i = inv_rho, inv_j = t.type1[j] == T_FLUID ? inv_rho : 0.0;
        const double m = 1.0 / (inv_i + inv_j);
        double r[3], u[3], nrm[3];
        for (int d = 0; d < 3; d++) {
            r[d] = R[3 + d] - R[d];
            u[d] = R[9 + d] - R[6 + d];
        }
        const double L = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        for (int d = 0; d < 3; d++) nrm[d] = L > 0.0 ? r[d] / L : r[d];
        const double rel = u[0] * nrm[0] + u[1] * nrm[1] + u[2] * nrm[2];
        const double I = -(1.0 + c.e) * rel * m;
        const double P = (c.cd - pr.dist) * m;
        double Xi[3], Xj[3], Vi[3], Vj[3], dv[3], dx[3];
        for (int d = 0; d < 3; d++) {
            Xi[d] = xb.p[d][i];
            Xj[d] = xb.p[d][j];
            Vi[d] = vb.p[d][i];
            Vj[d] = vb.p[d][j];
            dv[d] = -inv_i * Vi[d] + inv_j * Vj[d];
            dx[d] = -inv_i * Xi[d] + inv_j * Xj[d];
        }
        const double Ib = dv[0] * nrm[0] + dv[1] * nrm[1] + dv[2] * nrm[2];
        const double Pb = dx[0] * nrm[0] + dx[1] * nrm[1] + dx[2] * nrm[2];
        double nb[3];
        const double relb = -(1.0 + c.e) * m * Ib;
        for (int d = 0; d < 3; d++) nb[d] = I * dv[d] + P * dx[d] + relb * u[d];
        // stale distance: d_s = |x1_j - x1_i| at the collision pass's start
        const double dsb = -m * Pb;
        double rs[3];
        for (int d = 0; d < 3; d++) rs[d] = t.st1[d][j] - t.st1[d][i];
        const double Ls = sqrt(rs[0] * rs[0] + rs[1] * rs[1] + rs[2] * rs[2]);
        double rb[3] = {0.0, 0.0, 0.0};
        if (L > 0.0) {
            const double nn = nb[0] * nrm[0] + nb[1] * nrm[1] + nb[2] * nrm[2];
            for (int d = 0; d < 3; d++) rb[d] = (nb[d] - nn * nrm[d]) / L;
        }
        for (int d = 0; d < 3; d++) {
            const double ub = relb * nrm[d];
            xb.p[d][i] = Xi[d] - rb[d];
            xb.p[d][j] = Xj[d] + rb[d];
            vb.p[d][i] = Vi[d] - ub;
            vb.p[d][j] = Vj[d] + ub;
            if (Ls > 0.0) {
                xextra.p[d][j] += dsb * rs[d] / Ls;
                xextra.p[d][i] -= dsb * rs[d] / Ls;
            }
        }
    }
}

// explicit part, per particle: total velocity adjoint vt and a_bar = dt vt
__global__ void k_adj_explicit_local(int n, double dt, int planar, const int8_t* __restrict__ type0,
                                     Arr3 xb, Arr3 vb, Arr3 vt, Arr3 ab) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const bool f = type0[i] == T_FLUID;
    for (int d = 0; d < 3; d++) {
        const bool moves = f && !(planar && d == 2);
        const double v = moves ? vb.p[d][i] + dt * xb.p[d][i] : vb.p[d][i];
        vt.p[d][i] = v;
        ab.p[d][i] = moves ? dt * v : 0.0;
    }
}

// g_bar += sum of a_bar over all particles (fixed order: deterministic)
__global__ void k_adj_gsum(int n, Arr3 ab, double* __restrict__ gbar) {
    __shared__ double sh[3][1024];
    double s[3] = {0.0, 0.0, 0.0};
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        for (int d = 0; d < 3; d++) s[d] += ab.p[d][i];
    for (int d = 0; d < 3; d++) sh[d][threadIdx.x] = s[d];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int d = 0; d < 3; d++) sh[d][threadIdx.x] += sh[d][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int d = 0; d < 3; d++) gbar[d] += sh[d][0];
}

// explicit part, gathered over the step-start neighbour list: viscosity
// velocity adjoints and weight (position) adjoints, both sides of a pair.
__global__ void k_adj_explicit_gather(int n, Consts c, TapeStep t, Arr3 ab, Arr3 vt, Arr3 xb,
                                      Arr3 vb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double va[3] = {vt.p[0][i], vt.p[1][i], vt.p[2][i]};
    if (t.type0[i] == T_GHOST) {
        for (int d = 0; d < 3; d++) vb.p[d][i] = va[d];
        return;
    }
    const bool fi = t.type0[i] == T_FLUID;
    const double V = c.visc_a;
    const double ai[3] = {ab.p[0][i], ab.p[1][i], ab.p[2][i]};
    double g[3] = {0.0, 0.0, 0.0};
    const int m = t.l0cnt[i];
    for (int q = 0; q < m; q++) {
        const int j = t.l0id[(size_t)q * n + i];
        const double d2 = d2_of(t.st0, i, j);
        if (!(d2 < c.t_v)) continue;
        const bool fj = t.type0[j] == T_FLUID;
        if (!fi && !fj) continue;
        const double d = sqrt(d2);
        const double w = c.re_v / d - 1.0;
        double W = 0.0;
        for (int dd = 0; dd < 3; dd++) {
            const double aj = fj ? ab.p[dd][j] : 0.0;
            const double du = t.st0[3 + dd][j] - t.st0[3 + dd][i];
            va[dd] += V * w * (aj - (fi ? ai[dd] : 0.0));
            if (fi) W += V * ai[dd] * du;
            if (fj) W -= V * aj * du;
        }
        const double coef = W * (-c.re_v / d2) / d;
        for (int dd = 0; dd < 3; dd++) g[dd] -= coef * (t.st0[dd][j] - t.st0[dd][i]);
    }
    for (int d = 0; d < 3; d++) {
        vb.p[d][i] = va[d];
        xb.p[d][i] += g[d];
    }
}

__global__ void k_interleave3(int n, Arr3 a, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        for (int d = 0; d < 3; d++) out[(size_t)3 * i + d] = a.p[d][i];
}
__global__ void k_deinterleave3(int n, const double* __restrict__ in, Arr3 a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        for (int d = 0; d < 3; d++) a.p[d][i] = in[(size_t)3 * i + d];
}

}  // namespace
}  // namespace mpsg

// ------------------------------------------------------------------ host side

struct mps_trajectory {
    mps_engine* e = nullptr;
    int n = 0, steps = 0, every = 0, nseg = 0, nsens = 0;
    double* ic[6]{};          // initial positions/velocities (id order)
    int8_t* ic_type = nullptr;
    std::vector<double*> ck;  // checkpoint s: ck[6 s + d]
    std::vector<int8_t*> ckt;
    double* fin[6]{};         // final state of the last forward
    int8_t* fin_type = nullptr;
    int32_t* sensor = nullptr;
    double* sens_out = nullptr;   // steps x nsens
    double* sens_bar = nullptr;   // steps x nsens
    double* idp = nullptr;
    std::vector<TapeStep> tape;
    // adjoint work arrays (id order)
    double *xb[3]{}, *vb[3]{}, *ab[3]{}, *vt[3]{}, *xextra[3]{}, *cur[6]{};
    double *pplus = nullptr, *phat = nullptr, *phatbar = nullptr, *pbar = nullptr;
    int32_t* amin = nullptr;
    double* rec = nullptr;
    double* gbar = nullptr;
    double* hstage = nullptr;  // 3 n host doubles
    double g_fwd[3]{};
    bool forward_done = false;
    std::vector<void*> allocs;

    template <typename T>
    cudaError_t alloc(T** p, size_t count) {
        void* q = nullptr;
        cudaError_t er = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
        if (er == cudaSuccess) {
            allocs.push_back(q);
            *p = (T*)q;
        }
        return er;
    }
};

namespace mpsg {

void tape_phase(mps_engine* e, TapePhase ph) {
    const TapeStep& t = *e->tape;
    const Consts& c = e->c;
    const int n = e->n;
    cudaStream_t st = e->st;
    StateBuf& s = e->S();
    switch (ph) {
        case TAPE_START:
            k_tape_state<<<nblk(n), kT, 0, st>>>(n, s.id, s, c.planar, c.z0, arr6(t.st0), t.type0);
            break;
        case TAPE_LIST0:
            launch_build_list(c, s, e->sc, e->nb, e->ds, st);
            k_tape_list<<<nblk(n), kT, 0, st>>>(n, e->nb.n_pad, s.id, e->nb.cnt, e->nb.slot, t.l0cnt,
                                                 t.l0id);
            break;
        case TAPE_EXPLICIT:
            k_tape_state<<<nblk(n), kT, 0, st>>>(n, s.id, s, c.planar, c.z0, arr6(t.st1), t.type1);
            break;
        case TAPE_COLLISION:
            k_tape_state<<<nblk(n), kT, 0, st>>>(n, s.id, s, c.planar, c.z0, arr6(t.st2), nullptr);
            k_tape_pairs<<<64, kT, 0, st>>>(e->pairs, e->cand_base + n, e->pair_cap, t.pairs, t.npairs,
                                            t.pair_cap, e->ds);
            break;
        case TAPE_LIST2:
            k_tape_list<<<nblk(n), kT, 0, st>>>(n, e->nb.n_pad, s.id, e->nb.cnt, e->nb.slot, t.l2cnt,
                                                 t.l2id);
            break;
        case TAPE_SOLVE:
            k_tape_solve<<<nblk(n), kT, 0, st>>>(n, s.id, e->kv.x, s.bc, s.dir, t.praw, t.bc, t.dir);
            break;
    }
}

}  // namespace mpsg

namespace {

int tfail(int code, const std::string& m) {
    set_last_error(m);
    return code;
}

#define TCU(call)                                                                                \
    do {                                                                                         \
        cudaError_t err_ = (call);                                                               \
        if (err_ != cudaSuccess)                                                                 \
            return tfail(MPS_ERR_CUDA, std::string(#call " failed: ") + cudaGetErrorString(err_)); \
    } while (0)

Arr3 a3(double* const* p) { return Arr3{{p[0], p[1], p[2]}}; }

// engine state <- (x, v, type) arrays in id order
void restore(mps_trajectory* t, double* const* src, const int8_t* type_src) {
    mps_engine* e = t->e;
    k_restore_state<<<nblk(t->n), kT, 0, e->st>>>(t->n, e->S().id, e->S(), e->c.planar, arr6(src),
                                                  type_src);
}

void snapshot(mps_trajectory* t, double* const* dst, int8_t* type_dst) {
    mps_engine* e = t->e;
    k_tape_state<<<nblk(t->n), kT, 0, e->st>>>(t->n, e->S().id, e->S(), e->c.planar, e->c.z0,
                                               arr6(dst), type_dst);
}

int set_gravity(mps_trajectory* t, const double* g) {
    mps_engine* e = t->e;
    if (e->c.planar && g[2] != 0.0)
        return tfail(MPS_ERR_ARG, "a planar engine needs gravity z = 0");
    bool same = true;
    for (int d = 0; d < 3; d++) same = same && e->c.g[d] == g[d];
    if (!same) {
        engine_drop_graphs(e);
        for (int d = 0; d < 3; d++) {
            e->c.g[d] = g[d];
            e->P.gravity[d] = g[d];
        }
    }
    return MPS_OK;
}

int record_sensors(mps_trajectory* t, int step) {
    if (t->nsens == 0) return MPS_OK;
    mps_engine* e = t->e;
    k_to_id<<<nblk(t->n), kT, 0, e->st>>>(t->n, e->S().id, e->S().p, t->idp);
    k_pick<<<nblk(t->nsens), kT, 0, e->st>>>(t->nsens, t->sensor, t->idp,
                                             t->sens_out + (size_t)step * t->nsens);
    return MPS_OK;
}

// One reverse step on tape record T (the step's forward has just been taped).
int reverse_step(mps_trajectory* t, const TapeStep& T, int step) {
    mps_engine* e = t->e;
    const Consts& c = e->c;
    const int n = t->n, G = nblk(n);
    cudaStream_t st = e->st;
    Arr3 xb = a3(t->xb), vb = a3(t->vb), ab = a3(t->ab), vt = a3(t->vt), xx = a3(t->xextra);
    // move and pressure gradient
    k_adj_move<<<G, kT, 0, st>>>(n, c.dt, c.planar, T.type1, xb, vb, ab);
    k_adj_pplus<<<G, kT, 0, st>>>(n, T.praw, t->pplus);
    k_adj_minp<<<G, kT, 0, st>>>(n, c, T, t->pplus, t->phat, t->amin);
    k_adj_grad_local<<<G, kT, 0, st>>>(n, c, T, ab, t->phatbar);
    k_adj_grad_gather<<<G, kT, 0, st>>>(n, c, T, t->pplus, t->phat, ab, t->phatbar, t->amin, xb,
                                        t->pbar);
    if (t->nsens)
        k_adj_sensor<<<nblk(t->nsens), kT, 0, st>>>(t->nsens, t->sensor,
                                                    t->sens_bar + (size_t)step * t->nsens, t->pbar);
    // transpose Poisson solve (A is symmetric): A lambda = masked p_bar
    k_adj_assemble<<<G, kT, 0, st>>>(n, c, T, t->pbar, e->A);
    TCU(cudaMemsetAsync(e->ds, 0, sizeof(DevStats), st));
    launch_solve_fp64(c, e->A, e->kv, 1e-14, 4 * (int64_t)n + 100, e->ds, st);
    k_adj_ppe_gather<<<G, kT, 0, st>>>(n, c, T, e->kv.x, xb);
    // collision pass
    k_copy6<<<G, kT, 0, st>>>(n, arr6(T.st1), arr6(t->cur));
    k_zero3<<<G, kT, 0, st>>>(n, xx);
    k_adj_collision<<<1, 1, 0, st>>>(n, c, T, arr6(t->cur), t->rec, xb, vb, xx);
    k_add3<<<G, kT, 0, st>>>(n, xx, xb);
    // explicit part
    k_adj_explicit_local<<<G, kT, 0, st>>>(n, c.dt, c.planar, T.type0, xb, vb, vt, ab);
    k_adj_gsum<<<1, 1024, 0, st>>>(n, ab, t->gbar);
    k_adj_explicit_gather<<<G, kT, 0, st>>>(n, c, T, ab, vt, xb, vb);
    TCU(cudaMemcpyAsync(e->hs, e->ds, sizeof(DevStats), cudaMemcpyDeviceToHost, st));
    TCU(cudaStreamSynchronize(st));
    TCU(cudaGetLastError());
    if (e->hs->status & ST_TIMEOUT) return tfail(MPS_ERR_TIMEOUT, "adjoint PPE solve: a bounded wait gave up");
    return MPS_OK;
}

}  // namespace

extern "C" {

int mps_trajectory_create(mps_engine* e, int32_t n_steps, int32_t checkpoint_every,
                          const int32_t* sensor_ids, int32_t n_sensors, mps_trajectory** out) {
    if (!e || !out || n_steps <= 0 || checkpoint_every <= 0 || n_sensors < 0 ||
        (n_sensors > 0 && !sensor_ids))
        return tfail(MPS_ERR_ARG, "mps_trajectory_create: bad arguments");
    *out = nullptr;
    if (e->c.ho_on)
        return tfail(MPS_ERR_ARG, "trajectories do not support the higher-order source term");
    for (int k = 0; k < n_sensors; k++)
        if (sensor_ids[k] < 0 || sensor_ids[k] >= e->n)
            return tfail(MPS_ERR_ARG, "mps_trajectory_create: sensor id out of range");
    auto* t = new mps_trajectory();
    t->e = e;
    t->n = e->n;
    t->steps = n_steps;
    t->every = std::min(checkpoint_every, n_steps);
    t->nseg = (n_steps + t->every - 1) / t->every;
    t->nsens = n_sensors;
    const size_t n = t->n, K = e->c.K;
    auto bail = [&](const char* what) {
        mps_trajectory_destroy(t);
        return tfail(MPS_ERR_CUDA, std::string("mps_trajectory_create: cudaMalloc failed (") + what + ")");
    };
    for (int d = 0; d < 6; d++)
        if (t->alloc(&t->ic[d], n) || t->alloc(&t->fin[d], n) || t->alloc(&t->cur[d], n)) return bail("state");
    if (t->alloc(&t->ic_type, n) || t->alloc(&t->fin_type, n)) return bail("types");
    t->ck.resize((size_t)6 * t->nseg);
    t->ckt.resize(t->nseg);
    for (int s = 0; s < t->nseg; s++) {
        for (int d = 0; d < 6; d++)
            if (t->alloc(&t->ck[6 * s + d], n)) return bail("checkpoints");
        if (t->alloc(&t->ckt[s], n)) return bail("checkpoints");
    }
    if (t->alloc(&t->sensor, std::max(n_sensors, 1)) ||
        t->alloc(&t->sens_out, (size_t)n_steps * std::max(n_sensors, 1)) ||
        t->alloc(&t->sens_bar, (size_t)n_steps * std::max(n_sensors, 1)) || t->alloc(&t->idp, n))
        return bail("sensors");
    t->tape.resize(t->every);
    const int32_t pcap = (int32_t)n + 1024;
    for (auto& T : t->tape) {
        for (int d = 0; d < 6; d++)
            if (t->alloc(&T.st0[d], n) || t->alloc(&T.st1[d], n) || t->alloc(&T.st2[d], n)) return bail("tape");
        if (t->alloc(&T.praw, n) || t->alloc(&T.type0, n) || t->alloc(&T.type1, n) ||
            t->alloc(&T.bc, n) || t->alloc(&T.dir, n) || t->alloc(&T.l0cnt, n) ||
            t->alloc(&T.l0id, n * K) || t->alloc(&T.l2cnt, n) || t->alloc(&T.l2id, n * K) ||
            t->alloc(&T.pairs, pcap) || t->alloc(&T.npairs, 1))
            return bail("tape");
        T.pair_cap = pcap;
    }
    for (int d = 0; d < 3; d++)
        if (t->alloc(&t->xb[d], n) || t->alloc(&t->vb[d], n) || t->alloc(&t->ab[d], n) ||
            t->alloc(&t->vt[d], n) || t->alloc(&t->xextra[d], n))
            return bail("adjoint");
    if (t->alloc(&t->pplus, n) || t->alloc(&t->phat, n) || t->alloc(&t->phatbar, n) ||
        t->alloc(&t->pbar, n) || t->alloc(&t->amin, n) || t->alloc(&t->rec, (size_t)pcap * 13) ||
        t->alloc(&t->gbar, 4))
        return bail("adjoint");
    if (cudaMallocHost(&t->hstage, sizeof(double) * 3 * n) != cudaSuccess) {
        t->hstage = nullptr;
        return bail("pinned stage");
    }
    if (n_sensors)
        TCU(cudaMemcpy(t->sensor, sensor_ids, sizeof(int32_t) * n_sensors, cudaMemcpyHostToDevice));
    // the engine's current state is the initial condition
    snapshot(t, t->ic, t->ic_type);
    TCU(cudaStreamSynchronize(e->st));
    TCU(cudaGetLastError());
    for (int d = 0; d < 3; d++) t->g_fwd[d] = e->c.g[d];
    *out = t;
    return MPS_OK;
}

int mps_trajectory_destroy(mps_trajectory* t) {
    if (!t) return MPS_OK;
    if (t->e && t->e->st) cudaStreamSynchronize(t->e->st);
    for (void* p : t->allocs) cudaFree(p);
    if (t->hstage) cudaFreeHost(t->hstage);
    delete t;
    return MPS_OK;
}

int mps_trajectory_forward(mps_trajectory* t, const double* vel0, const double* gravity,
                           double* sensor_pressure, double* pos_final, double* vel_final) {
    if (!t) return tfail(MPS_ERR_ARG, "null trajectory");
    mps_engine* e = t->e;
    const int n = t->n;
    cudaStream_t st = e->st;
    if (gravity) {
        int rc = set_gravity(t, gravity);
        if (rc) return rc;
    }
    for (int d = 0; d < 3; d++) t->g_fwd[d] = e->c.g[d];
    if (vel0) {
        if (e->c.planar)
            for (int i = 0; i < n; i++)
                if (vel0[3 * i + 2] != 0.0) return tfail(MPS_ERR_ARG, "a planar engine keeps v_z = 0");
        std::memcpy(t->hstage, vel0, sizeof(double) * 3 * n);
        TCU(cudaMemcpyAsync(e->stage, t->hstage, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
        k_deinterleave3<<<nblk(n), kT, 0, st>>>(n, e->stage, Arr3{{t->ic[3], t->ic[4], t->ic[5]}});
    }
    restore(t, t->ic, t->ic_type);
    for (int s = 0; s < t->steps; s++) {
        if (s % t->every == 0) snapshot(t, &t->ck[6 * (s / t->every)], t->ckt[s / t->every]);
        mps_step_stats stt;
        int rc = engine_step(e, false, &stt);
        if (rc) return rc;
        record_sensors(t, s);
    }
    snapshot(t, t->fin, t->fin_type);
    if (sensor_pressure && t->nsens)
        TCU(cudaMemcpyAsync(sensor_pressure, t->sens_out, sizeof(double) * t->steps * t->nsens,
                            cudaMemcpyDeviceToHost, st));
    for (int w = 0; w < 2; w++) {
        double* host = w == 0 ? pos_final : vel_final;
        if (!host) continue;
        k_interleave3<<<nblk(n), kT, 0, st>>>(n, Arr3{{t->fin[3 * w], t->fin[3 * w + 1], t->fin[3 * w + 2]}},
                                              e->stage);
        TCU(cudaMemcpyAsync(t->hstage, e->stage, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
        TCU(cudaStreamSynchronize(st));
        std::memcpy(host, t->hstage, sizeof(double) * 3 * n);
    }
    TCU(cudaStreamSynchronize(st));
    TCU(cudaGetLastError());
    t->forward_done = true;
    return MPS_OK;
}

int mps_trajectory_backward(mps_trajectory* t, const double* d_sensor_pressure,
                            const double* d_pos_final, const double* d_vel_final, double* d_pos0,
                            double* d_vel0, double* d_gravity) {
    if (!t) return tfail(MPS_ERR_ARG, "null trajectory");
    if (!t->forward_done) return tfail(MPS_ERR_ARG, "mps_trajectory_backward: run the forward first");
    mps_engine* e = t->e;
    const int n = t->n;
    cudaStream_t st = e->st;
    // the forward's gravity (a later change of the engine's would alter the recompute)
    int rc = set_gravity(t, t->g_fwd);
    if (rc) return rc;
    const int32_t saved_log = e->debug_log_count;
    // seeds
    for (int w = 0; w < 2; w++) {
        const double* host = w == 0 ? d_pos_final : d_vel_final;
        double** dst = w == 0 ? t->xb : t->vb;
        if (host) {
            std::memcpy(t->hstage, host, sizeof(double) * 3 * n);
            TCU(cudaMemcpyAsync(e->stage, t->hstage, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
            k_deinterleave3<<<nblk(n), kT, 0, st>>>(n, e->stage, Arr3{{dst[0], dst[1], dst[2]}});
            TCU(cudaStreamSynchronize(st));
        } else {
            k_zero3<<<nblk(n), kT, 0, st>>>(n, Arr3{{dst[0], dst[1], dst[2]}});
        }
    }
    if (t->nsens) {
        if (d_sensor_pressure)
            TCU(cudaMemcpyAsync(t->sens_bar, d_sensor_pressure, sizeof(double) * t->steps * t->nsens,
                                cudaMemcpyHostToDevice, st));
        else
            TCU(cudaMemsetAsync(t->sens_bar, 0, sizeof(double) * t->steps * t->nsens, st));
    }
    TCU(cudaMemsetAsync(t->gbar, 0, sizeof(double) * 4, st));
    for (int seg = t->nseg - 1; seg >= 0; seg--) {
        const int s0 = seg * t->every, s1 = std::min(t->steps, s0 + t->every);
        restore(t, &t->ck[6 * seg], t->ckt[seg]);
        for (int s = s0; s < s1; s++) {  // re-run the segment with the tape attached
            e->tape = &t->tape[s - s0];
            mps_step_stats stt;
            rc = engine_step(e, false, &stt);
            e->tape = nullptr;
            if (rc) return rc;
        }
        for (int s = s1 - 1; s >= s0; s--) {
            rc = reverse_step(t, t->tape[s - s0], s);
            if (rc) return rc;
        }
    }
    // leave the engine at the forward's final state
    restore(t, t->fin, t->fin_type);
    e->debug_log_count = saved_log;
    for (int w = 0; w < 2; w++) {
        double* host = w == 0 ? d_pos0 : d_vel0;
        if (!host) continue;
        k_interleave3<<<nblk(n), kT, 0, st>>>(n, a3(w == 0 ? t->xb : t->vb), e->stage);
        TCU(cudaMemcpyAsync(t->hstage, e->stage, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
        TCU(cudaStreamSynchronize(st));
        std::memcpy(host, t->hstage, sizeof(double) * 3 * n);
    }
    double g[4];
    TCU(cudaMemcpyAsync(g, t->gbar, sizeof(double) * 4, cudaMemcpyDeviceToHost, st));
    TCU(cudaStreamSynchronize(st));
    TCU(cudaGetLastError());
    if (d_gravity)
        for (int d = 0; d < 3; d++) d_gravity[d] = (e->c.planar && d == 2) ? 0.0 : g[d];
    return MPS_OK;
}

}  // extern "C"
