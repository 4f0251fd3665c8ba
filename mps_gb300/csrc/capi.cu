// C ABI of the engine (include/mps_gb300.h): device memory, the per-step
// kernel sequence of MPS::stepForward (src/mps.cpp:111-130), and the
// host<->device views in particle-id order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "engine_impl.cuh"

using namespace mpsg;

namespace mpsg {

// RefValues::RefValues, src/mps.cpp:132-163 (host, same operation order).
void ref_values(int dim, double l0, double re, double* n0o, double* lamo) {
    double n0 = 0.0, lam = 0.0;
    int zb = dim == 2 ? 0 : -4, ze = dim == 2 ? 1 : 5;
    for (int ix = -4; ix < 5; ix++)
        for (int iy = -4; iy < 5; iy++)
            for (int iz = zb; iz < ze; iz++) {
                if (ix == 0 && iy == 0 && iz == 0) continue;
                double x = l0 * (double)ix, y = l0 * (double)iy, z = l0 * (double)iz;
                double dist = std::sqrt((x * x + y * y) + z * z);
                double w = dist < re ? (re / dist) - 1.0 : 0.0;
                n0 += w;
                lam += (dist * dist) * w;
            }
    lam /= n0;
    *n0o = n0;
    if (lamo) *lamo = lam;
}

// Smallest t with sqrt_rn(t) >= re, so that sqrt_rn(d2) < re <=> d2 < t.
double sq_threshold(double re) {
    if (!(re > 0.0)) return 0.0;
    double t = re * re;
    while (t > 0.0 && std::sqrt(t) >= re) t = std::nextafter(t, 0.0);
    while (std::sqrt(t) < re) t = std::nextafter(t, std::numeric_limits<double>::infinity());
    return t;
}

// Bucket::Bucket's grid (src/bucket.cpp:10-22): int(extent / len) + 3 cells
// per axis.  The reference trusts its settings; here the domain must be
// finite with max >= min on every axis and each axis at most 2^30 cells, so
// that every axis has at least the 3 cells the clamped cell coordinate
// [1, cells - 2] and the 3x3(x3) sweep need.
bool bucket_grid(const mps_params& P, double len, int32_t dims[3], std::string* why) {
    static const char* ax = "xyz";
    if (!(len > 0.0) || !std::isfinite(len)) {
        if (why) *why = "bucket length (the largest effective radius) must be finite and positive";
        return false;
    }
    for (int d = 0; d < 3; d++) {
        const double lo = P.domain_min[d], hi = P.domain_max[d];
        if (!std::isfinite(lo) || !std::isfinite(hi) || !(hi >= lo)) {
            if (why)
                *why = std::string("domain ") + ax[d] + " range must be finite with max >= min";
            return false;
        }
        const double q = (hi - lo) / len;
        if (!(q < 1073741824.0)) {
            if (why) *why = std::string("domain ") + ax[d] + " extent is too many bucket cells";
            return false;
        }
        dims[d] = (int32_t)q + 3;
    }
    return true;
}

}  // namespace mpsg

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

#define CU(call)                                                                          \
    do {                                                                                  \
        cudaError_t err_ = (call);                                                        \
        if (err_ != cudaSuccess)                                                          \
            return fail(MPS_ERR_CUDA, std::string(#call " failed: ") + cudaGetErrorString(err_)); \
    } while (0)

int lattice_count(int dim, double ratio) {
    int r = (int)std::ceil(ratio) + 1, cnt = 0;
    for (int ix = -r; ix <= r; ix++)
        for (int iy = -r; iy <= r; iy++)
            for (int iz = (dim == 2 ? 0 : -r); iz <= (dim == 2 ? 0 : r); iz++) {
                double d = std::sqrt((double)(ix * ix + iy * iy + iz * iz));
                if ((ix || iy || iz) && d < ratio) cnt++;
            }
    return cnt;
}

__global__ void k_type_from_host_order(int n, const int32_t* __restrict__ id,
                                       const int32_t* __restrict__ src, int8_t* __restrict__ dst) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) dst[k] = (int8_t)src[id[k]];
}
__global__ void k_to_host_order(int n, const int32_t* __restrict__ id, const double* __restrict__ src,
                                int comps, int comp, double* __restrict__ dst) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) dst[(size_t)id[k] * comps + comp] = src[k];
}
__global__ void k_i8_to_host_order(int n, const int32_t* __restrict__ id, const int8_t* __restrict__ src,
                                   int32_t* __restrict__ dst) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) dst[id[k]] = src[k];
}
// xyz-interleaved host layout <-> the slot-ordered component arrays (one
// launch per vector; planar engines keep no z array: z is the constant zc)
__global__ void k_vec3_to_host(int n, const int32_t* __restrict__ id, const double* __restrict__ d0,
                               const double* __restrict__ d1, const double* __restrict__ d2,
                               double zc, double* __restrict__ dst) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const size_t o = (size_t)id[k] * 3;
    dst[o] = d0[k];
    dst[o + 1] = d1[k];
    dst[o + 2] = d2 ? d2[k] : zc;
}
__global__ void k_vec3_from_host(int n, const int32_t* __restrict__ id, const double* __restrict__ src,
                                 double* __restrict__ d0, double* __restrict__ d1, double* __restrict__ d2) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const size_t o = (size_t)id[k] * 3;
    d0[k] = src[o];
    d1[k] = src[o + 1];
    if (d2) d2[k] = src[o + 2];
}
// Upload checks before anything is written: planar engines keep z = z0 and
// v_z = 0 (bit 1), types lie in {-1, 0, 1, 2} (bit 2).
__global__ void k_check_upload(int n, const double* __restrict__ pos, const double* __restrict__ vel,
                               const int32_t* __restrict__ type, int planar, double z0,
                               int32_t* __restrict__ flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int32_t f = 0;
    if (planar && ((pos && pos[3 * (size_t)i + 2] != z0) || (vel && vel[3 * (size_t)i + 2] != 0.0))) f |= 1;
    if (type && (type[i] < -1 || type[i] > 2)) f |= 2;
    if (f) atomicOr(flag, f);
}
// The step's record for mps_run_report: its DevStats and the device time.
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__global__ void k_stats_record(const DevStats* __restrict__ ds, DevStats* ring, int32_t* pos, int32_t cap) {
    const int k = *pos;
    if (k < cap) {
        DevStats r = *ds;
        r.t_end = global_ns();
        ring[k] = r;
    }
    *pos = k + 1;
}
__global__ void k_stamp(unsigned long long* t) { *t = global_ns(); }
__global__ void k_iota(int n, int32_t* a) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) a[k] = k;
}

}  // namespace

namespace {

int alloc_state(mps_engine* e, StateBuf& s) {
    size_t n = e->n_pad;
    CU(e->alloc(&s.x, n));
    CU(e->alloc(&s.y, n));
    CU(e->alloc(&s.z, n));
    CU(e->alloc(&s.xyf, n));
    CU(e->alloc(&s.zf, n));
    CU(e->alloc(&s.xylo, n));
    CU(e->alloc(&s.vf, n));
    CU(e->alloc(&s.pf, n));
    CU(e->alloc(&s.vx, n));
    CU(e->alloc(&s.vy, n));
    CU(e->alloc(&s.vz, n));
    CU(e->alloc(&s.p, n));
    CU(e->alloc(&s.minp, n));
    CU(e->alloc(&s.ndr, n));
    CU(e->alloc(&s.nd_last, n));
    CU(e->alloc(&s.id, n));
    CU(e->alloc(&s.type, n));
    CU(e->alloc(&s.bc, n));
    CU(e->alloc(&s.dir, n));
    return MPS_OK;
}

Mg active_mg(const mps_engine* e) {
    Mg g = e->mg;
    g.enabled = e->mg.enabled && e->mg_requested != 0;
    g.additive = e->mg_requested == 1 || e->mg_requested == 3 || e->mg_requested == 4;
    g.smooth = e->mg_requested == 3;
    g.overlap = e->mg_requested == 1 && e->cycle_overlap;
    return g;
}

// The public code of a step's device status bits (check_status's order).
int32_t status_code(int32_t s) {
    if (s & ST_TIMEOUT) return MPS_ERR_TIMEOUT;
    if (s & ST_NONFINITE) return MPS_ERR_NONFINITE;
    if (s & ST_CAPACITY) return MPS_ERR_CAPACITY;
    if (s & ST_ASYMMETRIC) return MPS_ERR_ASYMMETRIC;
    if (s & ST_NOT_CONVERGED) return MPS_ERR_NOT_CONVERGED;
    return MPS_OK;
}

int check_status(mps_engine* e) {
    int32_t s = e->hs->status;
    if (s & ST_TIMEOUT) return fail(MPS_ERR_TIMEOUT, "a bounded device-side wait gave up");
    if (s & ST_NONFINITE)
        return fail(MPS_ERR_NONFINITE, "a pressure or particle position became non-finite");
    if (s & ST_CAPACITY)
        return fail(MPS_ERR_CAPACITY, "neighbour or collision list capacity exceeded (max neighbours " +
                                          std::to_string(e->hs->max_neighbors) + ", capacity " +
                                          std::to_string(e->c.K) + ")");
    if (s & ST_ASYMMETRIC) return fail(MPS_ERR_ASYMMETRIC, symmetry_message(e));
    if (s & ST_NOT_CONVERGED)
        return fail(MPS_ERR_NOT_CONVERGED,
                    "the pressure solve stopped at its iteration cap with relative residual " +
                        std::to_string(e->hs->cg_rel_residual) + " (the step completed with that pressure)");
    return MPS_OK;
}

// The step in three parts (the batch interleaves many engines' parts around
// one shared solve launch).  Launches only; the caller synchronises.  With a
// tape attached, every phase boundary is also recorded for the adjoint
// (plus a neighbour list at the step-start positions).
//
// Part 1: setNeighbors + calcGravity + calcViscosity + moveParticles,
// setNeighbors + collision, setNeighbors + setBoundaryCondition +
// setSourceTerm + setMatrix + ensureDirichletBoundaryConnection.
void enqueue_pre_solve(mps_engine* e) {
    Consts& c = e->c;
    cudaStream_t st = e->st;
    const int mixed = e->precision == MPS_PRECISION_MIXED;
    const bool taping = e->tape != nullptr;
    if (taping) tape_phase(e, TAPE_START);
    launch_rebuild(c, e->S(), e->buf[e->cur ^ 1], e->sc, e->ds, st);
    e->swap();
    if (taping) tape_phase(e, TAPE_LIST0);
    launch_explicit(c, e->S(), e->buf[e->cur ^ 1], e->sc, mixed, e->ds, st);
    e->swap();
    if (taping) tape_phase(e, TAPE_EXPLICIT);
    launch_rebuild(c, e->S(), e->buf[e->cur ^ 1], e->sc, e->ds, st);
    e->swap();
    launch_collision(c, e->S(), e->sc, e->cand_cnt, e->cand_base, e->cw, e->pairs, e->pair_cap,
                     e->sc.scan_tmp, e->ds, st);
    if (taping) tape_phase(e, TAPE_COLLISION);
    launch_rebuild(c, e->S(), e->buf[e->cur ^ 1], e->sc, e->ds, st);
    e->swap();
    launch_build_list_bc_source(c, e->S(), e->sc, e->nb, e->A, e->ds, st);
    if (taping) tape_phase(e, TAPE_LIST2);
    launch_assemble(c, e->S(), e->nb, e->A, e->ds, st);
    launch_dirichlet(c, e->S(), e->nb, e->A, e->parent, e->has_surface, e->ds, st);
    // solvePoissonEquation's symmetry test (src/mps.cpp:418-442); the mixed
    // solver's setup reads the matrix anyway and forms the fingerprint there
    if (!mixed) launch_symmetry_check(c, e->S(), e->A, e->ds, st);
}

// Mixed solver only: FP32 operator and multigrid hierarchy of this step.
void enqueue_solver_setup(mps_engine* e) {
    if (e->precision != MPS_PRECISION_MIXED) return;
    launch_mixed_setup(e->c, e->sc, e->A, e->mf, e->kv, e->S().id, e->warm_start != 0, e->ds, e->st);
    launch_symmetry_locate(e->c, e->S(), e->A, e->ds, e->st);
    launch_mg_setup(e->c, e->A, e->mf, active_mg(e), e->st);
}

// Part 3: removeNegativePressure, setMinimumPressure, calcPressureGradient,
// moveParticlesWithPressureGradient, getCourantNumber (+ setNumberDensity).
void enqueue_post_solve(mps_engine* e, bool do_export) {
    Consts& c = e->c;
    cudaStream_t st = e->st;
    const int mixed = e->precision == MPS_PRECISION_MIXED;
    launch_pressure_post(c, e->S(), e->nb, e->kv.x, e->kv.x_prev, e->ax, e->ay, e->az, mixed, e->ds,
                         st);
    if (do_export || c.ho_on) {
        launch_rebuild(c, e->S(), e->buf[e->cur ^ 1], e->sc, e->ds, st);
        e->swap();
        launch_build_list(c, e->S(), e->sc, e->nb, e->ds, st);
        launch_number_density(c, e->S(), e->nb, st);
    }
}

// One MPS::stepForward (src/mps.cpp:111-130).
void enqueue_step(mps_engine* e, bool do_export) {
    g_launches = 0;
    cudaStream_t st = e->st;
    enqueue_pre_solve(e);
    // inside a stream capture the solve's timing events are external event
    // nodes; outside one, plain records
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(st, &cap);
    const unsigned evflag = cap == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : 0u;
    cudaEventRecordWithFlags(e->ev[2], st, evflag);
    enqueue_solver_setup(e);
    const int64_t mi = e->max_iter > 0 ? e->max_iter : 2 * (int64_t)e->c.n;
    if (e->precision == MPS_PRECISION_MIXED)
        launch_solve_mixed(e->c, e->A, e->mf, active_mg(e), e->kv, e->tol, mi, e->warm_start != 0,
                           e->ds, st);
    else
        launch_solve_fp64(e->c, e->A, e->kv, e->tol, mi, e->ds, st);
    cudaEventRecordWithFlags(e->ev[3], st, evflag);
    if (e->tape) tape_phase(e, TAPE_SOLVE);
    enqueue_post_solve(e, do_export);
    k_stats_record<<<1, 1, 0, st>>>(e->ds, e->ring, e->ring_pos, e->ring_cap);
    ++g_launches;
    e->step_launches = g_launches;
}

// Algorithmic bytes of one pressure solve: each array a solver pass streams,
// counted once at its stored width (gathered vector entries count once, as
// the row's own entry).  Per stored off-diagonal entry and pass: FP64 12 B
// (column + value), compact FP32 5 B (value + index byte).  Per row and
// iteration: FP64 CG 116 B (8 vectors); MIXED inner iteration 69 B with the
// Jacobi preconditioner; with the multigrid V-cycle, per cell of level 1
// 72 B (segment bounds, the up pass's 9-point stencil and 8 vector words)
// and of levels >= 2 132 B (the same plus the 4x4 restriction weights), and,
// additive at level 0, 85 B per row (165 B with the smoothed transfer: the
// 9 row-to-cell sums read twice and the neighbourhood's residuals; 145 B in
// the overlapped arrangement of mode 1: the operator pass on y = D^-1 r
// 29 B, the pass that forms u, w and the dot products 64 B with 8
// row-to-cell sums and the row sum, the vector update 48 B, the level-1
// sums 4 B), multiplicative 155 B per row and two more level-0 operator
// passes (every operator pass reads the row's FP32 row sum).  MIXED adds per
// refinement the FP64 residual (12 B/entry + 36 B/row) and once the FP32
// operator setup (17 B/entry + 28 B/row written and read; 36 B/row more for
// the row-to-cell sums of the multigrid modes, from which level 1's stencils
// are summed).
double solve_bytes(const mps_engine* e, const DevStats& h) {
    const double nnz = (double)h.nnz_off, n = (double)e->n, it = (double)h.cg_iterations;
    if (e->precision == MPS_PRECISION_FP64) return it * (12.0 * nnz + 116.0 * n) + 36.0 * n;
    const Mg g = active_mg(e);
    const bool mg = g.enabled != 0;
    const bool additive = mg && g.additive;
    const double ent = e->c.planar ? 5.0 : 8.0;
    const double row_add = g.smooth ? 165.0 : g.overlap ? 145.0 : 85.0;
    double per_it = !mg ? (ent * nnz + 69.0 * n)
                        : additive ? (ent * nnz + row_add * n) : (3.0 * ent * nnz + 155.0 * n);
    if (mg)
        for (int l = 1; l <= e->mg.nlev; l++)
            per_it += (l == 1 ? 72.0 : 132.0) * e->mg.lev[l].nx * e->mg.lev[l].ny;
    const double ref = (double)h.refinements + 1.0;
    const double setup = 17.0 * nnz + 28.0 * n + (mg ? 36.0 * n : 0.0);
    return it * per_it + ref * (12.0 * nnz + 36.0 * n) + setup;
}

void fill_stats(mps_engine* e, mps_step_stats* out) {
    DevStats& h = *e->hs;
    double cour = 0.0;
    unsigned long long b = h.courant_bits;
    std::memcpy(&cour, &b, sizeof cour);
    e->debug_log_count += h.n_new_ghosts + h.n_unconnected;
    if (cour > e->P.cfl) e->debug_log_count++;  // src/mps.cpp:559-565
    if (!out) return;
    out->courant = cour;
    out->cg_relative_residual = h.cg_rel_residual;
    out->cg_iterations = h.cg_iterations;
    out->refinements = h.refinements;
    out->debug_log_count = e->debug_log_count;
    out->n_collision_candidates = h.n_cand;
    out->n_new_ghosts = h.n_new_ghosts;
    out->n_unconnected = h.n_unconnected;
    out->n_inner = h.n_inner;
    out->n_surface = h.n_surface;
    out->status = status_code(h.status);
    float ms = 0.f, ms2 = 0.f;
    // events a step did not record (batched steps) read as 0 ms
    if (cudaEventElapsedTime(&ms, e->ev[0], e->ev[1]) != cudaSuccess) ms = 0.f;
    if (cudaEventElapsedTime(&ms2, e->ev[2], e->ev[3]) != cudaSuccess) ms2 = 0.f;
    cudaGetLastError();
    out->ms_step = ms;
    out->ms_solve = ms2;
    out->kernel_launches = e->step_launches;
    out->nnz_offdiag = (int64_t)h.nnz_off;
    out->max_neighbors = h.max_neighbors;
    out->graph_replayed = e->last_step_graphed;
    out->solve_bytes = solve_bytes(e, h);
}

void drop_graphs(mps_engine* e) {
    for (int p = 0; p < 2; p++)
        if (e->gexec[p]) {
            cudaGraphExecDestroy(e->gexec[p]);
            e->gexec[p] = nullptr;
        }
}

// Captures one non-export step (stats reset, kernels, stats read-back) as a
// graph for the current buffer parity.  Returns false if the capture was
// refused; the step then runs eagerly and the engine stops trying.
bool capture_step(mps_engine* e) {
    const int par = e->cur;
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(e->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaMemsetAsync(e->ds, 0, sizeof(DevStats), e->st);
    enqueue_step(e, false);
    cudaMemcpyAsync(e->hs, e->ds, sizeof(DevStats), cudaMemcpyDeviceToHost, e->st);
    cudaError_t ce = cudaStreamEndCapture(e->st, &g);
    const int end_parity = e->cur;
    e->cur = par;  // nothing ran yet: the launch below performs the swaps
    cudaGraphExec_t x = nullptr;
    if (ce == cudaSuccess && g) ce = cudaGraphInstantiate(&x, g, 0);
    if (g) cudaGraphDestroy(g);
    if (ce != cudaSuccess || !x) {
        cudaGetLastError();
        return false;
    }
    e->gexec[par] = x;
    e->graph_launches[par] = e->step_launches;
    e->graph_end_parity[par] = end_parity;
    return true;
}

// One MPS::stepForward: a graph replay for non-export steps where graphs are
// on, else the kernels launched one by one.  Waits for the step's stats.
// Enqueues one MPS::stepForward (a graph replay for non-export steps where
// graphs are on, else the kernels one by one); the step's stats reach e->hs
// and its record e->ring when the stream gets there.
int launch_one_step(mps_engine* e, bool do_export) {
    const int par = e->cur;
    bool graphed = false;
    if (!do_export && !e->tape && e->use_graph && !e->graph_broken) {
        if (!e->gexec[par] && !capture_step(e)) e->graph_broken = 1;
        graphed = e->gexec[par] != nullptr;
    }
    if (graphed) {
        CU(cudaEventRecord(e->ev[0], e->st));
        CU(cudaGraphLaunch(e->gexec[par], e->st));
        CU(cudaEventRecord(e->ev[1], e->st));
        e->cur = e->graph_end_parity[par];
        e->step_launches = e->graph_launches[par];
    } else {
        CU(cudaMemsetAsync(e->ds, 0, sizeof(DevStats), e->st));
        CU(cudaEventRecord(e->ev[0], e->st));
        enqueue_step(e, do_export);
        CU(cudaEventRecord(e->ev[1], e->st));
        CU(cudaMemcpyAsync(e->hs, e->ds, sizeof(DevStats), cudaMemcpyDeviceToHost, e->st));
    }
    e->last_step_graphed = graphed ? 1 : 0;
    return MPS_OK;
}

// One MPS::stepForward; waits for its stats.
int run_one_step(mps_engine* e, bool do_export, mps_step_stats* stats) {
    int rc = launch_one_step(e, do_export);
    if (rc) return rc;
    CU(cudaStreamSynchronize(e->st));
    CU(cudaGetLastError());
    fill_stats(e, stats);
    return check_status(e);
}

// Default multigrid weights per mode.  Additive (mode 1): the particle-level
// term omega D^-1 r only has to be positive, and the cell-level V(1,1) uses
// the same omega on Galerkin 9-point stencils, whose Jacobi spectrum
// D^-1 A_c stays well below 2, so undamped Jacobi still smooths there;
// omega 1, s 1.4 took the fewest CG iterations on the 1M dam break (69 vs
// 73 at 0.9/1.5).  Multiplicative (mode 2) smooths the particle matrix
// itself, whose D^-1 A can approach 2: there the damped 0.9 stays.
void mg_default_weights(int mode, float* omega, float* scale) {
    if (mode == 2) {
        *omega = 0.9f;
        *scale = 1.5f;
    } else {
        *omega = 1.0f;
        *scale = 1.4f;
    }
}

}  // namespace

extern "C" {

const char* mps_last_error(void) { return g_last_error.c_str(); }

int32_t mps_particle_count(const mps_engine* e) { return e ? e->n : 0; }

void* mps_stream(mps_engine* e) { return e ? (void*)e->st : nullptr; }

int mps_create(const mps_params* prm, int32_t n, const double* pos, const double* vel,
               const int32_t* type, mps_engine** out) {
    if (!prm || !pos || !vel || !type || !out || n <= 0)
        return fail(MPS_ERR_ARG, "mps_create: null pointer or non-positive particle count");
    *out = nullptr;
    const mps_params& P = *prm;
    if (!(P.particle_distance > 0) || !(P.dt > 0) || !(P.density > 0) || (P.dim != 2 && P.dim != 3))
        return fail(MPS_ERR_ARG, "mps_create: invalid dim, particle distance, dt or density");
    if (!(P.re_pressure > 0) || !(P.re_viscosity > 0) || !(P.re_surface > 0))
        return fail(MPS_ERR_ARG, "mps_create: effective radii must be positive");
    for (int32_t i = 0; i < n; i++)
        if (type[i] < -1 || type[i] > 2)
            return fail(MPS_ERR_ARG, "mps_create: particle type outside {-1,0,1,2}");
    int32_t grid[3];
    {
        std::string why;
        const double len = std::max({P.re_pressure, P.re_viscosity, P.re_surface});
        if (!bucket_grid(P, len, grid, &why)) return fail(MPS_ERR_ARG, "mps_create: " + why);
    }
    int dev = 0, ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(MPS_ERR_NO_DEVICE, "no CUDA device");
    cudaGetDevice(&dev);
    cudaDeviceProp prop;
    CU(cudaGetDeviceProperties(&prop, dev));
    if (prop.major != 10 || prop.minor != 3)
        return fail(MPS_ERR_NO_DEVICE, "this build targets sm_103 (GB300); device is sm_" +
                                           std::to_string(prop.major) + std::to_string(prop.minor));
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop) return fail(MPS_ERR_NO_DEVICE, "device lacks cooperative launch");

    mps_engine* e = new mps_engine();
    e->device = dev;
    e->P = P;
    e->n = n;
    e->n_pad = (n + 31) & ~31;
    Consts& c = e->c;
    c.n = n;
    c.dim = P.dim;
    c.qc_on = P.quasi_compressibility_on != 0;
    c.ho_on = P.higher_order_on != 0;
    c.l0 = P.particle_distance;
    c.dt = P.dt;
    for (int d = 0; d < 3; d++) {
        c.dmin[d] = P.domain_min[d];
        c.dmax[d] = P.domain_max[d];
        c.g[d] = P.gravity[d];
    }
    c.rho = P.density;
    c.re_p = P.re_pressure;
    c.re_v = P.re_viscosity;
    c.re_s = P.re_surface;
    c.re_max = std::max({P.re_pressure, P.re_viscosity, P.re_surface});  // src/settings.cpp:138
    c.cd = P.collision_distance;
    c.len = c.re_max;
    // Bucket::Bucket, src/bucket.cpp:10-22
    c.numX = grid[0];
    c.numY = grid[1];
    c.numZ = grid[2];
    bool planar = P.gravity[2] == 0.0;
    for (int32_t i = 0; i < n && planar; i++)
        planar = pos[3 * i + 2] == pos[2] && vel[3 * i + 2] == 0.0;
    c.planar = planar;
    c.z0 = pos[2];
    double nk = planar ? (double)c.numX * c.numY : (double)c.numX * c.numY * c.numZ;
    if (nk > 1.5e9) {
        delete e;
        return fail(MPS_ERR_ARG, "mps_create: bucket grid too large for the domain and radius");
    }
    c.nkeys = (int32_t)nk;
    c.t_p = sq_threshold(c.re_p);
    c.t_v = sq_threshold(c.re_v);
    c.t_s = sq_threshold(c.re_s);
    c.t_max = sq_threshold(c.re_max);
    c.t_cd = sq_threshold(c.cd);
    {
        // FP32 pre-filter bounds: coordinates of magnitude <= M round to FP32
        // within 2^-24 M, so an FP32 distance is within 4 * 2^-23 * M of the
        // exact one (two roundings per coordinate, three coordinates, and the
        // subtraction); FP32 arithmetic adds a relative 1e-6, covered by 1e-5.
        double M = 0.0;
        for (int d = 0; d < 3; d++) M = std::max({M, std::fabs(P.domain_min[d]), std::fabs(P.domain_max[d])});
        M += 10.0 * c.re_max;
        const double delta = 4.0 * std::ldexp(1.0, -23) * M;
        auto fbound = [&](double re) {
            const double r = (re + delta) * (1.0 + 1e-5);
            return std::nextafter((float)(r * r), std::numeric_limits<float>::infinity());
        };
        c.ft_max = fbound(c.re_max);
        c.ft_v = fbound(c.re_v);
        c.ft_cd = fbound(c.cd);
        const double tv = std::min(c.t_max, c.t_v);
        c.fv_in = std::nextafter((float)(tv * (1.0 - std::ldexp(1.0, -16))), 0.0f);
        c.fv_out = std::nextafter((float)(tv * (1.0 + std::ldexp(1.0, -16))), std::numeric_limits<float>::infinity());
    }
    ref_values(P.dim, c.l0, c.re_p, &c.n0_p, &c.lam_p);
    ref_values(P.dim, c.l0, c.re_v, &c.n0_v, &c.lam_v);
    ref_values(P.dim, c.l0, c.re_s, &c.n0_s, &c.lam_s);
    const double dimd = (double)P.dim;
    c.beta_n0s = P.surface_threshold * c.n0_s;
    c.visc_a = (P.kinematic_viscosity * (2.0 * dimd)) / (c.n0_v * c.lam_v);
    c.mat_c = 2.0 * dimd / (c.lam_p * c.n0_p);
    c.qc_term = P.compressibility / (P.dt * P.dt);
    c.src_g1 = P.relaxation * (1.0 / (P.dt * P.dt));
    c.ho_g1 = P.higher_order_gamma * (1.0 / (P.dt * P.dt));
    c.ho_c = 1.0 / (c.n0_p * P.dt);
    c.grad_scale = dimd / c.n0_p;
    c.e = P.restitution;
    c.fre_v = (float)c.re_v;
    c.fre_p = (float)c.re_p;
    c.fvisc_a = (float)c.visc_a;
    c.fgrad_scale = (float)c.grad_scale;
    int lc = lattice_count(P.dim, c.re_max / c.l0);
    c.K = std::max(32, ((2 * lc + 8 + 31) / 32) * 32);
    e->nb.n_pad = e->n_pad;
    e->mf.rs_stride = e->n_pad;
    e->mf.enabled = c.planar;

    int rc = MPS_OK;
    auto bail = [&](int code) {
        mps_destroy(e);
        return code;
    };
    cudaError_t ce = cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking);
    if (ce != cudaSuccess) return bail(fail(MPS_ERR_CUDA, cudaGetErrorString(ce)));
    for (auto& ev : e->ev)
        if (cudaEventCreate(&ev) != cudaSuccess) return bail(fail(MPS_ERR_CUDA, "event create"));
    if ((rc = alloc_state(e, e->buf[0])) || (rc = alloc_state(e, e->buf[1]))) return bail(rc);
    const size_t np = e->n_pad, K = c.K;
    if (e->alloc(&e->sc.key, np) || e->alloc(&e->sc.rank, np) || e->alloc(&e->sc.perm, np) ||
        e->alloc(&e->sc.skey, np) || e->alloc(&e->sc.cell_count, (size_t)c.nkeys + 2) ||
        e->alloc(&e->sc.cell_start, (size_t)c.nkeys + 2) ||
        e->alloc(&e->sc.scan_tmp, scan_tmp_ints(std::max(c.nkeys + 1, n + 1))) ||
        e->alloc(&e->nb.cnt, np) || e->alloc(&e->nb.slot, np * K) || e->alloc(&e->nb.dist, np * K) ||
        e->alloc(&e->nb.wp, np * K) || e->alloc(&e->A.src, np) || e->alloc(&e->A.diag, np) ||
        e->alloc(&e->A.offcnt, np) || e->alloc(&e->A.col, np * K) || e->alloc(&e->A.val, np * K) ||
        e->alloc(&e->A.slice_w, np / 32 + 1) || e->alloc(&e->A.val32, np * K) ||
        e->alloc(&e->A.diag32, np) || e->alloc(&e->A.rsum, np) || e->alloc(&e->A.rsum32, np) ||
        e->alloc(&e->kv.x, np) || e->alloc(&e->kv.r, np) ||
        e->alloc(&e->kv.x_prev, np) ||
        e->alloc(&e->kv.p, np) || e->alloc(&e->kv.q, np) || e->alloc(&e->kv.z, np) ||
        e->alloc(&e->kv.inv_diag, np) || e->alloc(&e->kv.r32, np) || e->alloc(&e->kv.p32, np) ||
        e->alloc(&e->kv.s32, np) || e->alloc(&e->kv.w32, np) || e->alloc(&e->kv.x32, np) ||
        e->alloc(&e->kv.u32, np) ||
        e->alloc(&e->kv.inv_diag32, np) || e->alloc(&e->kv.barrier, 64) ||
        e->alloc(&e->kv.totals, 8) || e->alloc(&e->mf.idx8, np * K) ||
        e->alloc(&e->mf.sell_row, np) || e->alloc(&e->mf.rs, 3 * np) ||
        e->alloc(&e->cand_cnt, np + 1) || e->alloc(&e->cand_base, np + 2) ||
        e->alloc(&e->cw.jn, np) || e->alloc(&e->cw.jl, np * kCollJList) || e->alloc(&e->cw.ver, np) ||
        e->alloc(&e->cw.ctl, 4) ||
        e->alloc(&e->parent, np + 1) || e->alloc(&e->has_surface, np) || e->alloc(&e->ax, np) ||
        e->alloc(&e->ay, np) || e->alloc(&e->az, np) || e->alloc(&e->stage, 9 * np) ||
        e->alloc(&e->stage_i, 3 * np) || e->alloc(&e->dflag, 1) || e->alloc(&e->ds, 1))
        return bail(fail(MPS_ERR_CUDA, "cudaMalloc failed (out of device memory?)"));
    e->pair_cap = (int32_t)std::min<size_t>(4 * np + 1024, (size_t)1 << 30);
    if (e->alloc(&e->pairs, e->pair_cap)) return bail(fail(MPS_ERR_CUDA, "cudaMalloc pairs"));
    solver_setup(e->kv, e->n_pad, dev);
    if (e->kv.grid <= 0)
        return bail(fail(MPS_ERR_NO_DEVICE, "the persistent solver does not fit co-resident on this device"));
    // multigrid hierarchy (planar scenes): level 1 = the numX x numY cell grid
    if (c.planar) {
        Mg& g = e->mg;
        g.enabled = 1;
        mg_default_weights(1, &g.omega, &g.scale);
        g.additive = 1;
        int nx = c.numX, ny = c.numY, l = 1;
        for (;;) {
            g.lev[l].nx = nx;
            g.lev[l].ny = ny;
            size_t cells = (size_t)nx * ny;
            if (e->alloc(&g.lev[l].st, 9 * cells) || e->alloc(&g.lev[l].invd, cells) ||
                e->alloc(&g.lev[l].r, cells) || e->alloc(&g.lev[l].e, cells) ||
                e->alloc(&g.lev[l].t, cells) || e->alloc(&g.lev[l].act, cells) ||
                (l >= 2 && e->alloc(&g.lev[l].rw, 16 * cells)))
                return bail(fail(MPS_ERR_CUDA, "cudaMalloc multigrid level"));
            if (cells <= (size_t)kMgMaxCoarsest || l == kMgMaxLevels - 1) break;
            nx = (nx + 1) / 2;
            ny = (ny + 1) / 2;
            l++;
        }
        g.nlev = l;
        if ((size_t)g.lev[l].nx * g.lev[l].ny > (size_t)kMgMaxCoarsest) g.enabled = 0;
        g.ngrid = 0;
        while (g.ngrid + 1 < g.nlev && (size_t)g.lev[g.ngrid + 1].nx * g.lev[g.ngrid + 1].ny > kMgBlockCells)
            g.ngrid++;
        if (e->alloc(&g.e0, np) || e->alloc(&g.res0, np) ||
            e->alloc(&g.dense, (size_t)kMgMaxCoarsest * kMgMaxCoarsest) || e->alloc(&g.rowcell, 9 * np) ||
            e->alloc(&g.nact, kMgMaxLevels) || e->alloc(&g.act1_rng, (size_t)c.numX * c.numY) ||
            e->alloc(&g.cell_end, np))
            return bail(fail(MPS_ERR_CUDA, "cudaMalloc multigrid"));
        g.n_pad = (int32_t)np;
    }
    if (e->alloc(&e->kv.partials, (size_t)e->kv.grid * 16))
        return bail(fail(MPS_ERR_CUDA, "cudaMalloc partials"));
    if (cudaMallocHost(&e->hs, sizeof(DevStats)) != cudaSuccess ||
        cudaMallocHost(&e->ring_host, sizeof(DevStats) * (e->ring_cap + 1)) != cudaSuccess)
        return bail(fail(MPS_ERR_CUDA, "cudaMallocHost"));
    if (e->alloc(&e->ring, e->ring_cap) || e->alloc(&e->ring_pos, 1) || e->alloc(&e->ring_t0, 1))
        return bail(fail(MPS_ERR_CUDA, "cudaMalloc step records"));
    cudaMemsetAsync(e->ring_pos, 0, sizeof(int32_t), e->st);
    // zero-init everything that a kernel may read before writing
    StateBuf& s = e->buf[0];
    for (int b = 0; b < 2; b++) {
        StateBuf& t = e->buf[b];
        cudaMemsetAsync(t.p, 0, np * 8, e->st);
        cudaMemsetAsync(t.minp, 0, np * 8, e->st);
        cudaMemsetAsync(t.ndr, 0, np * 8, e->st);
        cudaMemsetAsync(t.nd_last, 0, np * 8, e->st);
        cudaMemsetAsync(t.bc, 0, np, e->st);
        cudaMemsetAsync(t.dir, 0, np, e->st);
        cudaMemsetAsync(t.z, 0, np * 8, e->st);
        cudaMemsetAsync(t.vz, 0, np * 8, e->st);
    }
    cudaMemsetAsync(e->kv.x, 0, np * 8, e->st);
    cudaMemsetAsync(e->kv.x_prev, 0, np * 8, e->st);
    cudaMemsetAsync(e->nb.cnt, 0, np * 4, e->st);
    k_iota<<<(n + 255) / 256, 256, 0, e->st>>>(n, s.id);
    // upload the initial condition (identity slot order, ids = indices)
    CU(cudaMemcpyAsync(e->stage, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, e->st));
    CU(cudaMemcpyAsync(e->stage + 3 * np, vel, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, e->st));
    k_vec3_from_host<<<(n + 255) / 256, 256, 0, e->st>>>(n, s.id, e->stage, s.x, s.y, s.z);
    k_vec3_from_host<<<(n + 255) / 256, 256, 0, e->st>>>(n, s.id, e->stage + 3 * np, s.vx, s.vy, s.vz);
    CU(cudaMemcpyAsync(e->stage_i, type, sizeof(int32_t) * n, cudaMemcpyHostToDevice, e->st));
    k_type_from_host_order<<<(n + 255) / 256, 256, 0, e->st>>>(n, s.id, e->stage_i, s.type);
    e->cur = 0;
    // MPS::loadInitialState's setNumberDensity (src/mps.cpp:106)
    CU(cudaMemsetAsync(e->ds, 0, sizeof(DevStats), e->st));
    launch_rebuild(c, e->S(), e->buf[e->cur ^ 1], e->sc, e->ds, e->st);
    e->swap();
    launch_initial_number_density(c, e->S(), e->sc, e->nb, e->ds, e->st);
    CU(cudaMemcpyAsync(e->hs, e->ds, sizeof(DevStats), cudaMemcpyDeviceToHost, e->st));
    CU(cudaStreamSynchronize(e->st));
    CU(cudaGetLastError());
    if ((rc = check_status(e))) return bail(rc);
    *out = e;
    return MPS_OK;
}

int mps_destroy(mps_engine* e) {
    if (!e) return MPS_OK;
    if (e->st) cudaStreamSynchronize(e->st);
    drop_graphs(e);
    for (void* p : e->allocs) cudaFree(p);
    if (e->hs) cudaFreeHost(e->hs);
    if (e->ring_host) cudaFreeHost(e->ring_host);
    for (auto& ev : e->ev)
        if (ev) cudaEventDestroy(ev);
    if (e->xst) cudaStreamSynchronize(e->xst);
    if (e->xhost) cudaFreeHost(e->xhost);
    if (e->xhost_i) cudaFreeHost(e->xhost_i);
    if (e->xev_ready) cudaEventDestroy(e->xev_ready);
    if (e->xev_done) cudaEventDestroy(e->xev_done);
    if (e->xst) cudaStreamDestroy(e->xst);
    if (e->st) cudaStreamDestroy(e->st);
    delete e;
    return MPS_OK;
}

int mps_set_solver(mps_engine* e, int32_t precision, double tol, int64_t max_iter) {
    if (!e) return fail(MPS_ERR_ARG, "null engine");
    if (precision != MPS_PRECISION_FP64 && precision != MPS_PRECISION_MIXED)
        return fail(MPS_ERR_ARG, "unknown precision");
    drop_graphs(e);
    e->precision = precision;
    e->tol = tol > 0 ? tol
                     : (precision == MPS_PRECISION_FP64 ? std::numeric_limits<double>::epsilon() : 1e-10);
    e->max_iter = max_iter > 0 ? max_iter : 0;
    return MPS_OK;
}

int mps_set_initial_guess(mps_engine* e, int32_t previous) {
    if (!e) return fail(MPS_ERR_ARG, "null engine");
    drop_graphs(e);
    e->warm_start = previous ? 1 : 0;
    return MPS_OK;
}

int mps_set_multigrid(mps_engine* e, int32_t mode, float omega, float scale) {
    if (!e) return fail(MPS_ERR_ARG, "null engine");
    if (mode < 0 || mode > 4) return fail(MPS_ERR_ARG, "multigrid mode must be 0, 1, 2, 3 or 4");
    if (mode && !e->mg.enabled)
        return fail(MPS_ERR_ARG, "multigrid needs a planar scene (2-D, constant z)");
    float dw, ds;
    mg_default_weights(mode, &dw, &ds);
    if (omega == 0.f) omega = dw;
    if (scale == 0.f) scale = ds;
    if (!(omega > 0.f && omega <= 1.f) || !(scale >= 1.f && scale < 2.f))
        return fail(MPS_ERR_ARG, "multigrid weights out of range (0 < omega <= 1, 1 <= scale < 2)");
    drop_graphs(e);
    e->mg_requested = mode;
    e->mg.omega = omega;
    e->mg.scale = scale;
    return MPS_OK;
}

int mps_selftest_wait_limit(int32_t* blocks_gave_up, double* seconds) {
    int gave = 0, status = 0;
    float ms = 0.f;
    constexpr int kBlocks = 8;
    if (selftest_wait_limit(kBlocks, &gave, &status, &ms) != 0)
        return fail(MPS_ERR_CUDA, "mps_selftest_wait_limit: CUDA call failed");
    if (blocks_gave_up) *blocks_gave_up = gave;
    if (seconds) *seconds = ms * 1e-3;
    if (gave != kBlocks || !(status & ST_TIMEOUT))
        return fail(MPS_ERR_TIMEOUT, "mps_selftest_wait_limit: not every block gave up with the timeout status");
    return MPS_OK;
}

int mps_set_collisions(mps_engine* e, int32_t serial) {
    if (!e) return fail(MPS_ERR_ARG, "null engine");
    drop_graphs(e);
    e->cw.serial = serial ? 1 : 0;
    return MPS_OK;
}

int mps_set_graphs(mps_engine* e, int32_t enabled) {
    if (!e) return fail(MPS_ERR_ARG, "null engine");
    e->use_graph = enabled ? 1 : 0;
    if (!enabled) drop_graphs(e);
    return MPS_OK;
}

int mps_run(mps_engine* e, int32_t n_steps, mps_step_stats* stats) {
    if (!e || n_steps < 0) return fail(MPS_ERR_ARG, "mps_run: bad arguments");
    for (int32_t s = 0; s < n_steps; s++) {
        int rc = run_one_step(e, false, stats);
        if (rc) return rc;
    }
    return MPS_OK;
}

int mps_run_report(mps_engine* e, int32_t n_steps, mps_step_stats* stats) {
    if (!e || n_steps < 0 || (n_steps > 0 && !stats)) return fail(MPS_ERR_ARG, "mps_run_report: bad arguments");
    int32_t done = 0;
    int warn = MPS_OK;
    while (done < n_steps) {
        const int32_t m = std::min(e->ring_cap, n_steps - done);
        CU(cudaMemsetAsync(e->ring_pos, 0, sizeof(int32_t), e->st));
        k_stamp<<<1, 1, 0, e->st>>>(e->ring_t0);
        for (int32_t k = 0; k < m; k++) {
            int rc = launch_one_step(e, false);
            if (rc) return rc;
        }
        CU(cudaMemcpyAsync(e->ring_host, e->ring, sizeof(DevStats) * m, cudaMemcpyDeviceToHost, e->st));
        unsigned long long* t0h = &e->ring_host[e->ring_cap].t_end;  // the spare record
        CU(cudaMemcpyAsync(t0h, e->ring_t0, sizeof(unsigned long long), cudaMemcpyDeviceToHost, e->st));
        CU(cudaStreamSynchronize(e->st));
        CU(cudaGetLastError());
        unsigned long long prev = *t0h;
        for (int32_t k = 0; k < m; k++) {
            *e->hs = e->ring_host[k];
            mps_step_stats* o = stats + done + k;
            fill_stats(e, o);
            o->ms_step = (float)((double)(e->ring_host[k].t_end - prev) * 1e-6);
            o->ms_solve = 0.f;  // not timed in these runs
            prev = e->ring_host[k].t_end;
            const int rc = check_status(e);
            if (rc == MPS_ERR_NOT_CONVERGED) {  // a warning: the step completed
                warn = rc;
                continue;
            }
            if (rc) return rc;  // the later steps of this group have been made too
        }
        done += m;
    }
    return warn;
}

int mps_step(mps_engine* e, int32_t is_time_to_export, mps_step_stats* stats) {
    if (!e) return fail(MPS_ERR_ARG, "null engine");
    return run_one_step(e, is_time_to_export != 0, stats);
}

int mps_download(mps_engine* e, double* pos, double* vel, double* pressure, double* min_pressure,
                 double* ndr, int32_t* type, int32_t* bc, int32_t* dirichlet) {
    if (!e) return fail(MPS_ERR_ARG, "null engine");
    const int n = e->n, T = 256, G = (n + 255) / 256;
    const size_t np = e->n_pad;
    StateBuf& s = e->S();
    // every array gathers into its own staging region and is copied out; one
    // wait at the end.  Planar engines keep no z / v_z: they are z0 / 0.
    const bool pl = e->c.planar;
    if (pos) {
        k_vec3_to_host<<<G, T, 0, e->st>>>(n, s.id, s.x, s.y, pl ? nullptr : s.z, e->c.z0, e->stage);
        CU(cudaMemcpyAsync(pos, e->stage, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, e->st));
    }
    if (vel) {
        k_vec3_to_host<<<G, T, 0, e->st>>>(n, s.id, s.vx, s.vy, pl ? nullptr : s.vz, 0.0, e->stage + 3 * np);
        CU(cudaMemcpyAsync(vel, e->stage + 3 * np, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, e->st));
    }
    double* sc[3] = {pressure, min_pressure, ndr};
    double* sd[3] = {s.p, s.minp, s.ndr};
    for (int q = 0; q < 3; q++) {
        if (!sc[q]) continue;
        double* st = e->stage + (6 + q) * np;
        k_to_host_order<<<G, T, 0, e->st>>>(n, s.id, sd[q], 1, 0, st);
        CU(cudaMemcpyAsync(sc[q], st, sizeof(double) * n, cudaMemcpyDeviceToHost, e->st));
    }
    int32_t* ic[3] = {type, bc, dirichlet};
    int8_t* id8[3] = {s.type, s.bc, s.dir};
    for (int q = 0; q < 3; q++) {
        if (!ic[q]) continue;
        int32_t* st = e->stage_i + q * np;
        k_i8_to_host_order<<<G, T, 0, e->st>>>(n, s.id, id8[q], st);
        CU(cudaMemcpyAsync(ic[q], st, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, e->st));
    }
    CU(cudaStreamSynchronize(e->st));
    CU(cudaGetLastError());
    return MPS_OK;
}

int mps_upload(mps_engine* e, const double* pos, const double* vel, const int32_t* type) {
    if (!e) return fail(MPS_ERR_ARG, "null engine");
    const int n = e->n, T = 256, G = (n + 255) / 256;
    const size_t np = e->n_pad;
    StateBuf& s = e->S();
    const bool pl = e->c.planar;
    // copy in and check on the device; the state changes only if all is valid
    double* ps = pos ? e->stage : nullptr;
    double* vs = vel ? e->stage + 3 * np : nullptr;
    int32_t* ts = type ? e->stage_i : nullptr;
    if (pos) CU(cudaMemcpyAsync(ps, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, e->st));
    if (vel) CU(cudaMemcpyAsync(vs, vel, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, e->st));
    if (type) CU(cudaMemcpyAsync(ts, type, sizeof(int32_t) * n, cudaMemcpyHostToDevice, e->st));
    CU(cudaMemsetAsync(e->dflag, 0, sizeof(int32_t), e->st));
    k_check_upload<<<G, T, 0, e->st>>>(n, ps, vs, ts, pl ? 1 : 0, e->c.z0, e->dflag);
    CU(cudaMemcpyAsync(&e->hs->upload_flag, e->dflag, sizeof(int32_t), cudaMemcpyDeviceToHost, e->st));
    CU(cudaStreamSynchronize(e->st));
    CU(cudaGetLastError());
    const int32_t f = e->hs->upload_flag;
    if (f & 1) return fail(MPS_ERR_ARG, "mps_upload: a planar engine keeps z and v_z constant");
    if (f & 2) return fail(MPS_ERR_ARG, "mps_upload: bad particle type");
    if (pos) k_vec3_from_host<<<G, T, 0, e->st>>>(n, s.id, ps, s.x, s.y, pl ? nullptr : s.z);
    if (vel) k_vec3_from_host<<<G, T, 0, e->st>>>(n, s.id, vs, s.vx, s.vy, pl ? nullptr : s.vz);
    if (type) k_type_from_host_order<<<G, T, 0, e->st>>>(n, s.id, ts, s.type);
    CU(cudaStreamSynchronize(e->st));
    CU(cudaGetLastError());
    return MPS_OK;
}

int mps_neighbors(mps_engine* e, int64_t* offsets, int32_t* ids, double* dist, int64_t* total) {
    if (!e) return fail(MPS_ERR_ARG, "null engine");
    const int n = e->n, np = e->n_pad, K = e->c.K;
    std::vector<int32_t> cnt(n), id(n), slot((size_t)np * K);
    std::vector<double> dd((size_t)np * K);
    CU(cudaStreamSynchronize(e->st));
    CU(cudaMemcpy(cnt.data(), e->nb.cnt, 4 * n, cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(id.data(), e->S().id, 4 * n, cudaMemcpyDeviceToHost));
    int64_t tot = 0;
    for (int k = 0; k < n; k++) tot += cnt[k];
    if (total) *total = tot;
    if (!ids) return MPS_OK;
    CU(cudaMemcpy(slot.data(), e->nb.slot, 4 * (size_t)np * K, cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(dd.data(), e->nb.dist, 8 * (size_t)np * K, cudaMemcpyDeviceToHost));
    std::vector<int32_t> slot_of(n);
    for (int k = 0; k < n; k++) slot_of[id[k]] = k;
    int64_t o = 0;
    offsets[0] = 0;
    for (int i = 0; i < n; i++) {
        int k = slot_of[i];
        for (int m = 0; m < cnt[k]; m++) {
            ids[o] = id[slot[(size_t)m * np + k]];
            if (dist) dist[o] = dd[(size_t)m * np + k];
            o++;
        }
        offsets[i + 1] = o;
    }
    return MPS_OK;
}

int mps_system(mps_engine* e, double* source, int64_t* row_ptr, int32_t* col, double* val,
               int64_t* nnz) {
    if (!e) return fail(MPS_ERR_ARG, "null engine");
    const int n = e->n, np = e->n_pad, K = e->c.K;
    std::vector<int32_t> id(n), offcnt(n), scol((size_t)np * K);
    std::vector<int8_t> bc(n);
    std::vector<double> src(n), diag(n), sval((size_t)np * K);
    CU(cudaStreamSynchronize(e->st));
    CU(cudaMemcpy(id.data(), e->S().id, 4 * n, cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(bc.data(), e->S().bc, n, cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(offcnt.data(), e->A.offcnt, 4 * n, cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(src.data(), e->A.src, 8 * n, cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(diag.data(), e->A.diag, 8 * n, cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(scol.data(), e->A.col, 4 * (size_t)np * K, cudaMemcpyDeviceToHost));
    CU(cudaMemcpy(sval.data(), e->A.val, 8 * (size_t)np * K, cudaMemcpyDeviceToHost));
    std::vector<int32_t> slot_of(n);
    for (int k = 0; k < n; k++) slot_of[id[k]] = k;
    int64_t tot = 0;
    for (int k = 0; k < n; k++)
        if (bc[k] == BC_INNER) tot += offcnt[k] + 1;
    if (nnz) *nnz = tot;
    if (source)
        for (int i = 0; i < n; i++) source[i] = src[slot_of[i]];
    if (!row_ptr) return MPS_OK;
    int64_t o = 0;
    row_ptr[0] = 0;
    std::vector<std::pair<int32_t, double>> row;
    for (int i = 0; i < n; i++) {
        int k = slot_of[i];
        if (bc[k] == BC_INNER) {
            row.clear();
            row.push_back({i, diag[k]});
            size_t base = (size_t)(k >> 5) * K * 32 + (k & 31);
            for (int m = 0; m < offcnt[k]; m++)
                row.push_back({id[scol[base + (size_t)m * 32]], sval[base + (size_t)m * 32]});
            std::sort(row.begin(), row.end(), [](auto& a, auto& b) { return a.first < b.first; });
            for (auto& r : row) {
                if (col) col[o] = r.first;
                if (val) val[o] = r.second;
                o++;
            }
        }
        row_ptr[i + 1] = o;
    }
    return MPS_OK;
}

int mps_collisions(mps_engine* e, int32_t* pi, int32_t* pj, double* dist, int32_t* count) {
    if (!e) return fail(MPS_ERR_ARG, "null engine");
    CU(cudaStreamSynchronize(e->st));
    int32_t cnt = std::min(e->hs->n_cand, e->pair_cap);
    if (count) *count = cnt;
    if (!pi || cnt == 0) return MPS_OK;
    std::vector<CollPair> v(cnt);
    CU(cudaMemcpy(v.data(), e->pairs, sizeof(CollPair) * cnt, cudaMemcpyDeviceToHost));
    for (int t = 0; t < cnt; t++) {
        pi[t] = v[t].ii;
        pj[t] = v[t].ij;
        if (dist) dist[t] = v[t].dist;
    }
    return MPS_OK;
}

}  // extern "C"

namespace mpsg {
// Lets the other translation units of the library report through mps_last_error().
void set_last_error(const std::string& m) { g_last_error = m; }
int engine_step(mps_engine* e, bool do_export, mps_step_stats* stats) {
    return run_one_step(e, do_export, stats);
}
void engine_drop_graphs(mps_engine* e) { drop_graphs(e); }
void engine_pre_solve(mps_engine* e) { enqueue_pre_solve(e); }
void engine_solver_setup(mps_engine* e) { enqueue_solver_setup(e); }
void engine_post_solve(mps_engine* e, bool do_export) { enqueue_post_solve(e, do_export); }
Mg engine_active_mg(const mps_engine* e) { return active_mg(e); }
int engine_collect(mps_engine* e, mps_step_stats* stats) {
    fill_stats(e, stats);
    return check_status(e);
}
}  // namespace mpsg
