// Host-side engine object shared by the translation units of the C ABI
// (capi.cu: the step; adjoint.cu: trajectories and their adjoint; batch.cu:
// many scenes per launch).  Not part of the public header.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <limits>
#include <string>
#include <vector>

#include "../../include/mps_gb300.h"
#include "engine.cuh"

namespace mpsg {

// One step's record for the adjoint, in particle-id order (device memory).
// st*[0..5] = x, y, z, vx, vy, vz at: step start (st0), after the explicit
// part (st1, calcViscosity + moveParticles), after the collision pass (st2).
// Lists hold the ids of the neighbours (distance < re_max) found by the
// neighbour search before the explicit part (l0, at st0) and before the
// pressure part (l2, at st2), in the reference's sweep order, column-major
// with stride n (entry m of particle i at m * n + i).
struct TapeStep {
    double* st0[6];
    double* st1[6];
    double* st2[6];
    double* praw;           // PPE solution (pressure before removeNegativePressure)
    int8_t *type0, *type1;  // types at step start / after the explicit part
    int8_t *bc, *dir;       // boundary condition and Dirichlet connection of the pressure part
    int32_t *l0cnt, *l0id;
    int32_t *l2cnt, *l2id;
    CollPair* pairs;        // collision candidates in processing order (particle ids)
    int32_t* npairs;
    int32_t pair_cap;
};

enum TapePhase { TAPE_START, TAPE_LIST0, TAPE_EXPLICIT, TAPE_COLLISION, TAPE_LIST2, TAPE_SOLVE };

}  // namespace mpsg

struct mps_engine {
    int device = 0;
    cudaStream_t st = nullptr;
    mps_params P{};
    mpsg::Consts c{};
    int n = 0, n_pad = 0;
    mpsg::StateBuf buf[2]{};
    int cur = 0;
    mpsg::SortScratch sc{};
    mpsg::NbList nb{};
    mpsg::Ppe A{};
    mpsg::Krylov kv{};
    mpsg::MatFree mf{};
    mpsg::Mg mg{};
    // 0 Jacobi, 1 multigrid additive at level 0, 2 multiplicative, 3 additive
    // with the smoothed particle-to-cell transfer, 4 mode 1's preconditioner
    // with the operator pass after the cycle (mode 1 overlaps them)
    int32_t mg_requested = 1;
    // mode 1 may use the overlapped single-scene kernel (batch scenes share
    // the batched kernel, which has no overlapped form)
    int32_t cycle_overlap = 1;
    int32_t *cand_cnt = nullptr, *cand_base = nullptr;
    mpsg::CollWork cw{};
    mpsg::CollPair* pairs = nullptr;
    int32_t pair_cap = 0;
    int32_t* parent = nullptr;
    int8_t* has_surface = nullptr;
    double *ax = nullptr, *ay = nullptr, *az = nullptr;
    double* stage = nullptr;   // 9 n doubles for host transfers (pos, vel, p, p_min, ndr)
    int32_t* stage_i = nullptr;  // 3 n ints (type, bc, dirichlet)
    int32_t* dflag = nullptr;    // device flag of the upload checks
    mpsg::DevStats* ds = nullptr;
    mpsg::DevStats* hs = nullptr;  // pinned
    // per-step records of runs that wait once for many steps (mps_run_report):
    // every step appends its DevStats to `ring` at ring_pos (capacity
    // ring_cap); ring_t0 holds the device time at the start of such a run
    mpsg::DevStats* ring = nullptr;
    mpsg::DevStats* ring_host = nullptr;  // pinned
    int32_t* ring_pos = nullptr;
    unsigned long long* ring_t0 = nullptr;
    int32_t ring_cap = 256;
    int precision = MPS_PRECISION_FP64;
    double tol = std::numeric_limits<double>::epsilon();
    int64_t max_iter = 0;
    // the mixed solver starts from the last solve's solution (0: from zero)
    int32_t warm_start = 1;
    int32_t debug_log_count = 0;
    int32_t step_launches = 0;
    // CUDA graphs of a non-export step, one per buffer parity at step start
    // (a step swaps the state buffers an even or odd number of times).
    int32_t use_graph = 1;
    int32_t graph_broken = 0;  // capture was refused once: steps run eagerly
    cudaGraphExec_t gexec[2]{};
    int32_t graph_launches[2]{};
    int graph_end_parity[2]{};
    int32_t last_step_graphed = 0;
    // Set while a trajectory records a step for its adjoint (eager launches).
    const mpsg::TapeStep* tape = nullptr;
    cudaEvent_t ev[4]{};
    // asynchronous export (io.cu): device gather buffer, pinned host
    // snapshot, side stream; allocated on first use
    double* xdev = nullptr;   // 8 x n_pad: pos 3, vel 3, pressure, ndr
    int32_t* xdev_i = nullptr;  // 2 x n_pad: type, bc
    double* xhost = nullptr;
    int32_t* xhost_i = nullptr;
    cudaStream_t xst = nullptr;
    cudaEvent_t xev_ready = nullptr, xev_done = nullptr;
    int32_t x_pending = 0;
    std::vector<void*> allocs;

    template <typename T>
    cudaError_t alloc(T** p, size_t count) {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) {
            allocs.push_back(q);
            *p = (T*)q;
        }
        return e;
    }
    mpsg::StateBuf& S() { return buf[cur]; }
    void swap() { cur ^= 1; }
};

namespace mpsg {

#define MPSG_HIDDEN __attribute__((visibility("hidden")))

// mps_last_error() message of this thread.
MPSG_HIDDEN void set_last_error(const std::string& m);
// RefValues::RefValues (src/mps.cpp:132-163): n0 and lambda (lam may be NULL)
// of the 9x9(x9) lattice for radius re, in the reference's operation order.
MPSG_HIDDEN void ref_values(int dim, double l0, double re, double* n0, double* lam);
// Smallest t with sqrt_rn(t) >= re (0 for re <= 0): sqrt_rn(d2) < re <=> d2 < t.
MPSG_HIDDEN double sq_threshold(double re);
// Bucket::Bucket's cells per axis (src/bucket.cpp:10-22) for bucket length
// len; false (with the reason) unless the domain is finite with max >= min and
// fits, so that every axis has at least 3 cells.
MPSG_HIDDEN bool bucket_grid(const mps_params& P, double len, int32_t dims[3], std::string* why);
// One MPS::stepForward on the engine's stream, waits for it, fills stats and
// returns the step's status (graph replay unless exporting or taping).
MPSG_HIDDEN int engine_step(mps_engine* e, bool do_export, mps_step_stats* stats);
// Drops the captured step graphs (after any change of launch parameters).
MPSG_HIDDEN void engine_drop_graphs(mps_engine* e);
// The step's parts (enqueue only, on e->st): everything before the pressure
// solve; the mixed solver's per-step setup; everything after the solve.
MPSG_HIDDEN void engine_pre_solve(mps_engine* e);
MPSG_HIDDEN void engine_solver_setup(mps_engine* e);
MPSG_HIDDEN void engine_post_solve(mps_engine* e, bool do_export);
// The multigrid hierarchy as the mixed solver uses it (disabled if not requested).
MPSG_HIDDEN Mg engine_active_mg(const mps_engine* e);
// After the step's device stats reached e->hs: fills stats, returns the status.
MPSG_HIDDEN int engine_collect(mps_engine* e, mps_step_stats* stats);
// Records a phase of the running step into e->tape (adjoint.cu).
MPSG_HIDDEN void tape_phase(mps_engine* e, TapePhase ph);
// The reference's message for the first asymmetric pair of the last step's
// matrix (symcheck.cu; after a step that raised ST_ASYMMETRIC).
MPSG_HIDDEN std::string symmetry_message(const mps_engine* e);

}  // namespace mpsg
