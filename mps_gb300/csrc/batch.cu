// Many independent scenes per step on one GPU.  No counterpart in the
// reference (one scene per process there).
//
// Every scene is a full engine (its own state, lists and matrix, in its own
// memory and stream).  A batch step is one CUDA graph: the scenes' work
// before the pressure solve runs as parallel branches (one per scene
// stream), then ONE persistent cooperative launch solves every scene's PPE —
// the blocks are split into one group per scene, each group with its own
// barrier, reductions and convergence test, so each scene stops at its own
// tolerance — and the scenes' work after the solve runs as parallel branches
// again.  Small scenes therefore share the GPU instead of each leaving most
// of it idle, and the step costs one graph launch.
//
// The solve launch's shape (threads per block, and the exponent alpha of the
// group-size model blocks_s ~ rows_s^alpha) is chosen by a small autotuner
// on the first step: every candidate solves that step's systems (the solve
// is idempotent: it starts from x = 0 and reads only the assembled system),
// the fastest is kept, and the step then finishes with it.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "engine_impl.cuh"

using namespace mpsg;

struct mps_batch {
    int device = 0;
    cudaStream_t st = nullptr;
    std::vector<mps_engine*> eng;
    std::vector<cudaEvent_t> ev_pre, ev_post;
    cudaEvent_t ev_fork = nullptr, t0 = nullptr, t1 = nullptr;
    BatchSolve bs;
    double tol = 1e-8;
    int64_t max_iter = 0;
    int32_t block = 0;  // 0: autotune at the next step
    double alpha = 1.0;
    std::vector<float> tune_ms;  // per candidate, in candidate order
    double* partials = nullptr;  // per scene: 2 x (max group) x 8 doubles
    int32_t max_grid = 0;
    cudaGraphExec_t gexec = nullptr;
    std::vector<int> graph_parity;
    int32_t graph_launches = 0;
    float last_ms = 0.f;
};

namespace {

int bfail(int code, const std::string& m) {
    set_last_error(m);
    return code;
}

#define BCU(call)                                                                                \
    do {                                                                                         \
        cudaError_t err_ = (call);                                                               \
        if (err_ != cudaSuccess)                                                                 \
            return bfail(MPS_ERR_CUDA, std::string(#call " failed: ") + cudaGetErrorString(err_)); \
    } while (0)

const int kBlocks[3] = {256, 512, 1024};
const double kAlphas[3] = {1.0, 1.25, 1.5};

void drop_graph(mps_batch* b) {
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    b->gexec = nullptr;
}

// warm = false: every scene's solve starts from zero (the autotuner's
// candidates solve the same systems one after another and must start alike).
int configure(mps_batch* b, int block, double alpha, bool warm = true) {
    std::vector<BatchScene> sc;
    const size_t per = (size_t)2 * b->max_grid * 8;
    for (size_t s = 0; s < b->eng.size(); s++) {
        mps_engine* e = b->eng[s];
        Krylov kv = e->kv;
        kv.partials = b->partials + s * per;
        const int64_t mi = b->max_iter > 0 ? b->max_iter : 2 * (int64_t)e->c.n;
        MatFree mf = e->mf;
        mf.skey = e->sc.skey;
        mf.cs = e->sc.cell_start;
        mf.numY = e->c.numY;
        mf.nkeys = e->c.nkeys;
        sc.push_back(BatchScene{e->c, e->A, mf, engine_active_mg(e), kv, e->ds, b->tol, mi,
                                warm ? e->warm_start : 0});
    }
    const int rc = batch_solve_setup(sc, block, alpha, b->device, b->bs);
    if (rc == 1) return bfail(MPS_ERR_ARG, "batch: more scenes than co-resident solver blocks");
    if (rc) return bfail(MPS_ERR_CUDA, "batch: solver setup failed");
    b->block = block;
    b->alpha = alpha;
    drop_graph(b);
    return MPS_OK;
}

// fork: every scene stream waits for the batch stream
void fork(mps_batch* b) {
    cudaEventRecord(b->ev_fork, b->st);
    for (mps_engine* e : b->eng) cudaStreamWaitEvent(e->st, b->ev_fork, 0);
}
void join(mps_batch* b, std::vector<cudaEvent_t>& evs) {
    for (size_t s = 0; s < b->eng.size(); s++) {
        cudaEventRecord(evs[s], b->eng[s]->st);
        cudaStreamWaitEvent(b->st, evs[s], 0);
    }
}

void enqueue_before_solve(mps_batch* b) {
    fork(b);
    for (mps_engine* e : b->eng) {
        cudaMemsetAsync(e->ds, 0, sizeof(DevStats), e->st);
        engine_pre_solve(e);
        engine_solver_setup(e);
    }
    join(b, b->ev_pre);
}

void enqueue_after_solve(mps_batch* b) {
    fork(b);
    for (mps_engine* e : b->eng) {
        engine_post_solve(e, false);
        cudaMemcpyAsync(e->hs, e->ds, sizeof(DevStats), cudaMemcpyDeviceToHost, e->st);
    }
    join(b, b->ev_post);
}

// First step with the autotuner: every candidate solves this step's systems.
int tuned_step(mps_batch* b) {
    enqueue_before_solve(b);
    b->tune_ms.clear();
    float best = 1e30f;
    int bb = 1024;
    double ba = 1.0;
    for (int blk : kBlocks)
        for (double al : kAlphas) {
            int rc = configure(b, blk, al, false);
            if (rc) return rc;
            float ms = 0.f;
            for (int rep = 0; rep < 2; rep++) {  // the second run is timed
                BCU(cudaEventRecord(b->t0, b->st));
                launch_solve_mixed_batched(b->bs, b->st);
                BCU(cudaEventRecord(b->t1, b->st));
                BCU(cudaStreamSynchronize(b->st));
                BCU(cudaEventElapsedTime(&ms, b->t0, b->t1));
            }
            b->tune_ms.push_back(ms);
            if (ms < best) {
                best = ms;
                bb = blk;
                ba = al;
            }
        }
    int rc = configure(b, bb, ba);
    if (rc) return rc;
    BCU(cudaEventRecord(b->t0, b->st));
    launch_solve_mixed_batched(b->bs, b->st);
    enqueue_after_solve(b);
    BCU(cudaEventRecord(b->t1, b->st));
    return MPS_OK;
}

int capture(mps_batch* b) {
    cudaGraph_t g = nullptr;
    BCU(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
    std::vector<int> par;
    for (mps_engine* e : b->eng) par.push_back(e->cur);
    g_launches = 0;
    enqueue_before_solve(b);
    launch_solve_mixed_batched(b->bs, b->st);
    enqueue_after_solve(b);
    const int32_t launches = g_launches;
    cudaError_t ce = cudaStreamEndCapture(b->st, &g);
    for (size_t s = 0; s < b->eng.size(); s++) b->eng[s]->cur = par[s];  // nothing ran yet
    if (ce != cudaSuccess || !g) {
        cudaGetLastError();
        return bfail(MPS_ERR_CUDA, std::string("batch: step capture failed: ") + cudaGetErrorString(ce));
    }
    ce = cudaGraphInstantiate(&b->gexec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
        b->gexec = nullptr;
        return bfail(MPS_ERR_CUDA, std::string("batch: graph instantiation failed: ") + cudaGetErrorString(ce));
    }
    b->graph_parity = par;
    b->graph_launches = launches;
    return MPS_OK;
}

}  // namespace

extern "C" {

int mps_batch_create(int32_t n_scenes, const mps_params* params, const int32_t* counts,
                     const double* pos, const double* vel, const int32_t* type, mps_batch** out) {
    if (n_scenes <= 0 || !params || !counts || !pos || !vel || !type || !out)
        return bfail(MPS_ERR_ARG, "mps_batch_create: bad arguments");
    *out = nullptr;
    auto* b = new mps_batch();
    cudaGetDevice(&b->device);
    auto bail = [&](int rc) {
        mps_batch_destroy(b);
        return rc;
    };
    size_t off = 0;
    for (int s = 0; s < n_scenes; s++) {
        if (counts[s] <= 0) return bail(bfail(MPS_ERR_ARG, "mps_batch_create: empty scene"));
        mps_engine* e = nullptr;
        int rc = mps_create(&params[s], counts[s], pos + 3 * off, vel + 3 * off, type + off, &e);
        if (rc) return bail(rc);
        e->cycle_overlap = 0;  // the batched solve kernel runs mode 1 in its plain form
        b->eng.push_back(e);
        if ((rc = mps_set_solver(e, MPS_PRECISION_MIXED, b->tol, 0))) return bail(rc);
        off += counts[s];
    }
    if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreate(&b->t0) != cudaSuccess || cudaEventCreate(&b->t1) != cudaSuccess)
        return bail(bfail(MPS_ERR_CUDA, "mps_batch_create: stream/event creation failed"));
    b->ev_pre.resize(n_scenes);
    b->ev_post.resize(n_scenes);
    for (int s = 0; s < n_scenes; s++)
        if (cudaEventCreateWithFlags(&b->ev_pre[s], cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->ev_post[s], cudaEventDisableTiming) != cudaSuccess)
            return bail(bfail(MPS_ERR_CUDA, "mps_batch_create: event creation failed"));
    for (int blk : kBlocks) b->max_grid = std::max(b->max_grid, batch_resident_grid(blk, b->device));
    if (b->max_grid < n_scenes)
        return bail(bfail(MPS_ERR_ARG, "mps_batch_create: more scenes than co-resident solver blocks"));
    if (cudaMalloc(&b->partials, sizeof(double) * 2 * b->max_grid * 8 * n_scenes) != cudaSuccess)
        return bail(bfail(MPS_ERR_CUDA, "mps_batch_create: cudaMalloc failed"));
    *out = b;
    return MPS_OK;
}

int mps_batch_destroy(mps_batch* b) {
    if (!b) return MPS_OK;
    if (b->st) cudaStreamSynchronize(b->st);
    drop_graph(b);
    batch_solve_free(b->bs);
    if (b->partials) cudaFree(b->partials);
    for (mps_engine* e : b->eng) mps_destroy(e);
    for (auto ev : b->ev_pre) cudaEventDestroy(ev);
    for (auto ev : b->ev_post) cudaEventDestroy(ev);
    for (cudaEvent_t ev : {b->ev_fork, b->t0, b->t1})
        if (ev) cudaEventDestroy(ev);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
    return MPS_OK;
}

int mps_batch_set_solver(mps_batch* b, double tol, int64_t max_iter) {
    if (!b) return bfail(MPS_ERR_ARG, "null batch");
    b->tol = tol > 0 ? tol : 1e-8;
    b->max_iter = max_iter > 0 ? max_iter : 0;
    for (mps_engine* e : b->eng) {
        int rc = mps_set_solver(e, MPS_PRECISION_MIXED, b->tol, b->max_iter);
        if (rc) return rc;
    }
    if (b->block) return configure(b, b->block, b->alpha);
    return MPS_OK;
}

int mps_batch_set_launch(mps_batch* b, int32_t block, double alpha) {
    if (!b) return bfail(MPS_ERR_ARG, "null batch");
    if (block == 0) {
        b->block = 0;
        drop_graph(b);
        return MPS_OK;
    }
    if (block != 256 && block != 512 && block != 1024)
        return bfail(MPS_ERR_ARG, "batch: block must be 0 (autotune), 256, 512 or 1024");
    if (!(alpha >= 0.0 && alpha <= 3.0)) return bfail(MPS_ERR_ARG, "batch: alpha outside [0, 3]");
    return configure(b, block, alpha);
}

int mps_batch_launch_info(mps_batch* b, int32_t* block, double* alpha, int32_t* grid,
                          float* tune_ms, int32_t* n_tune) {
    if (!b) return bfail(MPS_ERR_ARG, "null batch");
    if (block) *block = b->block;
    if (alpha) *alpha = b->alpha;
    if (grid) *grid = b->bs.grid;
    if (n_tune) *n_tune = (int32_t)b->tune_ms.size();
    if (tune_ms)
        for (size_t k = 0; k < b->tune_ms.size(); k++) tune_ms[k] = b->tune_ms[k];
    return MPS_OK;
}

int mps_batch_group_blocks(mps_batch* b, int32_t* blocks) {
    if (!b || !blocks) return bfail(MPS_ERR_ARG, "mps_batch_group_blocks: bad arguments");
    for (size_t s = 0; s < b->bs.group_blocks.size(); s++) blocks[s] = b->bs.group_blocks[s];
    return MPS_OK;
}

int mps_batch_step(mps_batch* b, int32_t n_steps, mps_step_stats* stats, float* ms_last_step) {
    if (!b || n_steps < 0) return bfail(MPS_ERR_ARG, "mps_batch_step: bad arguments");
    for (int32_t k = 0; k < n_steps; k++) {
        bool graphed = false;
        if (!b->block) {
            int rc = tuned_step(b);
            if (rc) return rc;
        } else {
            bool stale = !b->gexec;
            for (size_t s = 0; !stale && s < b->eng.size(); s++)
                stale = b->eng[s]->cur != b->graph_parity[s];
            if (stale) {
                drop_graph(b);
                int rc = capture(b);
                if (rc) return rc;
            }
            BCU(cudaEventRecord(b->t0, b->st));
            BCU(cudaGraphLaunch(b->gexec, b->st));
            BCU(cudaEventRecord(b->t1, b->st));
            // the graph performed each scene's buffer swaps
            for (size_t s = 0; s < b->eng.size(); s++) b->eng[s]->cur = b->graph_parity[s];
            graphed = true;
        }
        BCU(cudaStreamSynchronize(b->st));
        BCU(cudaGetLastError());
        BCU(cudaEventElapsedTime(&b->last_ms, b->t0, b->t1));
        int first_rc = MPS_OK;
        for (size_t s = 0; s < b->eng.size(); s++) {
            mps_engine* e = b->eng[s];
            mps_step_stats tmp;
            mps_step_stats* o = stats ? &stats[s] : &tmp;
            e->last_step_graphed = graphed ? 1 : 0;
            e->step_launches = graphed ? b->graph_launches : 0;
            int rc = engine_collect(e, o);
            o->ms_step = b->last_ms;
            o->ms_solve = 0.f;
            if (rc && !first_rc) first_rc = rc;
        }
        if (first_rc) return first_rc;
    }
    if (ms_last_step) *ms_last_step = b->last_ms;
    return MPS_OK;
}

int32_t mps_batch_size(const mps_batch* b) { return b ? (int32_t)b->eng.size() : 0; }

mps_engine* mps_batch_scene(mps_batch* b, int32_t s) {
    if (!b || s < 0 || s >= (int32_t)b->eng.size()) return nullptr;
    return b->eng[s];
}

void* mps_batch_stream(mps_batch* b) { return b ? (void*)b->st : nullptr; }

}  // extern "C"
