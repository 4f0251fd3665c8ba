/*
 * mps_gb300 — C ABI of the GB300 (sm_103a) MPS time-step engine.
 *
 * The engine replaces the body of the reference's MPS class
 * (iori3150/MPS src/mps.hpp:22-71, src/mps.cpp:96-130) behind plain C
 * functions: host pointers and sizes in, status codes out, no C++ types.
 * The particle state lives on the GPU in structure-of-arrays form, sorted
 * by neighbour cell; it is copied in at create/upload and out at
 * download.  One engine drives one GPU (the device current at create) and
 * is single-threaded, like the reference's caller.
 *
 * Particle type codes follow ParticleType (src/particle.hpp:5):
 * Ghost -1, Fluid 0, Wall 1, DummyWall 2.  Boundary codes follow
 * BoundaryCondition (src/particle.hpp:20): Ignored 0, Surface 1, Inner 2.
 * Particle ids are array indices (src/mps.cpp:192,290 rely on the same).
 *
 * Every function returns MPS_OK (0) or an MPS_ERR_* code;
 * mps_last_error() returns the message of the last failure.
 */
#ifndef MPS_GB300_H
#define MPS_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    MPS_OK = 0,
    MPS_ERR_ARG = 1,         /* invalid argument (null pointer, bad size, bad setting) */
    MPS_ERR_CUDA = 2,        /* a CUDA call failed; the engine should be destroyed */
    MPS_ERR_CAPACITY = 3,    /* a capacity was exceeded: neighbour list, or mps_read_csv arrays */
    MPS_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up (kernel returned early) */
    MPS_ERR_NO_DEVICE = 5,   /* no CUDA device, or not an sm_103 part */
    MPS_ERR_NONFINITE = 6,   /* a particle position became NaN/inf; it was made a ghost */
    MPS_ERR_NOT_CONVERGED = 7, /* the pressure solve reached its iteration cap before its
                                  tolerance; the step completed with that pressure, as the
                                  reference's does (its solver.info() check, src/mps.cpp:462-464,
                                  only logs): a warning, not a failure of the engine */
    MPS_ERR_ASYMMETRIC = 8   /* the assembled PPE matrix is not symmetric: the step skipped the
                                solve (the reference exits, src/mps.cpp:418-442); the message
                                names the first pair as the reference prints it */
};

enum { MPS_PRECISION_FP64 = 0, MPS_PRECISION_MIXED = 1 };

/* Settings::load's values (src/settings.hpp:35-86) in absolute units:
 * radii and the collision distance are ratio * particle distance. */
typedef struct {
    int32_t dim;
    int32_t quasi_compressibility_on;
    int32_t higher_order_on;
    int32_t pad0;
    double particle_distance;
    double dt;
    double domain_min[3];
    double domain_max[3];
    double density;
    double kinematic_viscosity;
    double gravity[3];
    double re_pressure;
    double re_viscosity;
    double re_surface;
    double surface_threshold;
    double compressibility;
    double higher_order_gamma;
    double relaxation;
    double collision_distance;
    double restitution;
    double cfl;
} mps_params;

/* What one step reports (the reference returns only the Courant number,
 * src/mps.cpp:129, and counts debug events in MPS::debugLogCount). */
typedef struct {
    double courant;                 /* max |v| dt / l0 over fluid (src/mps.cpp:547-571) */
    double cg_relative_residual;    /* ||b - A x|| / ||b|| of the returned pressure */
    int64_t cg_iterations;          /* Krylov iterations (inner ones for MIXED) */
    int32_t refinements;            /* FP64 residual recomputations (MIXED), else 0 */
    int32_t debug_log_count;        /* cumulative, as MPS::debugLogCount */
    int32_t n_collision_candidates; /* pairs the collision pass tested (dist < cd) */
    int32_t n_new_ghosts;           /* particles that left the domain this step */
    int32_t n_unconnected;          /* Inner particles without a Dirichlet path */
    int32_t n_inner;
    int32_t n_surface;
    int32_t status;                 /* MPS_OK or the MPS_ERR_* of a device-side failure */
    float ms_step;                  /* device time of the whole step */
    float ms_solve;                 /* device time of the pressure solve */
    int32_t kernel_launches;        /* kernels this step launched */
    int64_t nnz_offdiag;            /* stored off-diagonal PPE entries */
    int32_t max_neighbors;          /* largest neighbour count of the last build */
    int32_t graph_replayed;         /* 1: the step ran as one CUDA graph replay */
    double solve_bytes;             /* algorithmic HBM bytes of the pressure solve (model:
                                       every array the solver kernels stream counted once
                                       per pass at its stored width) */
} mps_step_stats;

typedef struct mps_engine mps_engine;

/* MPS::MPS + MPS::loadInitialState (src/mps.cpp:18-36, 96-109): copies the
 * initial condition to the GPU and computes the initial number density.
 * pos/vel are n*3 doubles (x,y,z per particle), type n ints. */
int mps_create(const mps_params* prm, int32_t n, const double* pos, const double* vel,
               const int32_t* type, mps_engine** out);
int mps_destroy(mps_engine* e);

/* Pressure solver: MPS_PRECISION_FP64 is the reference's Jacobi-CG in FP64
 * (tolerance default machine epsilon, iteration cap default 2n, as Eigen's
 * defaults, src/mps.cpp:452-460).  MPS_PRECISION_MIXED runs FP32 Krylov
 * iterations with FP64 dot products inside FP64 iterative refinement until
 * ||b - A x|| <= tol ||b|| (default tol 1e-10).  tol <= 0 / max_iter <= 0
 * keep the defaults. */
int mps_set_solver(mps_engine* e, int32_t precision, double tol, int64_t max_iter);

/* The MIXED solver's preconditioner on planar scenes.  mode 0: Jacobi;
 * mode 1 (default): aggregation multigrid, additive at the particle level,
 * u = omega D^-1 r + scale P V(P^T r) with P the piecewise-constant
 * particle-to-cell transfer and V a V(1,1) cycle over the cell grids (one
 * operator pass per iteration, applied to D^-1 r while the cycle runs, and
 * A u assembled from it and the rows' 3x3-cell sums of A); mode 4: mode 1's
 * preconditioner with the operator applied to u after the cycle (the same
 * iteration in the order of the textbook loop; kept for comparison, and the
 * form every batch scene uses); mode 3: the same with the smoothed
 * transfer P = P1 - omega D^-1 A P1, applied through the rows' 3x3-cell sums
 * of A (fewer iterations, no extra operator pass); mode 2:
 * the multiplicative V(1,1) cycle from the particle level (three operator
 * passes per iteration).  omega = Jacobi weight in (0,1], scale =
 * coarse-correction weight in [1,2); 0 picks the mode's default (modes 1,
 * 3 and 4: 1.0, 1.4; mode 2: 0.9, 1.5).  No counterpart in the reference (its
 * CG is Jacobi-preconditioned). */
int mps_set_multigrid(mps_engine* e, int32_t mode, float omega, float scale);

/* Initial guess of the MIXED solver.  previous = 1 (default): each solve
 * starts from the previous step's solution of the same particles (before
 * the negative-pressure clamp; 0 for particles that had no unknown and at
 * the first step), kept across mps_upload; a guess whose residual exceeds
 * ||b|| (a state replaced by the upload) is dropped for zero by the solve
 * itself.  previous = 0: from zero, as the reference's CG (Eigen's solve(),
 * src/mps.cpp:452-460).  Either way the solve stops at
 * ||b - A x|| <= tol ||b||; only the iterations it takes change.  The FP64
 * solver always starts from zero. */
int mps_set_initial_guess(mps_engine* e, int32_t previous);

/* Self-test of the device-side wait limits (no counterpart in the
 * reference): runs the solver's grid barrier on 8 blocks in a group that
 * counts 9, so no block can pass; every block must give up with the timeout
 * status (its own spin limit, 2^16 polls here against the solver's 2^23,
 * ~2.4 s; or the flag of the first block that gave up) and the kernel ends
 * normally, leaving the context usable.
 * MPS_OK when all 8 gave up with that status. */
int mps_selftest_wait_limit(int32_t* blocks_gave_up, double* seconds);

/* How the collision pass (src/mps.cpp:217-250) applies its candidate pairs.
 * serial = 0 (default): in parallel, each pair after exactly the earlier
 * pairs that touch its particles; serial = 1: one thread in the reference's
 * order.  Both give the same state bit for bit (the serial form is kept for
 * verification, and is what the parallel pass falls back to when one
 * particle is the partner of more than 8 pairs in a step). */
int mps_set_collisions(mps_engine* e, int32_t serial);

/* Non-export steps run as a CUDA graph replay (default on): the first step
 * at each buffer parity captures the step's kernel sequence, later steps
 * replay it.  Changing the solver or the multigrid settings drops the
 * graphs.  Export steps always launch eagerly.  No counterpart in the
 * reference (its step is a sequence of OpenMP loops). */
int mps_set_graphs(mps_engine* e, int32_t enabled);

/* MPS::stepForward (src/mps.cpp:111-130). */
int mps_step(mps_engine* e, int32_t is_time_to_export, mps_step_stats* stats);

/* n_steps consecutive non-export steps; stats of the last step.  Stops at
 * the first step that returns a status other than MPS_OK. */
int mps_run(mps_engine* e, int32_t n_steps, mps_step_stats* stats);

/* n_steps consecutive non-export steps with one host wait per up to 256
 * steps (the driver loop of Simulation::run between two exports,
 * src/simulation.cpp:39-60, without a host round trip per step): stats[k]
 * (n_steps entries) holds step k's stats, as mps_step would report them,
 * with ms_step from device timestamps and ms_solve 0.  A step whose solve
 * reached its iteration cap does not stop the run (stats[k].status says so,
 * and the call returns MPS_ERR_NOT_CONVERGED at the end); any other failure
 * returns its status at once (that step's stats are the last filled; the
 * steps that followed it in the same group of 256 have run). */
int mps_run_report(mps_engine* e, int32_t n_steps, mps_step_stats* stats);

/* The symmetry test of solvePoissonEquation (src/mps.cpp:418-442) on a host
 * CSR matrix (n rows, row_ptr n+1, col/val row_ptr[n]; columns need not be
 * sorted), run by the same device kernels every step runs on the engine's
 * own matrix: MPS_OK, or MPS_ERR_ASYMMETRIC with the reference's first pair
 * i < j (row-major) whose entries differ by more than 1e-10, else the first
 * pair that differs at all, in *pair_i, *pair_j (-1 when symmetric) and the
 * reference's message in mps_last_error().  The engine's matrices are
 * bitwise symmetric by construction, so the engine treats any difference as
 * an error (the reference tolerates differences up to 1e-10).  The CSR is
 * checked on the host (MPS_ERR_ARG for bad row_ptr or column indices)
 * before it is copied to the device. */
int mps_check_symmetry(int32_t n, const int64_t* row_ptr, const int32_t* col, const double* val,
                       int32_t* pair_i, int32_t* pair_j);

/* Self-check of the correctly rounded FP64 square root and division that the
 * sweeps compute on the integer and FP32 pipes, against the GPU's FP64
 * instructions, on n seeded cases of each (random significands and
 * exponents, the significands next to 2^52 and 2^53, equal significands, the
 * sweeps' operand ranges), on the current device.  result[0] and result[1]:
 * square-root and quotient mismatches (0 when the routines are exact);
 * result[2] and result[3]: the cases that took the integer path (the others
 * are outside it: zero, subnormal, non-finite, or a quotient outside the
 * normal range); result[4..6]: the first mismatch's operand bits and its kind
 * (1 square root, 2 quotient), zeros if none; result[7]: mismatches of the
 * exact subtraction of 1 in the weight function, the FP32 rounding and the
 * distance-cutoff comparison done on the integer pipe.  result holds 8
 * values.  MPS_OK or MPS_ERR_CUDA. */
int mps_selftest_exact64(uint64_t n, uint64_t seed, uint64_t* result);

/* Asynchronous export (the reference's Simulation::exportParticles,
 * src/simulation.cpp:231-245, and Exporter, src/exporter.cpp:10-167).
 * mps_export_begin snapshots the current state in id order: gathers on the
 * engine's stream, then a copy into engine-owned pinned host memory on a
 * second stream, so that mps_step may go on at once.  mps_export_view waits
 * for the copy and returns pointers into the snapshot (valid until the next
 * mps_export_begin); mps_export_write waits and writes the reference's CSV
 * (Ghost particles skipped, six decimals) and ASCII VTU files (either path
 * may be NULL).  view/write may run on another thread while mps_step runs
 * on the same handle; mps_export_begin must not overlap a view or write. */
typedef struct {
    int32_t n;
    const double* pos;       /* 3n, x y z per particle */
    const double* vel;       /* 3n */
    const double* pressure;  /* n */
    const double* ndr;       /* n, number density ratio */
    const int32_t* type;     /* n, ParticleType (-1 Ghost) */
    const int32_t* bc;       /* n, BoundaryCondition */
} mps_snapshot;
int mps_export_begin(mps_engine* e);
int mps_export_view(mps_engine* e, mps_snapshot* out);
int mps_export_write(mps_engine* e, const char* csv_path, const char* vtu_path, double time);
/* The same writers on caller arrays (no engine, no device). */
int mps_write_snapshot(const mps_snapshot* s, const char* csv_path, const char* vtu_path, double time);

/* The reference's particle CSV import (MPS::importInitialCondition,
 * src/mps.cpp:38-94): "Time (s),t", a count line, a header line, then one
 * row per particle whose ID equals its row index (empty lines skipped);
 * columns found by name.  Host only.  Fills up to `capacity` particles
 * (pos/vel xyz-interleaved; any array may be NULL) and sets *n to the row
 * count; returns MPS_ERR_CAPACITY with *n set when capacity is too small. */
int mps_read_csv(const char* path, int32_t capacity, int32_t* n, double* time, double* pos,
                 double* vel, int32_t* type);

/* Particle state in id order (host pointers; any may be NULL). */
int mps_download(mps_engine* e, double* pos, double* vel, double* pressure,
                 double* min_pressure, double* ndr, int32_t* type, int32_t* bc,
                 int32_t* dirichlet);

/* Replace positions, velocities and types (same n) — the host-owned state
 * of the reference's std::vector<Particle>.  Any pointer may be NULL to keep
 * that field. */
int mps_upload(mps_engine* e, const double* pos, const double* vel, const int32_t* type);

int32_t mps_particle_count(const mps_engine* e);

/* The CUDA stream (cudaStream_t) the engine enqueues its kernels on, for
 * callers that time or order their own work against the step. */
void* mps_stream(mps_engine* e);

/* Parity/debug views of the last step, in id order. */
/* Neighbour lists of the last neighbour build (src/mps.cpp:585-619) as CSR;
 * call with ids == NULL to get the total in *total. */
int mps_neighbors(mps_engine* e, int64_t* offsets, int32_t* ids, double* dist, int64_t* total);
/* Source term and PPE matrix (CSR, ascending columns, Dirichlet fix applied). */
int mps_system(mps_engine* e, double* source, int64_t* row_ptr, int32_t* col, double* val,
               int64_t* nnz);
/* Collision candidate pairs (i, j, stale distance) in processing order. */
int mps_collisions(mps_engine* e, int32_t* pi, int32_t* pj, double* dist, int32_t* count);

const char* mps_last_error(void);

/* ------------------------------------------------------------------------
 * Differentiable trajectories.  No counterpart in the reference (its step
 * is not differentiated).  A trajectory runs n_steps of the engine from one
 * initial condition and maps (initial velocities, initial positions,
 * gravity) to (pressure at the sensor particles after every step, final
 * positions and velocities).  mps_trajectory_backward returns the
 * vector-Jacobian product of that map: a hand-written adjoint of the whole
 * step, with the step's discrete structure frozen at the forward's values
 * (neighbour sets, ghosts, surface flags, Dirichlet connections, collision
 * candidates, the negative-pressure clamp and the minimum-pressure
 * argument).  Memory is bounded by checkpoints every checkpoint_every steps:
 * the backward pass recomputes each segment with a tape and walks it in
 * reverse; the transpose Poisson solve is an FP64 CG (A is symmetric).
 * Arrays are in particle-id order, xyz interleaved (n*3 doubles).  The
 * engine's solver setting applies to the forward (FP64 gives the derivative
 * of exactly what is run).  Not supported with the higher-order source term.
 * ------------------------------------------------------------------------ */
typedef struct mps_trajectory mps_trajectory;

/* The engine's current positions, velocities and types become the initial
 * condition.  sensor_ids: particles whose pressure is recorded per step. */
int mps_trajectory_create(mps_engine* e, int32_t n_steps, int32_t checkpoint_every,
                          const int32_t* sensor_ids, int32_t n_sensors, mps_trajectory** out);
int mps_trajectory_destroy(mps_trajectory* t);

/* Runs the trajectory.  vel0 (n*3) replaces the initial velocities (NULL =
 * those at create or of the last forward), gravity (3) the engine's gravity
 * (NULL = keep).  Outputs (any may be NULL): sensor_pressure
 * [n_steps][n_sensors], pos_final and vel_final (n*3).  The engine is left
 * at the final state. */
int mps_trajectory_forward(mps_trajectory* t, const double* vel0, const double* gravity,
                           double* sensor_pressure, double* pos_final, double* vel_final);

/* Adjoint of the last forward: given dL/d(sensor_pressure), dL/d(pos_final),
 * dL/d(vel_final) (any may be NULL = zero), returns dL/d(pos0), dL/d(vel0)
 * (n*3) and dL/d(gravity) (3); planar engines report 0 for z.  Afterwards
 * the engine holds the forward's final positions, velocities and types. */
int mps_trajectory_backward(mps_trajectory* t, const double* d_sensor_pressure,
                            const double* d_pos_final, const double* d_vel_final, double* d_pos0,
                            double* d_vel0, double* d_gravity);

/* No counterpart in the reference.  The initial number density ratio pass of
 * loadInitialState (neighbour search + ratio, the values mps_create computes)
 * for callers that cannot allocate device memory: a host application that
 * owns all device memory itself and forbids library allocations, or a
 * timing-critical loop that cannot take an allocation's implicit
 * synchronisation.  It allocates nothing: d_pos (n*3 doubles), d_type (n
 * ints) and d_ndr (n doubles, output) are device pointers the caller owns,
 * and the scratch is a fixed ~5 MB static device array inside this library
 * (held on every GPU that loads it until the process exits).  Limits: at most
 * 65,536 particles and 262,144 bucket cells; larger requests and a
 * non-finite or inverted domain return MPS_ERR_ARG.  The first call on a
 * device looks up the scratch address (make it before any stream capture)
 * and keeps it for the process; it is not valid after cudaDeviceReset.
 * Calls share the scratch, so calls whose GPU work overlaps race: issue
 * them on one stream.  Work is enqueued
 * on `stream` (a cudaStream_t; NULL = the legacy default stream) and the
 * call returns without waiting. */
int mps_number_density_static(const mps_params* prm, int32_t n, const double* d_pos,
                              const int32_t* d_type, double* d_ndr, void* stream);

/* ------------------------------------------------------------------------
 * Batches: many independent scenes advanced together.  No counterpart in
 * the reference (one scene per process there).  Each scene is a full engine
 * with the MIXED solver; a batch step is one CUDA graph in which the scenes'
 * work before and after the pressure solve runs as parallel branches and
 * every scene's PPE is solved by ONE persistent cooperative launch whose
 * blocks are split into a group per scene (each group converges on its own
 * scene's tolerance).  The solve launch's block size (256/512/1024) and the
 * exponent alpha of its group-size model (blocks ~ rows^alpha) are picked by
 * an autotuner on the first step unless set with mps_batch_set_launch.
 * ------------------------------------------------------------------------ */
typedef struct mps_batch mps_batch;

/* Scene s has counts[s] particles and settings params[s]; pos, vel (n*3)
 * and type (n) hold the scenes' arrays one after another. */
int mps_batch_create(int32_t n_scenes, const mps_params* params, const int32_t* counts,
                     const double* pos, const double* vel, const int32_t* type, mps_batch** out);
int mps_batch_destroy(mps_batch* b);
/* Relative residual target of every scene's solve (default 1e-8), iteration cap. */
int mps_batch_set_solver(mps_batch* b, double tol, int64_t max_iter);
/* block = 0: autotune at the next step; else 256, 512 or 1024 with alpha in [0, 3]. */
int mps_batch_set_launch(mps_batch* b, int32_t block, double alpha);
/* Current launch shape, and the autotuner's per-candidate solve times (ms) in
 * the order block in {256, 512, 1024} x alpha in {1.0, 1.25, 1.5}. */
int mps_batch_launch_info(mps_batch* b, int32_t* block, double* alpha, int32_t* grid,
                          float* tune_ms, int32_t* n_tune);
/* Blocks of the solve launch given to each scene (n_scenes entries). */
int mps_batch_group_blocks(mps_batch* b, int32_t* blocks);
/* n_steps non-export steps of every scene; stats (n_scenes entries, may be
 * NULL) of the last step, with ms_step = the batch step's device time. */
int mps_batch_step(mps_batch* b, int32_t n_steps, mps_step_stats* stats, float* ms_last_step);
int32_t mps_batch_size(const mps_batch* b);
/* Borrowed engine of scene s (for downloads and views; not to be destroyed). */
mps_engine* mps_batch_scene(mps_batch* b, int32_t s);
/* The cudaStream_t the batch's graph runs on. */
void* mps_batch_stream(mps_batch* b);

#ifdef __cplusplus
}
#endif
#endif /* MPS_GB300_H */
