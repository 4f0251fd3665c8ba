/*
 * CPU oracle for the MPS time step — TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain C++/OpenMP restatement of the reference's hot path
 * (iori3150/MPS: src/mps.cpp, src/bucket.cpp, src/particle.cpp), kept
 * serial where the reference is serial and multi-threaded where it uses
 * OpenMP.  Only the test suite, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg load it; the product library never links or calls it.
 *
 * Parity pin: the restatement is checked bit-for-bit against golden
 * vectors produced by the reference's own src/mps.cpp, src/bucket.cpp,
 * src/particle.cpp and src/settings.cpp compiled with project-written
 * stand-ins for the absent third-party headers (oracle/ref_shim/).  The
 * Eigen ConjugateGradient inside those stand-ins is itself a restatement of
 * Eigen's published algorithm (the Eigen submodule is empty, its pinned
 * commit unknown), so the pressure solve is pinned to that published
 * algorithm, not to Eigen's binary arithmetic.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Physical and numerical settings, absolute units (radii already multiplied
 * by the particle distance, as Settings::load does, src/settings.cpp:43-56). */
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
} orc_params;

typedef struct orc_state orc_state;

typedef struct {
    double courant;
    int64_t cg_iterations;
    double cg_error;
    int32_t debug_log_count;      /* cumulative, like MPS::debugLogCount */
    int32_t n_collision_candidates;
    int32_t n_inner;
    int32_t n_surface;
} orc_stats;

/* Create from an initial condition (ids are array indices, as the reference
 * assumes).  Runs loadInitialState's setNumberDensity (src/mps.cpp:96-109). */
orc_state* orc_create(const orc_params* prm, int32_t n, const double* pos /*n*3*/,
                      const double* vel /*n*3*/, const int32_t* type);
void orc_destroy(orc_state* s);

/* CG controls: tolerance (default machine epsilon), maximum iterations
 * (default 2n) and the number of identical solves per step (default 2, as
 * src/mps.cpp:457,460 does). */
void orc_set_cg(orc_state* s, double tol, int64_t max_iter, int32_t solves);

/* One MPS::stepForward (src/mps.cpp:111-130). */
int orc_step(orc_state* s, int32_t is_time_to_export, orc_stats* out);

/* Current per-particle state. Any pointer may be NULL. */
void orc_get_state(const orc_state* s, double* pos, double* vel, double* pressure,
                   double* min_pressure, double* ndr, int32_t* type, int32_t* bc,
                   int32_t* dirichlet);

/* Neighbour lists as left by the last setNeighbors (CSR: offsets n+1). */
int64_t orc_neighbor_total(const orc_state* s);
void orc_get_neighbors(const orc_state* s, int64_t* offsets, int32_t* ids, double* dist);

/* Source term (n) and PPE matrix (CSR over all n rows, columns ascending,
 * Dirichlet fix applied) of the last step. */
int64_t orc_matrix_nnz(const orc_state* s);
void orc_get_system(const orc_state* s, double* source, int64_t* row_ptr, int32_t* col,
                    double* val);

/* Collision candidate pairs of the last step in processing order. */
int32_t orc_collision_count(const orc_state* s);
void orc_get_collisions(const orc_state* s, int32_t* pi, int32_t* pj, double* dist);

/* Lattice reference values n0 and lambda (src/mps.cpp:132-163). */
void orc_ref_values(int32_t dim, double l0, double re, double* n0, double* lambda);

#ifdef __cplusplus
}
#endif
