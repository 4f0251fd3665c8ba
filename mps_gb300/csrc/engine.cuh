// Device-side data model and kernel entry points of the MPS engine.
//
// Layout in HBM: every per-particle field is a separate array ("slots"),
// kept sorted by neighbour-cell key so that the 3x3(x3) cell sweep of a
// particle reads a few contiguous slot ranges.  Each neighbour build
// re-sorts the state into the second of two buffers (StateBuf) and swaps.
// The particle id (its index in the reference's std::vector<Particle>)
// travels with the slot.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace mpsg {

// Kernels enqueued by this host thread (reported per step).
extern thread_local int32_t g_launches;

enum : int8_t { T_GHOST = -1, T_FLUID = 0, T_WALL = 1, T_DUMMY = 2 };
enum : int8_t { BC_IGNORED = 0, BC_SURFACE = 1, BC_INNER = 2 };

// Status bits raised on the device, reported through mps_step_stats.status.
enum : int32_t {
    ST_CAPACITY = 1,       // neighbour list overflow
    ST_TIMEOUT = 2,        // a bounded wait gave up
    ST_NONFINITE = 4,      // a particle position became NaN or infinite
    ST_NOT_CONVERGED = 8,  // the pressure solve stopped at its iteration cap
    ST_ASYMMETRIC = 16,    // the assembled PPE matrix is not symmetric (solve skipped)
};

// Constants of one scene, computed on the host with the reference's
// operation order (src/settings.cpp:43-56, src/mps.cpp:132-163 and the
// per-routine constant expressions).
struct Consts {
    int32_t dim;
    int32_t planar;   // z and v_z never change: sweep 3 cell columns, skip z arithmetic
    int32_t qc_on, ho_on;
    int32_t numX, numY, numZ, nkeys;
    int32_t K;        // neighbour-list capacity per particle
    int32_t n;        // particles
    double l0, dt;
    double dmin[3], dmax[3];
    double z0;        // the constant z of a planar scene
    double rho, g[3];
    double len;       // bucket edge = re_max
    double re_p, re_v, re_s, re_max, cd;
    // squared-distance thresholds: sqrt_rn(d2) < re  <=>  d2 < t_*
    double t_p, t_v, t_s, t_max, t_cd;
    double n0_p, n0_v, n0_s, lam_p, lam_v, lam_s;
    // FP32 squared-distance bounds of the candidate pre-filter: a candidate
    // whose FP32 squared distance exceeds one of these is certainly outside
    // that radius in exact FP64 (margin: the FP32 rounding of coordinates of
    // magnitude up to the domain bound), so only the rest get the exact test
    float ft_max, ft_v, ft_cd;
    // The mixed viscosity sweep decides "inside the radius" from the FP32
    // squared distance of its coordinate pairs when that lies outside
    // [fv_in, fv_out], a band of 2^-16 relative around the exact threshold
    // min(t_max, t_v) that holds the pairs' error bound (2^-20) many times;
    // inside the band it runs the exact FP64 test.
    float fv_in, fv_out;
    double beta_n0s;    // beta * n0 (src/mps.cpp:271)
    double visc_a;      // nu * (2 dim) / (n0 lambda)           src/mps.cpp:182
    double mat_c;       // 2 D / (lambda n0)                     src/mps.cpp:343
    double qc_term;     // alpha / (dt dt)                       src/mps.cpp:354
    double src_g1;      // gamma * (1 / (dt dt))                 src/mps.cpp:313
    double ho_g1;       // gamma_ho * (1 / (dt dt))              src/mps.cpp:291
    double ho_c;        // 1 / (n0 dt)                           src/mps.cpp:304
    double grad_scale;  // dim / n0                              src/mps.cpp:530
    double e;           // restitution
    float fre_v, fre_p, fvisc_a, fgrad_scale;  // FP32 copies for the mixed path
};

struct StateBuf {
    double *x, *y, *z, *vx, *vy, *vz;
    // FP32 copies of the positions, x and y interleaved (one 8-byte load per
    // candidate in the neighbour sweeps' pre-filter), written by the rebuild gather
    float2* xyf;
    float* zf;
    // The mixed step's FP32 work on planar scenes (written by the rebuild
    // gather unless noted): the low parts x - xyf and y - xyf rounded to FP32
    // (so that a coordinate difference is formed from FP32 pairs to within
    // FP32 rounding of the difference itself), the FP32 velocities, and the
    // pressure split the same way (hi, lo; written after the solve).
    float2* xylo;
    float2* vf;
    float2* pf;
    double *p, *minp, *ndr, *nd_last;
    int32_t* id;
    int8_t *type, *bc, *dir;
};

// Per-step device counters (one struct in device memory, copied out once per step).
struct DevStats {
    unsigned long long courant_bits;  // max of non-negative doubles via integer max
    int32_t status;
    int32_t n_new_ghosts;
    int32_t n_unconnected;
    int32_t n_cand;
    int32_t n_cand_particles;
    int32_t n_inner;
    int32_t n_surface;
    int32_t max_neighbors;
    int64_t cg_iterations;
    int32_t refinements;
    int32_t pad;
    double cg_rel_residual;
    unsigned long long nnz_off;
    int32_t upload_flag;  // host copy of mps_upload's device checks
    int32_t pad2;
    // symmetry check of the assembled matrix (symcheck.cu): the sum over
    // stored off-diagonal entries of +-hash(pair) * bits(value) mod 2^64 (0 for
    // a bitwise symmetric matrix), and, only when it is not 0, the first
    // asymmetric pair in id order stored as ~(i << 32 | j) (0: none), once for
    // pairs whose values differ by more than 1e-10 and once for any difference
    unsigned long long sym_fp;
    unsigned long long asym_big;
    unsigned long long asym_any;
    unsigned long long t_end;  // device time (ns) at the end of the step, in its per-step record
};

struct CollPair {
    int32_t si, sj;  // slots
    int32_t ii, ij;  // particle ids
    double dist;     // distance at detection (the reference's stale neighbour distance)
};

// ----------------------------------------------------------------- sort.cu
struct SortScratch {
    int32_t *key, *rank, *perm, *skey;  // per slot
    int32_t *cell_count, *cell_start;   // nkeys + 2
    int32_t *scan_tmp;                  // block sums
};
void launch_rebuild(const Consts& c, const StateBuf& in, const StateBuf& out, SortScratch& s,
                    DevStats* ds, cudaStream_t st);
// exclusive scan of n int32 (in-place allowed); out has n+1 entries (total last)
void launch_exclusive_scan(const int32_t* in, int32_t* out, int32_t n, int32_t* tmp,
                           cudaStream_t st);
size_t scan_tmp_ints(int32_t n);

// --------------------------------------------------------------- sweeps.cu
struct NbList {
    int32_t* cnt;    // per slot
    int32_t* slot;   // K x n_pad, column-major (entry m of slot k at m * n_pad + k)
    double* dist;
    double* wp;      // weight(dist, re_p)
    int32_t n_pad;
};

struct Ppe {
    double* src;      // per slot
    double* diag;     // per slot (0 for rows that are not Inner)
    int32_t* offcnt;  // per slot
    int32_t* col;     // SELL-32, width K: ((slot/32)*K + m)*32 + slot%32; padding = (own slot, 0)
    double* val;
    int32_t* slice_w; // max offcnt of each 32-slot slice
    float* val32;     // FP32 copy of val, quad layout (qsell_index) for the mixed solver
    float* diag32;
    // Row sums diag + sum of the row's off-diagonals, formed in FP64 from the
    // assembly's terms (the compressibility term plus the weights of
    // neighbours that are not unknowns; Dirichlet doubling added), and their
    // FP32 rounding.  The mixed solver applies its FP32 operator as
    // sum_j a_ij (v_j - v_i) + rsum_i v_i: on smooth vectors the FP32 sum of
    // a_ij v_j cancels to a small row sum and loses it, and the FP32-rounded
    // entries do not sum to it.
    double* rsum;
    float* rsum32;
};

// Quad SELL-32 layout of the mixed solver's FP32 operator: entry m of slot k
// at ((k/32) * K/4 + m/4) * 128 + (k%32) * 4 + m%4, i.e. each thread's next
// four entries are one 16-byte word and the warp's words are contiguous.
__host__ __device__ __forceinline__ size_t qsell_index(int k, int m, int K) {
    return ((size_t)(k >> 5) * (K >> 2) + (m >> 2)) * 128 + (size_t)(k & 31) * 4 + (m & 3);
}

// Compact FP32 form of the PPE operator for the mixed solver (planar
// scenes): SELL-32 like the FP64 matrix, but each entry is an FP32 value and
// one index byte: 2 bits for which of the row's 3 candidate column ranges
// (cells jx = ix-1, ix, ix+1 of its neighbour sweep) holds the column, 6 bits
// for the offset inside that range; the range starts come from the cell
// table.  5 B per entry instead of the FP64 matrix's 12 B.
struct MatFree {
    uint8_t* idx8;              // quad SELL-32 layout like Ppe::val32
    int8_t* sell_row;           // 1: this row uses the int32 SELL columns instead
    int32_t* rs;                // per slot: the 3 range starts (3 x rs_stride)
    int32_t rs_stride;
    const int32_t* skey;        // cell key per slot (from the last rebuild)
    const int32_t* cs;          // cell start table
    int32_t numY;
    int32_t nkeys;              // cells (ghost slots carry the sentinel key nkeys)
    int32_t enabled;            // planar scenes only
};

void launch_initial_number_density(const Consts& c, const StateBuf& s, const SortScratch& sc,
                                   const NbList& nb, DevStats* ds, cudaStream_t st);
void launch_explicit(const Consts& c, const StateBuf& in, const StateBuf& out,
                     const SortScratch& sc, int mixed, DevStats* ds, cudaStream_t st);
// Buffers of the collision pass's parallel application (sweeps.cu).
constexpr int kCollJList = 8;
struct CollWork {
    int32_t* jn;     // per particle id: pairs that have it as the fluid partner j
    int32_t* jl;     // per id: up to kCollJList of those pairs' indices (id * kCollJList + k)
    int32_t* ver;    // per id: pairs applied so far that touch the particle
    int32_t* ctl;    // [0] chunk ticket, [1] list overflow (the serial pass runs), [2] abort
    int32_t serial;  // 1: every pair applied by one thread in order (verification mode)
};
void launch_collision(const Consts& c, const StateBuf& s, const SortScratch& sc,
                      int32_t* cand_cnt, int32_t* cand_base, const CollWork& cw, CollPair* pairs,
                      int32_t pair_cap, int32_t* scan_tmp, DevStats* ds, cudaStream_t st);
void launch_build_list(const Consts& c, const StateBuf& s, const SortScratch& sc,
                       const NbList& nb, DevStats* ds, cudaStream_t st);
// The pressure part's build: the list, and with it setBoundaryCondition and
// setSourceTerm (src/mps.cpp:262-320; the higher-order source after it).
void launch_build_list_bc_source(const Consts& c, const StateBuf& s, const SortScratch& sc,
                                 const NbList& nb, const Ppe& A, DevStats* ds, cudaStream_t st);
void launch_assemble(const Consts& c, const StateBuf& s, const NbList& nb, const Ppe& A,
                     DevStats* ds, cudaStream_t st);
void launch_dirichlet(const Consts& c, const StateBuf& s, const NbList& nb, const Ppe& A,
                      int32_t* parent, int8_t* has_surface, DevStats* ds, cudaStream_t st);
// --------------------------------------------------------------- symcheck.cu
// The symmetry test of solvePoissonEquation (src/mps.cpp:418-442) on the
// assembled matrix: a one-pass fingerprint, and the first asymmetric pair
// when it is not zero; raises ST_ASYMMETRIC, which makes the solvers skip.
void launch_symmetry_check(const Consts& c, const StateBuf& s, const Ppe& A, DevStats* ds,
                           cudaStream_t st);
// The second half alone, after a kernel that accumulated the fingerprint
// (the mixed setup does, over slots, while it reads the matrix).
void launch_symmetry_locate(const Consts& c, const StateBuf& s, const Ppe& A, DevStats* ds,
                            cudaStream_t st);
// x_prev (may be null) receives the solution by particle id.
void launch_pressure_post(const Consts& c, const StateBuf& s, const NbList& nb,
                          const double* x, double* x_prev, double* ax, double* ay, double* az,
                          int mixed, DevStats* ds, cudaStream_t st);
void launch_number_density(const Consts& c, const StateBuf& s, const NbList& nb,
                           cudaStream_t st);

// Aggregation multigrid preconditioner of the mixed solver (planar scenes).
// Level 1 aggregates the particles of each bucket cell (the slots of a cell
// are contiguous), so it is the structured numX x numY cell grid with a
// 9-point stencil (a particle's neighbours lie in the 3x3 cells around it);
// each further level aggregates 2x2 cells and is again a 9-point grid.
// Coarse operators are Galerkin products with piecewise-constant transfer,
// built in a fixed order (deterministic); the coarsest level (<= 96
// unknowns) is solved with its dense inverse.
constexpr int kMgMaxLevels = 16;
// Levels with at most this many cells run in one block (between two grid
// barriers); larger ones run grid-wide.
constexpr int kMgBlockCells = 1024;
constexpr int kMgMaxCoarsest = 96;
struct MgLevel {
    int32_t nx, ny;
    float* st;    // 9 x (nx*ny), direction d = (dx+1)*3 + (dy+1), d = 4 is the diagonal
    float* invd;  // 1 / diagonal, 0 for cells without unknowns
    float *r, *e, *t;
    // levels >= 2: restriction weights, 16 x (nx*ny).  Coarse cell (X, Y)
    // gets the pre-smoothed residual of the finer level as
    // sum_k rw[k] r_f(2X - 1 + k / 4, 2Y - 1 + k % 4): the 2x2 children's
    // residuals after one Jacobi step from zero, folded into one 4x4 stencil
    // on the finer residual alone
    float* rw;
    // the cells with unknowns (invd > 0), listed by the setup in warp-sized
    // runs of ascending index; Mg::nact[l] of them.  The grid-wide phases of
    // the cycle visit only these: every other cell holds 0 in r, e and t
    // (cleared by the setup), which is what the full loops used to write
    int32_t* act;
};
struct Mg {
    int32_t enabled;
    int32_t nlev;   // coarse levels 1..nlev
    int32_t ngrid;  // levels 1..ngrid run grid-wide; ngrid+1..nlev run in block 0
    MgLevel lev[kMgMaxLevels];
    float* e0;      // level-0 correction (per slot)
    float* res0;    // level-0 residual (per slot)
    float* dense;   // inverse of the coarsest operator (cells x cells of level nlev)
    float omega;    // damped-Jacobi weight
    float scale;    // coarse-correction scale
    // 0: multiplicative V(1,1) from level 0 (Jacobi pre- and post-smoothing
    // around the coarse correction); 1: additive at level 0, u = omega D^-1 r
    // + scale P V1(P^T r) (no level-0 operator pass; still SPD)
    int32_t additive;
    // additive with a smoothed particle-to-cell transfer: P = P1 - omega D^-1 A P1
    // in place of P1 (the cell levels keep the operators of plain aggregation)
    int32_t smooth;
    // additive (plain transfer) in the overlapped arrangement of the
    // single-scene solve: the level-0 operator is applied to D^-1 r while the
    // cell levels run, and A u is assembled from it and B e1 (solver.cu,
    // solve_mixed_overlap)
    int32_t overlap;
    // B = A P1 per slot: the operator row's sums over the 3x3 cells around the
    // slot's own, entry d = (dx+1)*3 + (dy+1), diagonal included (9 x n_pad)
    float* rowcell;
    int32_t n_pad;
    int32_t* nact;  // per level: the length of lev[l].act (device, written by the setup)
    int2* act1_rng; // per entry of lev[1].act: the cell's first slot and slot count
    // per slot, for the overlapped solve's fused level-1 sums: if the slot is
    // the last of a level-1 cell with unknowns, cell | min(slots, 255) << 24,
    // else -1 (n_pad)
    int32_t* cell_end;
};

// --------------------------------------------------------------- solver.cu
struct Krylov {
    double *x, *r, *p, *q, *z, *inv_diag;
    // the last solve's solution (before the negative-pressure clamp) by
    // particle id: the mixed solver's initial guess at the next step
    double* x_prev;
    float *r32, *p32, *s32, *w32, *x32, *u32, *inv_diag32;
    double* partials;       // 2 x grid x 8 per-block partial sums
    unsigned int* barrier;  // monotonically increasing arrival counter
    double* totals;         // unused scratch (8 doubles)
    int32_t grid;           // cooperative grid size
    int32_t block;
};
void solver_setup(Krylov& k, int32_t n_pad, int device);
// Runs the grid barrier with one block that never arrives on `blocks`
// blocks; reports how many gave up, the status word and the kernel time.
int selftest_wait_limit(int blocks, int* gave_up, int* status, float* ms);
// Solves A x = b; returns through DevStats (iterations, residual, status).
void launch_solve_fp64(const Consts& c, const Ppe& A, const Krylov& k, double tol,
                       int64_t max_iter, DevStats* ds, cudaStream_t st);
// warm: x already holds the initial guess (launch_mixed_setup), else the
// solve starts from zero.
void launch_solve_mixed(const Consts& c, const Ppe& A, const MatFree& mf, const Mg& mg,
                        const Krylov& k, double tol, int64_t max_iter, bool warm, DevStats* ds,
                        cudaStream_t st);
// Batched mixed-precision solve: many scenes in one cooperative launch, the
// blocks split into one group per scene (group sizes ~ rows^alpha), each
// group with its own barrier, reductions and convergence test.
struct BatchScene {
    Consts c;
    Ppe A;
    MatFree mf;
    Mg mg;
    Krylov kv;
    DevStats* ds;
    double tol;
    int64_t max_iter;
    int32_t warm;  // the scene's x holds its initial guess (mps_set_initial_guess)
};
struct BatchSolve {
    int32_t n_scenes = 0;
    void* scenes = nullptr;         // device array of per-scene solve descriptors
    int2* bmap = nullptr;           // per block: (scene, rank in the scene's group)
    int32_t* gsize = nullptr;       // per scene: blocks in its group
    unsigned int* bars = nullptr;   // per scene: barrier counter (128-byte stride)
    int32_t block = 0, grid = 0;
    double alpha = 0.0;
    std::vector<int32_t> group_blocks;
};
// Blocks of `block` threads (256, 512 or 1024) co-resident on the device.
int batch_resident_grid(int block, int device);
void batch_group_sizes(const std::vector<int32_t>& rows, double alpha, int grid,
                       std::vector<int32_t>& out);
// 0 on success; 1 if the device holds fewer blocks than scenes; 2 on a CUDA error.
int batch_solve_setup(const std::vector<BatchScene>& scenes, int block, double alpha, int device,
                      BatchSolve& b);
void batch_solve_free(BatchSolve& b);
void launch_solve_mixed_batched(const BatchSolve& b, cudaStream_t st);
// Per-solve multigrid setup (after launch_mixed_setup).
void launch_mg_setup(const Consts& c, const Ppe& A, const MatFree& mf, const Mg& mg,
                     cudaStream_t st);
// FP32 copy of the assembled matrix in the compact layout of MatFree; with
// warm set, also the solve's initial guess x (k.x_prev at the slots' ids on
// rows with a diagonal, else 0); and the symmetry fingerprint of the matrix
// (over slots) into ds->sym_fp, for launch_symmetry_locate.
void launch_mixed_setup(const Consts& c, const SortScratch& sc, const Ppe& A, MatFree& mf,
                        const Krylov& k, const int32_t* ids, bool warm, DevStats* ds, cudaStream_t st);

}  // namespace mpsg
