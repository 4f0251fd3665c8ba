// CPU oracle for the MPS time step — TEST INFRASTRUCTURE ONLY (see
// mps_oracle.h).  Every routine below restates one routine of the reference
// and cites it; the arithmetic is written out component by component in the
// reference's evaluation order, and the file is compiled with
// -ffp-contract=off so no multiply-add is fused.
#include "mps_oracle.h"

#include "cg_restated.hpp"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <queue>
#include <vector>

namespace {

enum Type : int32_t { Ghost = -1, Fluid = 0, Wall = 1, Dummy = 2 };  // src/particle.hpp:5
enum Bc : int32_t { Ignored = 0, Surface = 1, Inner = 2 };            // src/particle.hpp:20

struct V3 {
    double x, y, z;
};

// Eigen's squaredNorm/dot for a 3-vector; the order (x+y)+z is this
// restatement's choice (in 2-D every z term is exactly zero).
inline double sq_norm(const V3& a) { return (a.x * a.x + a.y * a.y) + a.z * a.z; }
inline double dot3(const V3& a, const V3& b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline V3 sub(const V3& a, const V3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }

// weight(): src/mps.cpp:9-16
inline double weight(double dist, double re) {
    double w = 0.0;
    if (dist < re) w = (re / dist) - 1.0;
    return w;
}

struct Nb {
    int32_t id;
    double dist;
};

struct Coll {
    int32_t i, j;
    double dist;
};

}  // namespace

struct orc_state {
    orc_params P{};
    int32_t n = 0;
    std::vector<V3> pos, vel, acc;
    std::vector<int32_t> type, bc, dirichlet;
    std::vector<double> pressure, min_pressure, ndr, density;
    std::vector<std::vector<Nb>> nbr;

    // Bucket (src/bucket.hpp:8-19)
    int32_t numX = 0, numY = 0, numZ = 0;
    double len = 0.0;
    std::vector<int32_t> first, last, next;

    double re_max = 0.0;
    double n0_p = 0, lam_p = 0, n0_v = 0, lam_v = 0, n0_s = 0, lam_s = 0;

    std::vector<double> source;
    std::vector<int64_t> row_ptr;
    std::vector<int32_t> col;
    std::vector<double> val;
    std::vector<Coll> coll;

    double cg_tol = std::numeric_limits<double>::epsilon();
    int64_t cg_max_iter = -1;
    int32_t cg_solves = 2;
    int64_t last_cg_iter = 0;
    double last_cg_err = 0.0;
    int32_t debug_log_count = 0;
};

namespace {

// RefValues::RefValues: src/mps.cpp:132-163
void ref_values(int dim, double l0, double re, double* n0_out, double* lam_out) {
    double n0 = 0.0, lam = 0.0;
    int z_begin = (dim == 2) ? 0 : -4;
    int z_end = (dim == 2) ? 1 : 5;
    for (int ix = -4; ix < 5; ix++)
        for (int iy = -4; iy < 5; iy++)
            for (int iz = z_begin; iz < z_end; iz++) {
                if (ix == 0 && iy == 0 && iz == 0) continue;
                V3 r{l0 * (double)ix, l0 * (double)iy, l0 * (double)iz};
                double dist = std::sqrt(sq_norm(r));
                double dist2 = dist * dist;
                n0 += weight(dist, re);
                lam += dist2 * weight(dist, re);
            }
    lam /= n0;
    *n0_out = n0;
    *lam_out = lam;
}

// Cell coordinate int((x - lo) / len) + 1 (src/bucket.cpp:40-42, src/mps.cpp:595-597).
// Where the reference would index outside its padded grid (a particle that a
// collision pushed past the domain edge, or a non-finite position) the
// coordinate is clamped to [1, cells - 2] so that the 3x3 sweep stays inside
// the grid; inside the domain the clamp never acts.
inline int cell_coord(double x, double lo, double len, int cells) {
    double q = (x - lo) / len;
    if (!(q >= 0.0)) return 1;
    if (q >= (double)(cells - 2)) return cells - 2;
    return (int)q + 1;
}

// Bucket::storeParticles: src/bucket.cpp:24-51 (serial, ascending id per cell)
void store_particles(orc_state& s) {
    std::fill(s.first.begin(), s.first.end(), -1);
    std::fill(s.last.begin(), s.last.end(), -1);
    std::fill(s.next.begin(), s.next.end(), -1);
    const orc_params& P = s.P;
    for (int32_t i = 0; i < s.n; i++) {
        if (s.type[i] == Ghost) continue;
        int ix = cell_coord(s.pos[i].x, P.domain_min[0], s.len, s.numX);
        int iy = cell_coord(s.pos[i].y, P.domain_min[1], s.len, s.numY);
        int iz = cell_coord(s.pos[i].z, P.domain_min[2], s.len, s.numZ);
        int b = ix + iy * s.numX + iz * s.numX * s.numY;
        if (s.last[b] == -1)
            s.first[b] = i;
        else
            s.next[s.last[b]] = i;
        s.last[b] = i;
    }
}

// MPS::setNeighbors: src/mps.cpp:585-619 (ghosts keep their stale list)
void set_neighbors(orc_state& s) {
    store_particles(s);
    const orc_params& P = s.P;
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < s.n; i++) {
        if (s.type[i] == Ghost) continue;
        std::vector<Nb>& list = s.nbr[i];
        list.clear();
        int ix = cell_coord(s.pos[i].x, P.domain_min[0], s.len, s.numX);
        int iy = cell_coord(s.pos[i].y, P.domain_min[1], s.len, s.numY);
        int iz = cell_coord(s.pos[i].z, P.domain_min[2], s.len, s.numZ);
        for (int jx = ix - 1; jx <= ix + 1; jx++)
            for (int jy = iy - 1; jy <= iy + 1; jy++)
                for (int jz = iz - 1; jz <= iz + 1; jz++) {
                    int b = jx + jy * s.numX + jz * s.numX * s.numY;
                    for (int j = s.first[b]; j != -1; j = s.next[j]) {
                        double dist = std::sqrt(sq_norm(sub(s.pos[j], s.pos[i])));
                        if (j != i && dist < s.re_max) list.push_back({j, dist});
                    }
                }
    }
}

// MPS::checkBoundaryViolation: src/mps.cpp:643-667
void check_boundary(orc_state& s, int32_t i) {
    const orc_params& P = s.P;
    const V3& x = s.pos[i];
    bool inside = true;
    if (x.x < P.domain_min[0] || P.domain_max[0] < x.x) inside = false;
    if (x.y < P.domain_min[1] || P.domain_max[1] < x.y) inside = false;
    if (x.z < P.domain_min[2] || P.domain_max[2] < x.z) inside = false;
    if (!inside) {
#pragma omp atomic
        s.debug_log_count++;
        s.type[i] = Ghost;
    }
}

double number_density(const orc_state& s, int32_t i, double re) {  // src/mps.cpp:573-583
    double nd = 0.0;
    for (const Nb& nb : s.nbr[i])
        if (nb.dist < re) nd += weight(nb.dist, re);
    return nd;
}

// MPS::setNumberDensity: src/mps.cpp:627-641
void set_number_density(orc_state& s) {
    set_neighbors(s);
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < s.n; i++) {
        if (s.bc[i] == Surface)
            s.ndr[i] = 0.0;
        else
            s.ndr[i] = number_density(s, i, s.P.re_pressure) / s.n0_p;
    }
}

// calcGravity + calcViscosity + moveParticles: src/mps.cpp:165-215
void explicit_part(orc_state& s) {
    const orc_params& P = s.P;
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < s.n; i++) {
        if (s.type[i] == Fluid)
            s.acc[i] = {P.gravity[0], P.gravity[1], P.gravity[2]};
        else
            s.acc[i] = {0.0, 0.0, 0.0};
    }
    const double re = P.re_viscosity;
    const double a = (P.kinematic_viscosity * (2.0 * (double)P.dim)) / (s.n0_v * s.lam_v);
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < s.n; i++) {
        if (s.type[i] != Fluid) continue;
        V3 t{0.0, 0.0, 0.0};
        const V3 vi = s.vel[i];
        for (const Nb& nb : s.nbr[i]) {
            if (nb.dist < re) {
                double w = weight(nb.dist, re);
                const V3& vj = s.vel[nb.id];
                t.x += (vj.x - vi.x) * w;
                t.y += (vj.y - vi.y) * w;
                t.z += (vj.z - vi.z) * w;
            }
        }
        s.acc[i].x += t.x * a;
        s.acc[i].y += t.y * a;
        s.acc[i].z += t.z * a;
    }
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < s.n; i++) {
        if (s.type[i] == Fluid) {
            V3& v = s.vel[i];
            V3& x = s.pos[i];
            v.x += s.acc[i].x * P.dt;
            v.y += s.acc[i].y * P.dt;
            v.z += s.acc[i].z * P.dt;
            x.x += v.x * P.dt;
            x.y += v.y * P.dt;
            x.z += v.z * P.dt;
            check_boundary(s, i);
        }
        s.acc[i] = {0.0, 0.0, 0.0};
    }
}

inline double inverse_density(const orc_state& s, int32_t i) {  // src/particle.cpp:19-29
    return s.type[i] == Fluid ? 1.0 / s.density[i] : 0.0;
}

// MPS::collision: src/mps.cpp:217-250 — serial, in place, id order.
void collision(orc_state& s) {
    const orc_params& P = s.P;
    s.coll.clear();
    for (int32_t i = 0; i < s.n; i++) {
        if (s.type[i] != Fluid) continue;
        for (const Nb& nb : s.nbr[i]) {
            const int32_t j = nb.id;
            const double dist = nb.dist;
            if (s.type[j] == Fluid && j >= i) continue;
            if (!(dist < P.collision_distance)) continue;
            s.coll.push_back({i, j, dist});
            double inv_i = inverse_density(s, i);
            double inv_j = inverse_density(s, j);
            double reduced = 1.0 / (inv_i + inv_j);
            V3 d = sub(s.pos[j], s.pos[i]);
            double z = sq_norm(d);
            V3 nrm = d;
            if (z > 0.0) {
                double r = std::sqrt(z);
                nrm = {d.x / r, d.y / r, d.z / r};
            }
            double rel = dot3(sub(s.vel[j], s.vel[i]), nrm);
            if (rel < 0.0) {
                double impulse = -(1.0 + P.restitution) * rel * reduced;
                double ci = impulse * inv_i, cj = impulse * inv_j;
                s.vel[i] = {s.vel[i].x - ci * nrm.x, s.vel[i].y - ci * nrm.y,
                            s.vel[i].z - ci * nrm.z};
                s.vel[j] = {s.vel[j].x + cj * nrm.x, s.vel[j].y + cj * nrm.y,
                            s.vel[j].z + cj * nrm.z};
                double depth = P.collision_distance - dist;
                double pimp = depth * reduced;
                double pi_ = pimp * inv_i, pj_ = pimp * inv_j;
                s.pos[i] = {s.pos[i].x - pi_ * nrm.x, s.pos[i].y - pi_ * nrm.y,
                            s.pos[i].z - pi_ * nrm.z};
                s.pos[j] = {s.pos[j].x + pj_ * nrm.x, s.pos[j].y + pj_ * nrm.y,
                            s.pos[j].z + pj_ * nrm.z};
            }
        }
    }
}

// MPS::setBoundaryCondition: src/mps.cpp:262-278
void set_boundary_condition(orc_state& s) {
    const double n0 = s.n0_s;
    const double beta = s.P.surface_threshold;
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < s.n; i++) {
        if (s.type[i] == Ghost || s.type[i] == Dummy)
            s.bc[i] = Ignored;
        else if (number_density(s, i, s.P.re_surface) < beta * n0)
            s.bc[i] = Surface;
        else
            s.bc[i] = Inner;
    }
}

// MPS::setSourceTerm: src/mps.cpp:280-320
void set_source_term(orc_state& s) {
    const orc_params& P = s.P;
    const double re = P.re_pressure;
    const double n0 = s.n0_p;
    const double dt = P.dt;
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < s.n; i++) {
        if (s.bc[i] != Inner) {
            s.source[i] = 0.0;
            continue;
        }
        if (P.higher_order_on) {
            const double gamma = P.higher_order_gamma;
            double b = gamma * (1.0 / (dt * dt)) * (s.ndr[i] - 1.0);
            for (const Nb& nb : s.nbr[i]) {
                if (s.bc[nb.id] == Ignored) continue;
                V3 r = sub(s.pos[nb.id], s.pos[i]);
                V3 u = sub(s.vel[nb.id], s.vel[i]);
                const double dist = nb.dist;
                if (dist < re) b -= (1.0 / (n0 * dt)) * re * dot3(r, u) / (dist * dist * dist);
            }
            s.source[i] = b;
        } else {
            const double gamma = P.relaxation;
            const double nd = number_density(s, i, re);
            s.source[i] = gamma * (1.0 / (dt * dt)) * (nd - n0) / n0;
        }
    }
}

// MPS::setMatrix: src/mps.cpp:322-360 (triplets -> CSR sorted by column)
void set_matrix(orc_state& s) {
    const orc_params& P = s.P;
    const double re = P.re_pressure;
    const double n0 = s.n0_p;
    const double lam = s.lam_p;
    const double D = (double)P.dim;
    std::vector<std::vector<std::pair<int32_t, double>>> rows(s.n);
    for (int32_t i = 0; i < s.n; i++) {
        if (s.bc[i] != Inner) continue;
        double cii = 0.0;
        for (const Nb& nb : s.nbr[i]) {
            if (s.bc[nb.id] == Ignored) continue;
            if (nb.dist < re) {
                double a = (2.0 * D / (lam * n0)) * weight(nb.dist, re) / s.density[i];
                cii += a;
                if (s.bc[nb.id] == Inner) rows[i].push_back({nb.id, -a});
            }
        }
        if (P.quasi_compressibility_on) cii += P.compressibility / (P.dt * P.dt);
        rows[i].push_back({i, cii});
    }
    s.row_ptr.assign(s.n + 1, 0);
    for (int32_t i = 0; i < s.n; i++) {
        std::sort(rows[i].begin(), rows[i].end(),
                  [](const auto& a, const auto& b) { return a.first < b.first; });
        s.row_ptr[i + 1] = s.row_ptr[i] + (int64_t)rows[i].size();
    }
    s.col.resize(s.row_ptr[s.n]);
    s.val.resize(s.row_ptr[s.n]);
    for (int32_t i = 0; i < s.n; i++) {
        int64_t k = s.row_ptr[i];
        for (auto& e : rows[i]) {
            s.col[k] = e.first;
            s.val[k] = e.second;
            k++;
        }
    }
}

// MPS::ensureDirichletBoundaryConnection: src/mps.cpp:362-415
void ensure_dirichlet(orc_state& s) {
    for (int32_t i = 0; i < s.n; i++) s.dirichlet[i] = (s.bc[i] == Surface) ? 1 : 0;
    const double re = s.P.re_pressure;
    for (int32_t i0 = 0; i0 < s.n; i0++) {
        if (s.bc[i0] != Surface) continue;
        std::queue<int32_t> q;
        q.push(i0);
        while (!q.empty()) {
            int32_t i = q.front();
            q.pop();
            for (const Nb& nb : s.nbr[i])
                if (nb.dist < re && !s.dirichlet[nb.id]) {
                    s.dirichlet[nb.id] = 1;
                    q.push(nb.id);
                }
        }
    }
    for (int32_t i = 0; i < s.n; i++) {
        if (!s.dirichlet[i] && s.bc[i] == Inner) {
            s.debug_log_count++;
            for (int64_t k = s.row_ptr[i]; k < s.row_ptr[i + 1]; k++)
                if (s.col[k] == i) s.val[k] *= 2.0;
        }
    }
}

// MPS::solvePoissonEquation: src/mps.cpp:417-470 (+ removeNegativePressure :472-479)
void solve_pressure(orc_state& s) {
    std::vector<double> x(s.n, 0.0);
    int64_t max_iter = s.cg_max_iter < 0 ? 2 * (int64_t)s.n : s.cg_max_iter;
    orc::CgResult r;
    for (int k = 0; k < std::max(1, s.cg_solves); k++)
        r = orc::cg_restated(s.n, s.row_ptr.data(), s.col.data(), s.val.data(),
                             s.source.data(), x.data(), s.cg_tol, max_iter);
    s.last_cg_iter = r.iterations;
    s.last_cg_err = r.error;
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < s.n; i++) s.pressure[i] = x[i];
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < s.n; i++)
        if (s.pressure[i] < 0.0) s.pressure[i] = 0.0;
}

// MPS::setMinimumPressure: src/mps.cpp:481-503
void set_minimum_pressure(orc_state& s) {
    const double re = s.P.re_pressure;
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < s.n; i++) {
        if (s.bc[i] == Ignored) continue;
        double m = s.pressure[i];
        for (const Nb& nb : s.nbr[i]) {
            if (s.type[nb.id] == Dummy) continue;
            if (nb.dist < re && m > s.pressure[nb.id]) m = s.pressure[nb.id];
        }
        s.min_pressure[i] = m;
    }
}

// calcPressureGradient + moveParticlesWithPressureGradient: src/mps.cpp:505-545
void pressure_gradient_and_move(orc_state& s) {
    const orc_params& P = s.P;
    const double re = P.re_pressure;
    const double n0 = s.n0_p;
    const double scale = (double)P.dim / n0;
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < s.n; i++) {
        if (s.type[i] != Fluid) continue;
        V3 g{0.0, 0.0, 0.0};
        const V3 xi = s.pos[i];
        const double pmin = s.min_pressure[i];
        for (const Nb& nb : s.nbr[i]) {
            if (s.type[nb.id] == Dummy) continue;
            const double dist = nb.dist;
            if (dist < re) {
                const V3& xj = s.pos[nb.id];
                double dp = s.pressure[nb.id] - pmin;
                double w = weight(dist, re);
                double d2 = dist * dist;
                g.x += (xj.x - xi.x) * dp * w / d2;
                g.y += (xj.y - xi.y) * dp * w / d2;
                g.z += (xj.z - xi.z) * dp * w / d2;
            }
        }
        g.x *= scale;
        g.y *= scale;
        g.z *= scale;
        s.acc[i] = {-1.0 * g.x / s.density[i], -1.0 * g.y / s.density[i],
                    -1.0 * g.z / s.density[i]};
    }
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < s.n; i++) {
        if (s.type[i] != Fluid) continue;
        V3& v = s.vel[i];
        V3& x = s.pos[i];
        const V3& a = s.acc[i];
        v.x += a.x * P.dt;
        v.y += a.y * P.dt;
        v.z += a.z * P.dt;
        x.x += a.x * P.dt * P.dt;
        x.y += a.y * P.dt * P.dt;
        x.z += a.z * P.dt * P.dt;
        check_boundary(s, i);
    }
}

// MPS::getCourantNumber: src/mps.cpp:547-571
double courant(orc_state& s) {
    double cmax = 0.0;
    for (int32_t i = 0; i < s.n; i++) {
        if (s.type[i] != Fluid) continue;
        double c = (std::sqrt(sq_norm(s.vel[i])) * s.P.dt) / s.P.particle_distance;
        cmax = std::max(cmax, c);
    }
    if (cmax > s.P.cfl) s.debug_log_count++;
    return cmax;
}

}  // namespace

extern "C" {

void orc_ref_values(int32_t dim, double l0, double re, double* n0, double* lambda) {
    ref_values(dim, l0, re, n0, lambda);
}

orc_state* orc_create(const orc_params* prm, int32_t n, const double* pos, const double* vel,
                      const int32_t* type) {
    orc_state* s = new orc_state();
    s->P = *prm;
    s->n = n;
    const orc_params& P = s->P;
    s->pos.resize(n);
    s->vel.resize(n);
    s->acc.assign(n, {0.0, 0.0, 0.0});
    s->type.assign(type, type + n);
    s->bc.assign(n, Ignored);
    s->dirichlet.assign(n, 0);
    s->pressure.assign(n, 0.0);
    s->min_pressure.assign(n, 0.0);
    s->ndr.assign(n, 0.0);
    s->density.assign(n, P.density);
    s->nbr.assign(n, {});
    s->source.assign(n, 0.0);
    for (int32_t i = 0; i < n; i++) {
        s->pos[i] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        s->vel[i] = {vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]};
    }
    // Settings::load (src/settings.cpp:43-56): re_max is the largest radius.
    s->re_max = std::max({P.re_pressure, P.re_viscosity, P.re_surface});
    ref_values(P.dim, P.particle_distance, P.re_pressure, &s->n0_p, &s->lam_p);
    ref_values(P.dim, P.particle_distance, P.re_viscosity, &s->n0_v, &s->lam_v);
    ref_values(P.dim, P.particle_distance, P.re_surface, &s->n0_s, &s->lam_s);
    // Bucket::Bucket: src/bucket.cpp:10-22
    s->len = s->re_max;
    s->numX = (int)((P.domain_max[0] - P.domain_min[0]) / s->len) + 3;
    s->numY = (int)((P.domain_max[1] - P.domain_min[1]) / s->len) + 3;
    s->numZ = (int)((P.domain_max[2] - P.domain_min[2]) / s->len) + 3;
    size_t cells = (size_t)s->numX * s->numY * s->numZ;
    s->first.assign(cells, -1);
    s->last.assign(cells, -1);
    s->next.assign(n, -1);
    set_number_density(*s);  // MPS::loadInitialState: src/mps.cpp:106
    return s;
}

void orc_destroy(orc_state* s) { delete s; }

void orc_set_cg(orc_state* s, double tol, int64_t max_iter, int32_t solves) {
    s->cg_tol = tol;
    s->cg_max_iter = max_iter;
    s->cg_solves = solves;
}

// MPS::stepForward: src/mps.cpp:111-130
int orc_step(orc_state* s, int32_t is_time_to_export, orc_stats* out) {
    set_neighbors(*s);
    explicit_part(*s);
    set_neighbors(*s);
    collision(*s);
    set_neighbors(*s);
    // MPS::calcPressure: src/mps.cpp:252-260
    set_boundary_condition(*s);
    set_source_term(*s);
    set_matrix(*s);
    ensure_dirichlet(*s);
    solve_pressure(*s);
    set_minimum_pressure(*s);
    pressure_gradient_and_move(*s);
    if (is_time_to_export || s->P.higher_order_on) set_number_density(*s);
    double c = courant(*s);
    if (out) {
        out->courant = c;
        out->cg_iterations = s->last_cg_iter;
        out->cg_error = s->last_cg_err;
        out->debug_log_count = s->debug_log_count;
        out->n_collision_candidates = (int32_t)s->coll.size();
        int32_t ni = 0, ns = 0;
        for (int32_t i = 0; i < s->n; i++) {
            ni += s->bc[i] == Inner;
            ns += s->bc[i] == Surface;
        }
        out->n_inner = ni;
        out->n_surface = ns;
    }
    return 0;
}

void orc_get_state(const orc_state* s, double* pos, double* vel, double* pressure,
                   double* min_pressure, double* ndr, int32_t* type, int32_t* bc,
                   int32_t* dirichlet) {
    for (int32_t i = 0; i < s->n; i++) {
        if (pos) {
            pos[3 * i] = s->pos[i].x;
            pos[3 * i + 1] = s->pos[i].y;
            pos[3 * i + 2] = s->pos[i].z;
        }
        if (vel) {
            vel[3 * i] = s->vel[i].x;
            vel[3 * i + 1] = s->vel[i].y;
            vel[3 * i + 2] = s->vel[i].z;
        }
        if (pressure) pressure[i] = s->pressure[i];
        if (min_pressure) min_pressure[i] = s->min_pressure[i];
        if (ndr) ndr[i] = s->ndr[i];
        if (type) type[i] = s->type[i];
        if (bc) bc[i] = s->bc[i];
        if (dirichlet) dirichlet[i] = s->dirichlet[i];
    }
}

int64_t orc_neighbor_total(const orc_state* s) {
    int64_t t = 0;
    for (const auto& l : s->nbr) t += (int64_t)l.size();
    return t;
}

void orc_get_neighbors(const orc_state* s, int64_t* offsets, int32_t* ids, double* dist) {
    int64_t k = 0;
    offsets[0] = 0;
    for (int32_t i = 0; i < s->n; i++) {
        for (const Nb& nb : s->nbr[i]) {
            ids[k] = nb.id;
            dist[k] = nb.dist;
            k++;
        }
        offsets[i + 1] = k;
    }
}

int64_t orc_matrix_nnz(const orc_state* s) { return s->row_ptr.empty() ? 0 : s->row_ptr.back(); }

void orc_get_system(const orc_state* s, double* source, int64_t* row_ptr, int32_t* col,
                    double* val) {
    if (source) std::memcpy(source, s->source.data(), sizeof(double) * s->n);
    if (s->row_ptr.empty()) {
        if (row_ptr)
            for (int32_t i = 0; i <= s->n; i++) row_ptr[i] = 0;
        return;
    }
    if (row_ptr) std::memcpy(row_ptr, s->row_ptr.data(), sizeof(int64_t) * (s->n + 1));
    if (col) std::memcpy(col, s->col.data(), sizeof(int32_t) * s->col.size());
    if (val) std::memcpy(val, s->val.data(), sizeof(double) * s->val.size());
}

int32_t orc_collision_count(const orc_state* s) { return (int32_t)s->coll.size(); }

void orc_get_collisions(const orc_state* s, int32_t* pi, int32_t* pj, double* dist) {
    for (size_t k = 0; k < s->coll.size(); k++) {
        pi[k] = s->coll[k].i;
        pj[k] = s->coll[k].j;
        dist[k] = s->coll[k].dist;
    }
}

}  // extern "C"
