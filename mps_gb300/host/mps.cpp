#include "mps.hpp"

#include <cmath>
#include <cstdlib>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "logger.hpp"

namespace {
void check(int rc) {
    if (rc != MPS_OK) throw std::runtime_error(std::string("mps engine: ") + mps_last_error());
}
double weight(double dist, double re) { return dist < re ? (re / dist) - 1.0 : 0.0; }
}  // namespace

// src/mps.cpp:132-163
RefValues::RefValues(const int& dim, const double& l0, const double& re) {
    int zb = dim == 2 ? 0 : -4, ze = dim == 2 ? 1 : 5;
    for (int ix = -4; ix < 5; ix++)
        for (int iy = -4; iy < 5; iy++)
            for (int iz = zb; iz < ze; iz++) {
                if (ix == 0 && iy == 0 && iz == 0) continue;
                Vec3 r(l0 * (double)ix, l0 * (double)iy, l0 * (double)iz);
                double dist = r.norm();
                initialNumberDensity += weight(dist, re);
                lambda += (dist * dist) * weight(dist, re);
            }
    lambda /= initialNumberDensity;
}

// src/mps.cpp:18-36
MPS::MPS(const std::filesystem::path& inputYamlPath) {
    settings.load(inputYamlPath);
    refValues.pressure = RefValues((int)settings.dim, settings.particleDistance, settings.effectiveRadius.pressure);
    refValues.viscosity = RefValues((int)settings.dim, settings.particleDistance, settings.effectiveRadius.viscosity);
    refValues.surfaceDetection =
        RefValues((int)settings.dim, settings.particleDistance, settings.effectiveRadius.surfaceDetection);
}

// src/mps.cpp:38-94: the CSV written by Exporter::toCsv; ids must be the row
// indices (the reference indexes particles by id).
double MPS::importInitialCondition() {
    // the engine's reader (one read, rows parsed on several threads)
    const std::string path = settings.inputCsvPath.string();
    int32_t n = 0;
    double t0 = 0.0;
    int rc = mps_read_csv(path.c_str(), 0, &n, &t0, nullptr, nullptr, nullptr);
    if (rc != MPS_OK && rc != MPS_ERR_CAPACITY) throw std::runtime_error(mps_last_error());
    std::vector<double> pos(3 * (size_t)n), vel(3 * (size_t)n);
    std::vector<int32_t> type(n);
    rc = mps_read_csv(path.c_str(), n, &n, &t0, pos.data(), vel.data(), type.data());
    if (rc != MPS_OK) throw std::runtime_error(mps_last_error());
    particles.clear();
    particles.reserve(n);
    for (int32_t i = 0; i < n; i++)
        particles.emplace_back(i, static_cast<ParticleType>(type[i]), Vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]),
                               Vec3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]), settings.density);
    return t0;
}

// src/mps.cpp:96-109: import, upload, initial number density.
double MPS::loadInitialState() {
    double t0 = importInitialCondition();
    mps_params p{};
    p.dim = (int32_t)settings.dim;
    p.quasi_compressibility_on = settings.quasiCompressibility.on;
    p.higher_order_on = settings.higherOrderSourceTerm.on;
    p.particle_distance = settings.particleDistance;
    p.dt = settings.dt;
    p.domain_min[0] = settings.domain.x.min;
    p.domain_min[1] = settings.domain.y.min;
    p.domain_min[2] = settings.domain.z.min;
    p.domain_max[0] = settings.domain.x.max;
    p.domain_max[1] = settings.domain.y.max;
    p.domain_max[2] = settings.domain.z.max;
    p.density = settings.density;
    p.kinematic_viscosity = settings.kinematicViscosity;
    for (int i = 0; i < 3; i++) p.gravity[i] = settings.gravity[i];
    p.re_pressure = settings.effectiveRadius.pressure;
    p.re_viscosity = settings.effectiveRadius.viscosity;
    p.re_surface = settings.effectiveRadius.surfaceDetection;
    p.surface_threshold = settings.thresholdForSurfaceDetection;
    p.compressibility = settings.quasiCompressibility.compressibility;
    p.higher_order_gamma = settings.higherOrderSourceTerm.gamma;
    p.relaxation = settings.relaxationCoefficientForPressure;
    p.collision_distance = settings.collisionDistance;
    p.restitution = settings.coefficientOfRestitution;
    p.cfl = settings.cflCondition;
    const size_t n = particles.size();
    std::vector<double> pos(3 * n), vel(3 * n);
    std::vector<int32_t> type(n);
    for (size_t i = 0; i < n; i++) {
        for (int c = 0; c < 3; c++) {
            pos[3 * i + c] = particles[i].position[c];
            vel[3 * i + c] = particles[i].velocity[c];
        }
        type[i] = (int32_t)particles[i].type;
    }
    mps_engine* e = nullptr;
    check(mps_create(&p, (int32_t)n, pos.data(), vel.data(), type.data(), &e));
    engine.reset(e);
    check(mps_set_solver(e, precision, tol, maxIter));
    syncParticles();
    return t0;
}

void MPS::setSolver(int prec, double t, long long mi) {
    precision = prec;
    tol = t;
    maxIter = mi;
    if (engine) check(mps_set_solver(engine.get(), precision, tol, maxIter));
}

void MPS::syncParticles() {
    const size_t n = particles.size();
    std::vector<double> pos(3 * n), vel(3 * n), p(n), mp(n), ndr(n);
    std::vector<int32_t> type(n), bc(n), dir(n);
    check(mps_download(engine.get(), pos.data(), vel.data(), p.data(), mp.data(), ndr.data(), type.data(),
                       bc.data(), dir.data()));
    for (size_t i = 0; i < n; i++) {
        Particle& q = particles[i];
        for (int c = 0; c < 3; c++) {
            q.position[c] = pos[3 * i + c];
            q.velocity[c] = vel[3 * i + c];
        }
        q.pressure = p[i];
        q.minimumPressure = mp[i];
        q.numberDensityRatio = ndr[i];
        q.type = static_cast<ParticleType>(type[i]);
        q.boundaryCondition = static_cast<BoundaryCondition>(bc[i]);
        q.isDirichletBoundaryConnected = dir[i] != 0;
    }
}

namespace {
// The debug and error lines the reference logs during one step
// (src/mps.cpp:547-571, 590-593, 362-415, 462-464).
void logStep(const mps_step_stats& st, double cfl) {
    if (st.n_new_ghosts > 0)
        mpslog::debug(std::to_string(st.n_new_ghosts) + " particle(s) went out of the domain.");
    if (st.n_unconnected > 0)
        mpslog::debug("There is no Dirichlet boundary condition connected to " + std::to_string(st.n_unconnected) +
                      " particle(s).");
    if (st.courant > cfl)
        mpslog::debug("Courant number is larger than CFL condition. Courant=" + std::to_string(st.courant));
    if (st.courant > 1.0) mpslog::error("Courant number is larger than 1.0. Exiting Simulation.");
    if (st.status == MPS_ERR_NOT_CONVERGED)  // the step goes on with that pressure
        mpslog::debug("Pressure calculation failed: the solve stopped at its iteration cap.");
}

// An asymmetric matrix ends the run as the reference's solvePoissonEquation
// does (src/mps.cpp:425-439): print the pair and exit.
void exitIfAsymmetric(int rc) {
    if (rc == MPS_ERR_ASYMMETRIC) {
        std::cout << mps_last_error() << std::endl;
        std::exit(1);
    }
}
}  // namespace

// src/mps.cpp:111-130 (the whole step on the GPU); the debug events the
// reference logs one by one are logged here as counts.
double MPS::stepForward(const bool isTimeToExport) {
    if (!engine) throw std::runtime_error("MPS::stepForward before loadInitialState");
    const int rc = mps_step(engine.get(), isTimeToExport ? 1 : 0, &stats);
    exitIfAsymmetric(rc);
    if (rc != MPS_ERR_NOT_CONVERGED) check(rc);
    logStep(stats, settings.cflCondition);
    debugLogCount = stats.debug_log_count;
    if (isTimeToExport && syncOnExport) syncParticles();
    return stats.courant;
}

std::vector<mps_step_stats> MPS::stepForwardMany(int n) {
    if (!engine) throw std::runtime_error("MPS::stepForwardMany before loadInitialState");
    std::vector<mps_step_stats> st(n > 0 ? n : 0);
    if (n <= 0) return st;
    const int rc = mps_run_report(engine.get(), n, st.data());
    exitIfAsymmetric(rc);
    if (rc != MPS_ERR_NOT_CONVERGED) check(rc);
    for (const auto& s : st) logStep(s, settings.cflCondition);
    stats = st.back();
    debugLogCount = stats.debug_log_count;
    return st;
}

void MPS::beginExport() {
    if (!engine) throw std::runtime_error("MPS::beginExport before loadInitialState");
    check(mps_export_begin(engine.get()));
}

// Safe on another thread while stepForward runs (see include/mps_gb300.h).
void MPS::writeExport(const std::filesystem::path& csv, const std::filesystem::path& vtu, double time) {
    const int rc = mps_export_write(engine.get(), csv.string().c_str(), vtu.string().c_str(), time);
    if (rc != MPS_OK) throw std::runtime_error(std::string("export failed: ") + mps_last_error());
}
