// The reference's MPS class (src/mps.hpp:22-71) with the same public surface:
// MPS(yaml), loadInitialState(), stepForward(isTimeToExport), and the public
// members settings, particles and debugLogCount.  The step itself runs on
// the GPU through the engine's C ABI (include/mps_gb300.h); `particles`
// mirrors the device state after loadInitialState and after every export
// step (call syncParticles() to refresh it at any other time).
#pragma once
#include <filesystem>
#include <memory>
#include <vector>

#include "bucket.hpp"
#include "mps_gb300.h"
#include "particle.hpp"
#include "settings.hpp"

class RefValues {
public:
    double initialNumberDensity = 0;
    double lambda = 0;
    RefValues() = default;
    RefValues(const int& dim, const double& particleDistance, const double& effectiveRadius);
};

class MPS {
public:
    Settings settings;
    std::vector<Particle> particles;
    int debugLogCount = 0;

    MPS() = default;
    explicit MPS(const std::filesystem::path& inputYamlPath);
    MPS(MPS&&) noexcept = default;
    MPS& operator=(MPS&&) noexcept = default;

    double loadInitialState();  // Initialize particles and return initial time
    double stepForward(const bool isTimeToExport);
    // n non-export steps with one host wait per up to 256 of them; each
    // step's stats (Courant number, debug counts) in order, with the same
    // debug logging stepForward does per step.
    std::vector<mps_step_stats> stepForwardMany(int n);

    // Additions of this implementation.
    void setSolver(int precision, double tol = 0.0, long long maxIter = 0);
    void syncParticles();
    const mps_step_stats& lastStepStats() const { return stats; }
    // Export steps refresh `particles` (the reference's behaviour) unless a
    // driver that exports from engine snapshots turns this off.
    bool syncOnExport = true;
    // Snapshot of the current state for export (mps_export_begin); the
    // following steps may run while writeExport() waits for it and writes.
    void beginExport();
    void writeExport(const std::filesystem::path& csv, const std::filesystem::path& vtu, double time);

private:
    struct EngineDeleter {
        void operator()(mps_engine* e) const { mps_destroy(e); }
    };
    std::unique_ptr<mps_engine, EngineDeleter> engine;
    mps_step_stats stats{};
    int precision = MPS_PRECISION_FP64;
    double tol = 0.0;
    long long maxIter = 0;
    struct {
        RefValues pressure, viscosity, surfaceDetection;
    } refValues;

    double importInitialCondition();
};
