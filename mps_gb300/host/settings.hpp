// Settings and Domain of the reference (src/settings.hpp:7-86), same members,
// read from the reference's settings.yml files unchanged.
#pragma once
#include <filesystem>

#include "vec3.hpp"

class Domain {
public:
    struct {
        double min, max, length;
    } x, y, z;

    Domain() = default;
    Domain(const double& xMin, const double& xMax, const double& yMin, const double& yMax,
           const double& zMin, const double& zMax);
};

class Settings {
public:
    double dim;
    double particleDistance;
    double dt;
    double finishTime;
    double outputInterval;
    double cflCondition;

    Domain domain;

    double density;
    double kinematicViscosity;

    Vec3 gravity;

    struct {
        double pressure;
        double viscosity;
        double surfaceDetection;
        double max;
    } effectiveRadius;

    double thresholdForSurfaceDetection;

    struct {
        bool on;
        double compressibility;
    } quasiCompressibility;
    struct {
        bool on;
        double gamma;
    } higherOrderSourceTerm;
    double relaxationCoefficientForPressure;

    double collisionDistance;
    double coefficientOfRestitution;

    std::filesystem::path inputCsvPath;

    // Throws std::runtime_error on a missing file or key (the reference logs
    // the fkYAML exception, src/settings.cpp:84-88).
    void load(const std::filesystem::path& inputYamlPath);
};
