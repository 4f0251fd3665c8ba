// Particle data model of the reference (src/particle.hpp:5-46), same names
// and members; Eigen::Vector3d is replaced by Vec3.
#pragma once
#include <vector>

#include "vec3.hpp"

enum class ParticleType { Ghost = -1, Fluid = 0, Wall = 1, DummyWall = 2 };

class Neighbor {
public:
    int id;
    double distance;
    Neighbor(int id, double distance) : id(id), distance(distance) {}
};

enum class BoundaryCondition { Ignored, Surface, Inner };

class Particle {
public:
    int id;
    ParticleType type;
    Vec3 position, velocity;
    Vec3 acceleration = Vec3::Zero();
    double pressure = 0.0, minimumPressure = 0.0;
    double density;
    double numberDensityRatio = 0.0;

    std::vector<Neighbor> neighbors;

    BoundaryCondition boundaryCondition = BoundaryCondition::Ignored;
    bool isDirichletBoundaryConnected = false;

    Particle(const int& id, const ParticleType& type, const Vec3& position, const Vec3& velocity,
             const double& density);

    double inverseDensity() const;
};
