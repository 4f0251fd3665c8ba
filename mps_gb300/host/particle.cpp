#include "particle.hpp"

Particle::Particle(const int& id, const ParticleType& type, const Vec3& position,
                   const Vec3& velocity, const double& density)
    : id(id), type(type), position(position), velocity(velocity), density(density) {}

// src/particle.cpp:19-29
double Particle::inverseDensity() const {
    return type == ParticleType::Fluid ? 1.0 / density : 0.0;
}
