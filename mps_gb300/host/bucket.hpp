// Bucket of the reference (src/bucket.hpp:8-19): the uniform cell grid of the
// neighbour search, cell edge re_max with one padding cell on every side.
// An interface mirror only: neither the engine nor this front end calls it
// (the GPU builds its own cell table every neighbour search, sort.cu).  It is
// kept so that host code written against the reference's Bucket still
// compiles; its storeParticles has no test of its own.
#pragma once
#include <vector>

#include "particle.hpp"
#include "settings.hpp"

class Bucket {
public:
    int num = 0, numX = 0, numY = 0, numZ = 0;
    double length = 0.0;
    Domain domain;
    std::vector<int> next, first, last;

    Bucket() = default;
    Bucket(const double& reMax, const Domain& domain, const int& particleSize);
    void storeParticles(std::vector<Particle>& particles);
};
