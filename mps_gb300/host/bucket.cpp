#include "bucket.hpp"

#include <algorithm>

// src/bucket.cpp:10-22
Bucket::Bucket(const double& reMax, const Domain& domain, const int& particleSize) {
    length = reMax;
    this->domain = domain;
    numX = (int)(domain.x.length / length) + 3;
    numY = (int)(domain.y.length / length) + 3;
    numZ = (int)(domain.z.length / length) + 3;
    num = numX * numY * numZ;
    first.assign(num, -1);
    last.assign(num, -1);
    next.assign(particleSize, -1);
}

namespace {
int cellCoord(double x, double lo, double len, int cells) {
    double q = (x - lo) / len;
    if (!(q >= 0.0)) return 1;
    if (q >= (double)(cells - 2)) return cells - 2;
    return (int)q + 1;
}
}  // namespace

// src/bucket.cpp:24-51: per-cell linked lists in ascending id order.
void Bucket::storeParticles(std::vector<Particle>& particles) {
    std::fill(first.begin(), first.end(), -1);
    std::fill(last.begin(), last.end(), -1);
    next.assign(particles.size(), -1);
    for (auto& p : particles) {
        if (p.type == ParticleType::Ghost) continue;
        int ix = cellCoord(p.position.x(), domain.x.min, length, numX);
        int iy = cellCoord(p.position.y(), domain.y.min, length, numY);
        int iz = cellCoord(p.position.z(), domain.z.min, length, numZ);
        int b = ix + iy * numX + iz * numX * numY;
        if (last[b] == -1)
            first[b] = p.id;
        else
            next[last[b]] = p.id;
        last[b] = p.id;
    }
}
