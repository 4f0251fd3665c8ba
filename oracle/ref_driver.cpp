// Harness around the reference's own MPS class — TEST INFRASTRUCTURE ONLY.
//
// It is compiled together with the reference's src/mps.cpp, src/bucket.cpp,
// src/particle.cpp and src/settings.cpp (read in place, never copied) and the
// project-written stand-ins under oracle/ref_shim/, and writes the particle
// state after loadInitialState and after each step as raw binary records that
// tests/golden/make_golden.py turns into golden fixtures.
//
//   ref_driver <settings.yml> <steps> <out_dir> [export_every] [phases]
//
// Relative inputCsvPath values resolve against the working directory, as in
// the reference (src/mps.cpp:39).  With "phases" the step is driven through
// the same private member sequence as MPS::stepForward (src/mps.cpp:111-130)
// so that the neighbour lists used by the collision pass can be recorded too.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <map>
#include <queue>
#include <string>
#include <vector>

#include "Eigen/Dense"
#include "Eigen/IterativeLinearSolvers"
#include "Eigen/Sparse"
#include "csv.hpp"
#include "fkYAML/node.hpp"
#include "spdlog/spdlog.h"

#define private public
#include "mps.hpp"
#undef private

namespace {

template <typename T>
void put(std::ofstream& o, const T& v) {
    o.write(reinterpret_cast<const char*>(&v), sizeof(T));
}
template <typename T>
void put_vec(std::ofstream& o, const std::vector<T>& v) {
    if (!v.empty()) o.write(reinterpret_cast<const char*>(v.data()), sizeof(T) * v.size());
}

void dump(MPS& m, const std::string& path, double time, double courant) {
    const auto& ps = m.particles;
    int64_t n = (int64_t)ps.size();
    std::vector<double> pos, vel, pr, mp, ndr, src;
    std::vector<int32_t> type, bc, dir, nid, col;
    std::vector<int64_t> noff{0}, rp;
    std::vector<double> nd, val;
    for (const auto& p : ps) {
        for (int c = 0; c < 3; c++) pos.push_back(p.position.v[c]);
        for (int c = 0; c < 3; c++) vel.push_back(p.velocity.v[c]);
        pr.push_back(p.pressure);
        mp.push_back(p.minimumPressure);
        ndr.push_back(p.numberDensityRatio);
        type.push_back((int32_t)p.type);
        bc.push_back((int32_t)p.boundaryCondition);
        dir.push_back(p.isDirichletBoundaryConnected ? 1 : 0);
        for (const auto& nb : p.neighbors) {
            nid.push_back(nb.id);
            nd.push_back(nb.distance);
        }
        noff.push_back((int64_t)nid.size());
    }
    src = m.sourceTerm.d;
    src.resize(n, 0.0);
    rp = m.coefficientMatrix.outer;
    rp.resize(n + 1, rp.empty() ? 0 : rp.back());
    col = m.coefficientMatrix.inner;
    val = m.coefficientMatrix.values;
    std::ofstream o(path, std::ios::binary);
    put(o, n);
    put(o, (int64_t)nid.size());
    put(o, (int64_t)col.size());
    put(o, time);
    put(o, courant);
    put(o, (int64_t)m.debugLogCount);
    put_vec(o, pos);
    put_vec(o, vel);
    put_vec(o, pr);
    put_vec(o, mp);
    put_vec(o, ndr);
    put_vec(o, type);
    put_vec(o, bc);
    put_vec(o, dir);
    put_vec(o, noff);
    put_vec(o, nid);
    put_vec(o, nd);
    put_vec(o, src);
    put_vec(o, rp);
    put_vec(o, col);
    put_vec(o, val);
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s settings.yml steps out_dir [export_every] [phases]\n", argv[0]);
        return 2;
    }
    std::filesystem::path yaml = argv[1];
    int steps = std::atoi(argv[2]);
    std::string out = argv[3];
    int export_every = argc > 4 ? std::atoi(argv[4]) : 0;
    bool phases = argc > 5 && std::string(argv[5]) == "phases";
    std::filesystem::create_directories(out);

    MPS m(yaml);
    // MPS::loadInitialState (src/mps.cpp:96-109) with one addition: Particle
    // leaves pressure, boundaryCondition and isDirichletBoundaryConnected
    // uninitialised (src/particle.hpp:30-41), and the first setNumberDensity
    // reads boundaryCondition.  They are set to 0 / Ignored / false here, the
    // values the oracle and the GPU engine define for them.
    double t = m.importInitialCondition();
    for (auto& p : m.particles) {
        p.pressure = 0.0;
        p.boundaryCondition = BoundaryCondition::Ignored;
        p.isDirichletBoundaryConnected = false;
    }
    m.sourceTerm.resize(m.particles.size());
    m.coefficientMatrix.resize(m.particles.size(), m.particles.size());
    m.bucket = Bucket(m.settings.effectiveRadius.max, m.settings.domain, m.particles.size());
    m.setNumberDensity();
    char name[512];
    std::snprintf(name, sizeof name, "%s/step_%04d.bin", out.c_str(), 0);
    dump(m, name, t, 0.0);
    for (int s = 1; s <= steps; s++) {
        t += m.settings.dt;
        bool ex = export_every > 0 && (s % export_every) == 0;
        double c;
        if (!phases) {
            c = m.stepForward(ex);
        } else {
            m.setNeighbors();
            m.calcGravity();
            m.calcViscosity();
            m.moveParticles();
            m.setNeighbors();
            std::snprintf(name, sizeof name, "%s/collide_%04d.bin", out.c_str(), s);
            dump(m, name, t, 0.0);
            m.collision();
            m.setNeighbors();
            m.calcPressure();
            m.calcPressureGradient();
            m.moveParticlesWithPressureGradient();
            if (ex || m.settings.higherOrderSourceTerm.on) m.setNumberDensity();
            c = m.getCourantNumber();
        }
        std::snprintf(name, sizeof name, "%s/step_%04d.bin", out.c_str(), s);
        dump(m, name, t, c);
    }
    return 0;
}
