// Exporter of the reference (src/exporter.hpp:8-29): CSV (Ghost particles
// skipped, six-decimal fixed notation) and ASCII VTU (all particles).
#pragma once
#include <filesystem>
#include <fstream>
#include <string>
#include <vector>

#include "particle.hpp"

class Exporter {
public:
    void toCsv(const std::filesystem::path& outputFilePath, const std::vector<Particle>& particles,
               const double& time);
    void toVtu(const std::filesystem::path& outputFilePath, const std::vector<Particle>& particles,
               const double& time);

private:
    void dataArrayBegin(std::ofstream& outFile, const std::string& numberOfComponents,
                        const std::string& type, const std::string& name);
    void dataArrayEnd(std::ofstream& outFile);
};
