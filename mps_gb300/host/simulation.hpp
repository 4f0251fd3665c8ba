// Simulation driver of the reference (src/simulation.hpp:11-39).
#pragma once
#include <chrono>
#include <filesystem>
#include <exception>
#include <fstream>
#include <thread>
#include <vector>

#include "mps.hpp"
#include "particle.hpp"

class Simulation {
public:
    void run(const std::filesystem::path& inputYamlPath, int precision = MPS_PRECISION_FP64);

private:
    MPS mps;

    int timeStep = 0;
    double time = 0.0;
    std::chrono::system_clock::time_point simulationStartTime, simulationEndTime;

    int outFileNum = 0;
    // Files of an export are written on this thread from an engine snapshot
    // while the next steps run; one export in flight at a time.
    std::thread exportWriter;
    std::exception_ptr exportError;
    std::ofstream timeStepReportFile;
    std::filesystem::path resultDirectory;

    void createResultDirectory(const std::filesystem::path& inputYamlPath);
    void prepareLogFile();
    void timeStepReport(const std::chrono::system_clock::time_point& timeStepStartTime,
                        const std::chrono::system_clock::time_point& timeStepEndTime,
                        const double& courantNumber, const bool& isDebugLogAdded);
    bool isTimeToExport();
    bool isTimeToExportAt(double t) const;
    void exportParticles(const std::vector<Particle>& particles);
    void exportSnapshot();
    void finishExport();
    void endSimulation();
};
