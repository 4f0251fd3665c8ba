#include "simulation.hpp"

#include <cmath>
#include <format>
#include <iostream>

#include "exporter.hpp"
#include "logger.hpp"

namespace fs = std::filesystem;
using std::chrono::duration_cast;
using std::chrono::milliseconds;
using std::chrono::seconds;
using std::chrono::system_clock;

// src/simulation.cpp:29-64
void Simulation::run(const fs::path& inputYamlPath, int precision) {
    createResultDirectory(inputYamlPath);
    prepareLogFile();

    mps = MPS(inputYamlPath);
    mps.setSolver(precision);
    time = mps.loadInitialState();
    mps.syncOnExport = false;  // exports are written from engine snapshots
    exportSnapshot();

    mpslog::info("START SIMULATION");
    simulationStartTime = system_clock::now();
    const double dt = mps.settings.dt, finish = mps.settings.finishTime;
    while (time + dt <= finish) {
        // The steps up to the next export step (or the end): the ones before
        // it run back to back on the device with one host wait per group,
        // and their report rows are written afterwards, each with its own
        // device step time; the export step runs as the reference's loop.
        int ahead = 0;
        bool exportStep = false;
        for (double t = time; t + dt <= finish;) {
            t += dt;  // the same additions as the loop below
            ahead++;
            if (isTimeToExportAt(t)) {
                exportStep = true;
                break;
            }
        }
        const int plain = exportStep ? ahead - 1 : ahead;
        if (plain > 0) {
            int before = mps.debugLogCount;
            auto start = system_clock::now();
            for (const mps_step_stats& s : mps.stepForwardMany(plain)) {
                time += dt;
                const auto end = start + std::chrono::duration_cast<system_clock::duration>(
                                             std::chrono::duration<double, std::milli>(s.ms_step));
                timeStepReport(start, end, s.courant, s.debug_log_count > before);
                before = s.debug_log_count;
                start = end;
                timeStep++;
            }
        }
        if (exportStep) {
            auto t0 = system_clock::now();
            int before = mps.debugLogCount;
            time += dt;
            double courant = mps.stepForward(true);
            exportSnapshot();
            timeStepReport(t0, system_clock::now(), courant, mps.debugLogCount > before);
            timeStep++;
        }
    }
    finishExport();
    simulationEndTime = system_clock::now();
    endSimulation();
}

// src/simulation.cpp:66-77
void Simulation::createResultDirectory(const fs::path& inputYamlPath) {
    resultDirectory = inputYamlPath.parent_path() / "result";
    if (fs::exists(resultDirectory)) fs::remove_all(resultDirectory);
    fs::create_directories(resultDirectory);
    fs::create_directory(resultDirectory / "csv");
    fs::create_directory(resultDirectory / "vtu");
    fs::copy(inputYamlPath, resultDirectory / inputYamlPath.filename());
}

// src/simulation.cpp:79-133
void Simulation::prepareLogFile() {
    mpslog::open_file((resultDirectory / "execution.log").string());
    fs::path path = resultDirectory / "time_step_report.csv";
    timeStepReportFile.open(path);
    if (!timeStepReportFile.is_open()) mpslog::error("Could not open the log file: " + path.string());
    timeStepReportFile << "Time Step,Dt (s),Time Before (s),Time After (s),Finish Time (s),"
                          "Elapsed Time (h:m:s),Elapsed Time (s),Remaining Time (h:m:s),"
                          "Average Time per Time Step (s),Time for This Time Step (s),"
                          "Number of Output Files,Courant Number\n";
}

// src/simulation.cpp:135-151
void Simulation::endSimulation() {
    auto total = duration_cast<seconds>(simulationEndTime - simulationStartTime);
    mpslog::info("END SIMULATION");
    if (mps.debugLogCount > 0)
        mpslog::info(std::format("There were {} debug-level logs. Check 'execution.log'.", mps.debugLogCount));
    else
        mpslog::info("There were no debug-level logs.");
    mpslog::info(std::format("Total Simulation Time = {:%T}", total));
    timeStepReportFile.close();
    mpslog::close_file();
}

// src/simulation.cpp:153-222
void Simulation::timeStepReport(const system_clock::time_point& start, const system_clock::time_point& end,
                                const double& courant, const bool& isDebugLogAdded) {
    auto elapsed = duration_cast<seconds>(end - simulationStartTime);
    double average = 0;
    if (timeStep != 0)
        average = duration_cast<milliseconds>(end - simulationStartTime).count() / (double)(1000 * timeStep);
    seconds remain{int(((mps.settings.finishTime - time) / time) * average * timeStep)};
    auto last = duration_cast<milliseconds>(end - start);
    auto before = std::format("{:.3f}", time - mps.settings.dt);
    auto after = std::format("{:.3f}", time);
    auto el = std::format("{:%T}", elapsed);
    auto av = std::format("{:.3f}", average);
    auto rm = std::format("{:%T}", remain);
    auto ls = std::format("{:%S}", last);
    auto cn = std::format("{:.2f}", courant);
    std::cout << std::format("{}: dt={}s  t={}s->{}s  fin={}s  elapsed={}  remain={}  ave={}s/step  "
                             "last={}s/step  out={}files  Courant={}",
                             timeStep, mps.settings.dt, before, after, mps.settings.finishTime, el, rm, av, ls,
                             outFileNum, cn)
              << std::endl;
    timeStepReportFile << std::format("{},{},{},{},{},{},{},{},{},{},{},{}\n", timeStep, mps.settings.dt, before,
                                      after, mps.settings.finishTime, el, elapsed.count(), rm, av, ls, outFileNum,
                                      cn);
    if (isDebugLogAdded) mpslog::debug(std::format("Time Step:{} Time:{}s->{}s", timeStep, before, after));
}

// src/simulation.cpp:224-229
bool Simulation::isTimeToExport() { return isTimeToExportAt(time); }

bool Simulation::isTimeToExportAt(double t) const {
    double interval = mps.settings.outputInterval;
    double rem = std::fmod(t, interval);
    rem = std::min(rem, interval - rem);
    return rem < mps.settings.dt / 10.0;
}

// src/simulation.cpp:231-245, asynchronously: the state is snapshotted on
// the device and copied to pinned memory while the next steps run, and a
// writer thread formats and writes the same two files.
void Simulation::exportSnapshot() {
    finishExport();
    mps.beginExport();
    const auto csv = resultDirectory / std::format("csv/output_{:04}.csv", outFileNum);
    const auto vtu = resultDirectory / std::format("vtu/output_{:04}.vtu", outFileNum);
    const double t = time;
    exportWriter = std::thread([this, csv, vtu, t] {
        try {
            mps.writeExport(csv, vtu, t);
        } catch (...) {
            exportError = std::current_exception();
        }
    });
    outFileNum++;
}

void Simulation::finishExport() {
    if (exportWriter.joinable()) exportWriter.join();
    if (exportError) {
        auto e = exportError;
        exportError = nullptr;
        std::rethrow_exception(e);
    }
}

// The reference's synchronous form, from the host particle vector.
void Simulation::exportParticles(const std::vector<Particle>& particles) {
    Exporter exporter;
    exporter.toCsv(resultDirectory / std::format("csv/output_{:04}.csv", outFileNum), particles, time);
    exporter.toVtu(resultDirectory / std::format("vtu/output_{:04}.vtu", outFileNum), particles, time);
    outFileNum++;
}
