// Command line of the reference (src/main.cpp:11-42): mps -s <settings.yml>.
// Additions: -p fp64|mixed selects the pressure solver; --check-settings
// prints the parsed settings and exits (no GPU needed).
#include <cstdlib>
#include <filesystem>
#include <iomanip>
#include <iostream>
#include <string>

#include "simulation.hpp"

namespace fs = std::filesystem;

static int check_settings(const fs::path& p) {
    Settings s;
    s.load(p);
    std::cout << std::setprecision(17);
    std::cout << "{\"dim\": " << s.dim << ", \"particle_distance\": " << s.particleDistance
              << ", \"dt\": " << s.dt << ", \"re_pressure\": " << s.effectiveRadius.pressure
              << ", \"re_viscosity\": " << s.effectiveRadius.viscosity
              << ", \"re_surface\": " << s.effectiveRadius.surfaceDetection << ", \"re_max\": " << s.effectiveRadius.max
              << ", \"domain_min\": [" << s.domain.x.min << ", " << s.domain.y.min << ", " << s.domain.z.min
              << "], \"domain_max\": [" << s.domain.x.max << ", " << s.domain.y.max << ", " << s.domain.z.max
              << "], \"gravity\": [" << s.gravity.x() << ", " << s.gravity.y() << ", " << s.gravity.z()
              << "], \"density\": " << s.density << ", \"kinematic_viscosity\": " << s.kinematicViscosity
              << ", \"surface_threshold\": " << s.thresholdForSurfaceDetection
              << ", \"quasi_compressibility_on\": " << s.quasiCompressibility.on
              << ", \"compressibility\": " << s.quasiCompressibility.compressibility
              << ", \"higher_order_on\": " << s.higherOrderSourceTerm.on
              << ", \"higher_order_gamma\": " << s.higherOrderSourceTerm.gamma
              << ", \"relaxation\": " << s.relaxationCoefficientForPressure
              << ", \"collision_distance\": " << s.collisionDistance
              << ", \"restitution\": " << s.coefficientOfRestitution << ", \"cfl\": " << s.cflCondition
              << ", \"finish_time\": " << s.finishTime << ", \"output_interval\": " << s.outputInterval
              << ", \"input_csv\": \"" << s.inputCsvPath.string() << "\"}" << std::endl;
    return 0;
}

int main(int argc, char** argv) {
    std::string setting, precision = "fp64";
    bool check = false;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        if ((a == "-s" || a == "--setting") && i + 1 < argc)
            setting = argv[++i];
        else if ((a == "-p" || a == "--precision") && i + 1 < argc)
            precision = argv[++i];
        else if (a == "--check-settings")
            check = true;
        else {
            std::cout << "usage: mps -s <settings.yml> [-p fp64|mixed] [--check-settings]" << std::endl;
            return EXIT_FAILURE;
        }
    }
    if (setting.empty()) {
        std::cout << "-s: required." << std::endl;
        return EXIT_FAILURE;
    }
    if (!fs::exists(setting)) {
        std::cout << "ERROR: Input YAML file cannot be found in specified path: " + setting << std::endl;
        return EXIT_FAILURE;
    }
    try {
        if (check) return check_settings(setting);
        std::cout << "Setting file: " << setting << std::endl;
        Simulation simulation;
        simulation.run(fs::path(setting), precision == "mixed" ? MPS_PRECISION_MIXED : MPS_PRECISION_FP64);
    } catch (const std::exception& e) {
        std::cout << "ERROR: " << e.what() << std::endl;
        return EXIT_FAILURE;
    }
    return 0;
}
