#include "settings.hpp"

#include <algorithm>
#include <fstream>
#include <sstream>
#include <stdexcept>

#include "yaml_lite.hpp"

Domain::Domain(const double& xMin, const double& xMax, const double& yMin, const double& yMax,
               const double& zMin, const double& zMax) {
    x.min = xMin;
    x.max = xMax;
    x.length = xMax - xMin;
    y.min = yMin;
    y.max = yMax;
    y.length = yMax - yMin;
    z.min = zMin;
    z.max = zMax;
    z.length = zMax - zMin;
}

// Settings::load, src/settings.cpp:12-89 (same keys; radii are ratio * l0).
void Settings::load(const std::filesystem::path& inputYamlPath) {
    std::ifstream ifs(inputYamlPath);
    if (!ifs.is_open()) throw std::runtime_error("Could not open setting file: " + inputYamlPath.string());
    std::stringstream buf;
    buf << ifs.rdbuf();
    YamlNode root = YamlNode::parse(buf.str());

    dim = root["dim"].asInt();
    particleDistance = root["particle distance"].asDouble();
    dt = root["dt"].asDouble();
    finishTime = root["finish time"].asDouble();
    outputInterval = root["output interval"].asDouble();
    cflCondition = root["CFL condition"].asDouble();

    auto rangeOf = [&](const char* key, int i) { return yaml_to_double(root[key].at(i), key); };
    domain = Domain(rangeOf("domain range X", 0), rangeOf("domain range X", 1),
                    rangeOf("domain range Y", 0), rangeOf("domain range Y", 1),
                    rangeOf("domain range Z", 0), rangeOf("domain range Z", 1));

    density = root["density"].asDouble();
    kinematicViscosity = root["kinematic viscosity"].asDouble();
    for (int i = 0; i < 3; i++) gravity[i] = yaml_to_double(root["gravity"].at(i), "gravity");

    const YamlNode& er = root["effective radius ratio"];
    effectiveRadius.pressure = er["pressure"].asDouble() * particleDistance;
    effectiveRadius.viscosity = er["viscosity"].asDouble() * particleDistance;
    effectiveRadius.surfaceDetection = er["surface detection"].asDouble() * particleDistance;
    effectiveRadius.max =
        std::max({effectiveRadius.pressure, effectiveRadius.viscosity, effectiveRadius.surfaceDetection});

    thresholdForSurfaceDetection = root["threshold for surface detection"].asDouble();

    const YamlNode& ps = root["pressure stabilization"];
    quasiCompressibility.on = ps["quasi compressibility"]["on"].asBool();
    quasiCompressibility.compressibility =
        quasiCompressibility.on ? ps["quasi compressibility"]["compressibility"].asDouble() : 0.0;
    higherOrderSourceTerm.on = ps["higher order source term"]["on"].asBool();
    higherOrderSourceTerm.gamma =
        higherOrderSourceTerm.on ? ps["higher order source term"]["gamma"].asDouble() : 0.0;
    relaxationCoefficientForPressure = root["relaxation coefficient for pressure"].asDouble();

    collisionDistance = root["collision distance ratio"].asDouble() * particleDistance;
    coefficientOfRestitution = root["coefficient of restitution"].asDouble();

    inputCsvPath = root["inputCsvPath"].scalar;
}
