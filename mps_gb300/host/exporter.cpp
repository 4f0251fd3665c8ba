#include "exporter.hpp"

#include <cstdio>
#include <stdexcept>

namespace {
// Fixed notation with six decimals, as the reference's CSV writer emits
// (inputs/*/input.csv).
std::string f6(double v) {
    char b[64];
    std::snprintf(b, sizeof b, "%.6f", v);
    return b;
}
}  // namespace

// src/exporter.cpp:10-55
void Exporter::toCsv(const std::filesystem::path& outFilePath, const std::vector<Particle>& particles,
                     const double& time) {
    std::ofstream out(outFilePath);
    if (!out.is_open()) throw std::runtime_error("Could not open target csv file: " + outFilePath.string());
    out << "Time (s)," << f6(time) << '\n';
    out << "Number of Particles," << particles.size() << '\n';
    out << "ID,Type,Position.x (m),Position.y (m),Position.z (m),Velocity.x (m/s),Velocity.y (m/s),"
           "Velocity.z (m/s),Pressure (Pa),Number Density Ratio\n";
    std::string line;
    for (const auto& p : particles) {
        if (p.type == ParticleType::Ghost) continue;
        line = std::to_string(p.id) + "," + std::to_string((int)p.type) + "," + f6(p.position.x()) + "," +
               f6(p.position.y()) + "," + f6(p.position.z()) + "," + f6(p.velocity.x()) + "," +
               f6(p.velocity.y()) + "," + f6(p.velocity.z()) + "," + f6(p.pressure) + "," +
               f6(p.numberDensityRatio) + "\n";
        out << line;
    }
}

// src/exporter.cpp:57-167
void Exporter::toVtu(const std::filesystem::path& outFilePath, const std::vector<Particle>& particles,
                     const double& time) {
    std::ofstream out(outFilePath);
    if (!out.is_open()) throw std::runtime_error("Could not open target vtu file: " + outFilePath.string());
    const char* nl = "\n";
    out << "<?xml version='1.0' encoding='UTF-8'?>" << nl;
    out << "<VTKFile byte_order='LittleEndian' version='0.1' type = 'UnstructuredGrid'>" << nl;
    out << "<UnstructuredGrid>" << nl;
    out << "<FieldData>" << nl;
    out << "<DataArray type='Float64' Name='Time' NumberOfComponents='1' NumberOfTuples='1' format='ascii'>"
        << nl;
    out << time << nl;
    out << "</DataArray>" << nl;
    out << "</FieldData>" << nl;
    out << "<Piece NumberOfCells='" << particles.size() << "' NumberOfPoints='" << particles.size() << "'>"
        << nl;
    out << "<Points>" << nl;
    out << "<DataArray NumberOfComponents='3' type='Float64' Name='position' format='ascii'>" << nl;
    for (const auto& p : particles) out << p.position.x() << " " << p.position.y() << " " << p.position.z() << nl;
    out << "</DataArray>" << nl;
    out << "</Points>" << nl;
    out << "<PointData>" << nl;
    dataArrayBegin(out, "1", "Int32", "Type");
    for (const auto& p : particles) out << (int)p.type << nl;
    dataArrayEnd(out);
    dataArrayBegin(out, "3", "Float64", "Velocity");
    for (const auto& p : particles) out << p.velocity.x() << " " << p.velocity.y() << " " << 0.0 << nl;
    dataArrayEnd(out);
    dataArrayBegin(out, "1", "Float64", "Pressure");
    for (const auto& p : particles) out << p.pressure << nl;
    dataArrayEnd(out);
    dataArrayBegin(out, "1", "Float64", "Number Density Ratio");
    for (const auto& p : particles) out << p.numberDensityRatio << nl;
    dataArrayEnd(out);
    dataArrayBegin(out, "1", "Int32", "Boundary Condition");
    for (const auto& p : particles) out << (int)p.boundaryCondition << nl;
    dataArrayEnd(out);
    out << "</PointData>" << nl;
    out << "<Cells>" << nl;
    out << "<DataArray type='Int32' Name='connectivity' format='ascii'>" << nl;
    for (size_t i = 0; i < particles.size(); i++) out << i << nl;
    out << "</DataArray>" << nl;
    out << "<DataArray type='Int32' Name='offsets' format='ascii'>" << nl;
    for (size_t i = 0; i < particles.size(); i++) out << i + 1 << nl;
    out << "</DataArray>" << nl;
    out << "<DataArray type='UInt8' Name='types' format='ascii'>" << nl;
    for (size_t i = 0; i < particles.size(); i++) out << "1" << nl;
    out << "</DataArray>" << nl;
    out << "</Cells>" << nl;
    out << "</Piece>" << nl;
    out << "</UnstructuredGrid>" << nl;
    out << "</VTKFile>" << nl;
}

void Exporter::dataArrayBegin(std::ofstream& out, const std::string& numberOfComponents,
                              const std::string& type, const std::string& name) {
    out << "<DataArray NumberOfComponents='" << numberOfComponents << "' type='" << type << "' Name='"
        << name << "' format='ascii'>\n";
}

void Exporter::dataArrayEnd(std::ofstream& out) { out << "</DataArray>\n"; }
