// Stand-in for vincentlaucsb/csv-parser as used by src/mps.cpp:38-94.  TEST
// INFRASTRUCTURE ONLY (project-written): comma-separated rows, optional
// header row, fields converted with strtod/strtol.
#pragma once
#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>

namespace csv {

class CSVField {
public:
    std::string s;
    template <typename T>
    T get() const {
        if constexpr (std::is_same_v<T, std::string>) return s;
        else if constexpr (std::is_integral_v<T>) return (T)std::strtol(s.c_str(), nullptr, 10);
        else return (T)std::strtod(s.c_str(), nullptr);
    }
};

class CSVFormat {
public:
    int header = 0;
    CSVFormat& no_header() { header = -1; return *this; }
    CSVFormat& header_row(int r) { header = r; return *this; }
};

class CSVRow {
public:
    std::vector<std::string> f;
    const std::map<std::string, size_t>* names = nullptr;
    CSVField operator[](size_t i) const { return CSVField{i < f.size() ? f[i] : std::string()}; }
    CSVField operator[](const std::string& n) const { return (*this)[names->at(n)]; }
};

class CSVReader {
public:
    std::vector<CSVRow> rows;
    std::map<std::string, size_t> names;
    CSVReader(const std::string& path, CSVFormat fmt) {
        std::ifstream in(path);
        std::string line;
        int idx = 0;
        while (std::getline(in, line)) {
            if (!line.empty() && line.back() == '\r') line.pop_back();
            std::vector<std::string> f;
            std::stringstream ss(line);
            std::string cell;
            while (std::getline(ss, cell, ',')) f.push_back(cell);
            if (fmt.header >= 0 && idx < fmt.header) { idx++; continue; }
            if (fmt.header >= 0 && idx == fmt.header) {
                for (size_t k = 0; k < f.size(); k++) names[f[k]] = k;
                idx++;
                continue;
            }
            if (line.empty()) { idx++; continue; }
            rows.push_back(CSVRow{f, &names});
            idx++;
        }
        for (auto& r : rows) r.names = &names;
    }
    std::vector<CSVRow>::iterator begin() { return rows.begin(); }
    std::vector<CSVRow>::iterator end() { return rows.end(); }
};

}  // namespace csv
