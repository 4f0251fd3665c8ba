// Minimal reader for the YAML subset of the reference's settings files:
// block mappings by indentation, flow sequences "[a, b, c]", scalars and
// "#" comments.
#pragma once
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

class YamlNode {
public:
    std::string scalar;
    std::map<std::string, std::shared_ptr<YamlNode>> map;
    std::vector<std::string> seq;
    bool is_map = false, is_seq = false;

    const YamlNode& operator[](const std::string& key) const;
    std::string at(size_t i) const;
    double asDouble() const;
    int asInt() const;
    bool asBool() const;

    static YamlNode parse(const std::string& text);
};

double yaml_to_double(const std::string& s, const std::string& what);
