#include "yaml_lite.hpp"

#include <cstdlib>
#include <sstream>

namespace {
std::string trim(const std::string& s) {
    size_t a = s.find_first_not_of(" \t\r");
    if (a == std::string::npos) return "";
    size_t b = s.find_last_not_of(" \t\r");
    return s.substr(a, b - a + 1);
}
std::string unquote(std::string t) {
    if (t.size() >= 2 && (t.front() == '"' || t.front() == '\'') && t.back() == t.front())
        t = t.substr(1, t.size() - 2);
    return t;
}
}  // namespace

double yaml_to_double(const std::string& s, const std::string& what) {
    char* end = nullptr;
    double v = std::strtod(s.c_str(), &end);
    if (end == s.c_str() || *end != '\0') throw std::runtime_error("not a number: " + what + " = " + s);
    return v;
}

const YamlNode& YamlNode::operator[](const std::string& key) const {
    auto it = map.find(key);
    if (it == map.end()) throw std::runtime_error("missing key in settings: " + key);
    return *it->second;
}

std::string YamlNode::at(size_t i) const {
    if (i >= seq.size()) throw std::runtime_error("sequence index out of range");
    return seq[i];
}

double YamlNode::asDouble() const { return yaml_to_double(scalar, scalar); }
int YamlNode::asInt() const { return (int)std::strtol(scalar.c_str(), nullptr, 10); }
bool YamlNode::asBool() const {
    if (scalar == "True" || scalar == "true" || scalar == "TRUE") return true;
    if (scalar == "False" || scalar == "false" || scalar == "FALSE") return false;
    throw std::runtime_error("not a boolean: " + scalar);
}

YamlNode YamlNode::parse(const std::string& text) {
    YamlNode root;
    root.is_map = true;
    std::vector<std::pair<int, YamlNode*>> stack{{-1, &root}};
    std::istringstream in(text);
    std::string line;
    while (std::getline(in, line)) {
        size_t h = line.find('#');
        if (h != std::string::npos) line = line.substr(0, h);
        if (trim(line).empty()) continue;
        int indent = (int)line.find_first_not_of(' ');
        std::string body = trim(line);
        size_t c = body.find(':');
        if (c == std::string::npos) throw std::runtime_error("unsupported settings line: " + body);
        std::string key = trim(body.substr(0, c));
        std::string val = trim(body.substr(c + 1));
        while (stack.back().first >= indent) stack.pop_back();
        YamlNode* parent = stack.back().second;
        auto child = std::make_shared<YamlNode>();
        parent->map[key] = child;
        if (val.empty()) {
            child->is_map = true;
            stack.push_back({indent, child.get()});
        } else if (val.front() == '[') {
            child->is_seq = true;
            size_t close = val.find(']');
            std::string inner = val.substr(1, close == std::string::npos ? std::string::npos : close - 1);
            std::stringstream ss(inner);
            std::string item;
            while (std::getline(ss, item, ',')) child->seq.push_back(unquote(trim(item)));
        } else {
            child->scalar = unquote(val);
        }
    }
    return root;
}
