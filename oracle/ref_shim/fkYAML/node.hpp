// Stand-in for fktn-k/fkYAML as used by src/settings.cpp:12-89.  TEST
// INFRASTRUCTURE ONLY (project-written): block mappings by indentation,
// flow sequences "[a, b]", scalars and "#" comments.
#pragma once
#include <cstdlib>
#include <istream>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

namespace fkyaml {

class exception : public std::runtime_error {
public:
    using std::runtime_error::runtime_error;
};

class node {
public:
    std::string scalar;
    std::map<std::string, std::shared_ptr<node>> map;
    std::vector<std::shared_ptr<node>> seq;

    node& operator[](const std::string& k) {
        auto it = map.find(k);
        if (it == map.end()) throw exception("missing key: " + k);
        return *it->second;
    }
    node& operator[](const char* k) { return (*this)[std::string(k)]; }
    node& operator[](int i) {
        if (i < 0 || (size_t)i >= seq.size()) throw exception("bad index");
        return *seq[i];
    }
    template <typename T>
    T get_value() const {
        if constexpr (std::is_same_v<T, std::string>) return scalar;
        else if constexpr (std::is_same_v<T, bool>) return scalar == "true" || scalar == "True" || scalar == "TRUE";
        else if constexpr (std::is_integral_v<T>) return (T)std::strtol(scalar.c_str(), nullptr, 10);
        else return (T)std::strtod(scalar.c_str(), nullptr);
    }

    static std::string trim(const std::string& s) {
        size_t a = s.find_first_not_of(" \t\r");
        if (a == std::string::npos) return "";
        size_t b = s.find_last_not_of(" \t\r");
        return s.substr(a, b - a + 1);
    }
    static std::shared_ptr<node> parse_value(const std::string& v) {
        auto n = std::make_shared<node>();
        std::string t = trim(v);
        if (!t.empty() && t.front() == '[') {
            std::string body = t.substr(1, t.find(']') - 1);
            size_t p = 0;
            while (p <= body.size()) {
                size_t q = body.find(',', p);
                if (q == std::string::npos) q = body.size();
                auto e = std::make_shared<node>();
                e->scalar = trim(body.substr(p, q - p));
                n->seq.push_back(e);
                p = q + 1;
            }
        } else {
            if (t.size() >= 2 && (t.front() == '"' || t.front() == '\'')) t = t.substr(1, t.size() - 2);
            n->scalar = t;
        }
        return n;
    }
    static node deserialize(std::istream& in) {
        node root;
        std::vector<std::pair<int, node*>> stack{{-1, &root}};
        std::string line;
        while (std::getline(in, line)) {
            size_t h = line.find('#');
            if (h != std::string::npos) line = line.substr(0, h);
            if (trim(line).empty()) continue;
            int indent = (int)line.find_first_not_of(' ');
            std::string body = trim(line);
            size_t c = body.find(':');
            if (c == std::string::npos) continue;
            std::string key = trim(body.substr(0, c));
            std::string val = trim(body.substr(c + 1));
            while (stack.back().first >= indent) stack.pop_back();
            node* parent = stack.back().second;
            if (val.empty()) {
                auto child = std::make_shared<node>();
                parent->map[key] = child;
                stack.push_back({indent, child.get()});
            } else {
                parent->map[key] = parse_value(val);
            }
        }
        return root;
    }
};

}  // namespace fkyaml
